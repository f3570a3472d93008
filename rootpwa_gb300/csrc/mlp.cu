// mlp.cu -- the warm-start network: a 3-layer perceptron
//   h1 = relu(W1 x + b1), h2 = relu(W2 h1 + b2), y = W3 h2 + b3
// with BF16 weights and activations, FP32 accumulation, FP32 master weights,
// its backward pass and an Adam update, all as hand-written kernels.
//
// One tiled GEMM kernel serves every product: C[M][N] = sum_k A(m, k) B(k, n)
// with A and B read through strides (so that X W^T, dY W and dY^T X are the
// same kernel), BF16 operands widened to FP32 in shared memory, 64 x 64 output
// tiles, 16 x 16 threads with 4 x 4 FP32 accumulators each, and an epilogue
// that adds a bias, applies relu or a relu mask and writes FP32 and/or BF16.
// A product of few output tiles (the batch has 256 rows, the layers 102 to
// 512 columns) and a long K is split into K slices, one block per (tile,
// slice), so that the grid covers the GPU; a second kernel sums the slices'
// FP32 partials in slice order (deterministic) and applies the epilogue.

#include "pwa_internal.h"

#include <cuda_bf16.h>

#include <algorithm>

namespace pwa {
namespace {

constexpr int kT = 64;   // output tile
constexpr int kKt = 16;  // k per shared-memory stage

// bias, relu, relu mask and the FP32 / BF16 stores of one output element
__device__ __forceinline__ void mlpEpilogue(const MlpGemm& g, int m, int n, float v)
{
	const size_t o = (size_t)m * g.N + n;
	if (g.bias)
		v += g.bias[n];
	if (g.relu)
		v = fmaxf(v, 0.f);
	const __nv_bfloat16* mask = reinterpret_cast<const __nv_bfloat16*>(g.mask);
	if (mask && !(__bfloat162float(mask[o]) > 0.f))
		v = 0.f;
	if (g.C32)
		g.C32[o] = v;
	if (g.C16)
		reinterpret_cast<__nv_bfloat16*>(g.C16)[o] = __float2bfloat16_rn(v);
}

__global__ void __launch_bounds__(256) mlpGemmKernel(const MlpGemm g)
{
	__shared__ float sa[kKt][kT + 4];
	__shared__ float sb[kKt][kT + 4];
	const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
	const int m0 = blockIdx.y * kT, n0 = blockIdx.x * kT;
	float acc[4][4];
#pragma unroll
	for (int i = 0; i < 4; ++i)
#pragma unroll
		for (int j = 0; j < 4; ++j)
			acc[i][j] = 0.f;
	const __nv_bfloat16* A = reinterpret_cast<const __nv_bfloat16*>(g.A);
	const __nv_bfloat16* B = reinterpret_cast<const __nv_bfloat16*>(g.B);
	// this block's K slice
	const int split = g.splitK > 1 ? g.splitK : 1;
	const int kc = ((g.K + split - 1) / split + kKt - 1) / kKt * kKt;
	const int kBeg = (int)blockIdx.z * kc, kEnd = min(g.K, kBeg + kc);
	for (int k0 = kBeg; k0 < kEnd; k0 += kKt) {
		// 64 x 16 of A and 16 x 64 of B; the element order follows the
		// operand's contiguous dimension so that neighbouring threads read
		// neighbouring addresses
		for (int e = threadIdx.x; e < kT * kKt; e += 256) {
			int r, k;
			if (g.aContigK) {
				r = e / kKt;
				k = e - r * kKt;
			} else {
				k = e / kT;
				r = e - k * kT;
			}
			const int gm = m0 + r, gk = k0 + k;
			sa[k][r] = (gm < g.M && gk < kEnd) ? __bfloat162float(A[(size_t)gm * g.lda_m + (size_t)gk * g.lda_k]) : 0.f;
		}
		for (int e = threadIdx.x; e < kT * kKt; e += 256) {
			int c, k;
			if (g.bContigK) {
				c = e / kKt;
				k = e - c * kKt;
			} else {
				k = e / kT;
				c = e - k * kT;
			}
			const int gn = n0 + c, gk = k0 + k;
			sb[k][c] = (gn < g.N && gk < kEnd) ? __bfloat162float(B[(size_t)gk * g.ldb_k + (size_t)gn * g.ldb_n]) : 0.f;
		}
		__syncthreads();
#pragma unroll
		for (int k = 0; k < kKt; ++k) {
			float a[4], b[4];
#pragma unroll
			for (int i = 0; i < 4; ++i) {
				a[i] = sa[k][ty + 16 * i];
				b[i] = sb[k][tx + 16 * i];
			}
#pragma unroll
			for (int i = 0; i < 4; ++i)
#pragma unroll
				for (int j = 0; j < 4; ++j)
					acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
		}
		__syncthreads();
	}
#pragma unroll
	for (int i = 0; i < 4; ++i)
#pragma unroll
		for (int j = 0; j < 4; ++j) {
			const int m = m0 + ty + 16 * i, n = n0 + tx + 16 * j;
			if (m >= g.M || n >= g.N)
				continue;
			if (split > 1)
				g.work[((size_t)blockIdx.z * g.M + m) * g.N + n] = acc[i][j];
			else
				mlpEpilogue(g, m, n, acc[i][j]);
		}
}

// sum of the K slices' partials in slice order, then the epilogue
__global__ void mlpSplitReduceKernel(const MlpGemm g)
{
	const size_t total = (size_t)g.M * g.N;
	for (size_t o = blockIdx.x * (size_t)blockDim.x + threadIdx.x; o < total; o += (size_t)gridDim.x * blockDim.x) {
		float v = 0.f;
		for (int z = 0; z < g.splitK; ++z)
			v += g.work[(size_t)z * total + o];
		mlpEpilogue(g, (int)(o / g.N), (int)(o % g.N), v);
	}
}

// column sums of an FP32 [M][N] matrix (bias gradients)
__global__ void colSumKernel(const float* X, int M, int N, float* out)
{
	const int n = blockIdx.x * blockDim.x + threadIdx.x;
	if (n >= N)
		return;
	float s = 0.f;
	for (int m = 0; m < M; ++m)
		s += X[(size_t)m * N + n];
	out[n] = s;
}

// squared error sum over n values (FP64 total, times `scale`) and
// dY = 2 (Y - T) scale
__global__ void mseKernel(const float* Y, const float* T, int n, float scale, float* dY32, uint16_t* dY16,
                          double* loss)
{
	double part = 0.;
	__nv_bfloat16* d16 = reinterpret_cast<__nv_bfloat16*>(dY16);
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		const float d = Y[i] - T[i];
		part += (double)d * d;
		const float gval = 2.f * d * scale;
		dY32[i] = gval;
		d16[i] = __float2bfloat16_rn(gval);
	}
	for (int o = 16; o > 0; o >>= 1)
		part += __shfl_xor_sync(0xffffffffu, part, o);
	if ((threadIdx.x & 31) == 0)
		atomicAdd(loss, part * (double)scale);
}

// Adam on FP32 master weights; refreshes the BF16 copy
__global__ void adamKernel(float* w, const float* g, float* m, float* v, uint16_t* w16, size_t n, float lr, float b1,
                           float b2, float eps, float c1, float c2)
{
	__nv_bfloat16* o16 = reinterpret_cast<__nv_bfloat16*>(w16);
	for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
		const float gi = g[i];
		const float mi = b1 * m[i] + (1.f - b1) * gi;
		const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
		m[i] = mi;
		v[i] = vi;
		const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
		w[i] = wi;
		o16[i] = __float2bfloat16_rn(wi);
	}
}

__global__ void toBf16Kernel(const float* x, uint16_t* y, size_t n)
{
	__nv_bfloat16* o = reinterpret_cast<__nv_bfloat16*>(y);
	for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
		o[i] = __float2bfloat16_rn(x[i]);
}

// rows idx[r] of src [*][rowLen] -> dst [r][rowLen] (element size esz bytes)
__global__ void gatherRowsKernel(const unsigned char* src, const uint32_t* idx, int rows, size_t rowBytes,
                                 unsigned char* dst)
{
	for (int r = blockIdx.x; r < rows; r += gridDim.x) {
		const unsigned char* s = src + (size_t)idx[r] * rowBytes;
		unsigned char* d = dst + (size_t)r * rowBytes;
		for (size_t i = threadIdx.x; i < rowBytes; i += blockDim.x)
			d[i] = s[i];
	}
}

}  // namespace

int mlpGemmSplit(const MlpGemm& g, int numSMs)
{
	const int tiles = ((g.N + kT - 1) / kT) * ((g.M + kT - 1) / kT);
	if (tiles >= numSMs || g.K < 8 * kKt)
		return 1;
	return std::max(1, std::min({16, (2 * numSMs + tiles - 1) / tiles, g.K / (4 * kKt)}));
}

int launchMlpGemm(const MlpGemm& g, cudaStream_t s)
{
	if (g.M <= 0 || g.N <= 0 || g.K <= 0)
		return setError(kErrArg, "MLP GEMM: empty shape");
	const int split = g.splitK > 1 ? g.splitK : 1;
	if (split > 1 && !g.work)
		return setError(kErrArg, "MLP GEMM: split K without a workspace");
	dim3 grid((g.N + kT - 1) / kT, (g.M + kT - 1) / kT, split);
	mlpGemmKernel<<<grid, 256, 0, s>>>(g);
	countLaunches(1);
	PWA_CHECK(cudaCheck(cudaGetLastError(), "MLP GEMM launch"));
	if (split == 1)
		return kOk;
	const size_t total = (size_t)g.M * g.N;
	const int blocks = (int)std::min<size_t>(4096, (total + 255) / 256);
	mlpSplitReduceKernel<<<blocks, 256, 0, s>>>(g);
	countLaunches(1);
	return cudaCheck(cudaGetLastError(), "MLP split-K reduce launch");
}

int launchColSum(const float* X, int M, int N, float* out, cudaStream_t s)
{
	colSumKernel<<<(N + 127) / 128, 128, 0, s>>>(X, M, N, out);
	countLaunches(1);
	return cudaCheck(cudaGetLastError(), "column sum launch");
}

int launchMse(const float* Y, const float* T, int n, float scale, float* dY32, uint16_t* dY16, double* loss,
              cudaStream_t s)
{
	const int blocks = std::min(1024, std::max(1, (n + 255) / 256));
	mseKernel<<<blocks, 256, 0, s>>>(Y, T, n, scale, dY32, dY16, loss);
	countLaunches(1);
	return cudaCheck(cudaGetLastError(), "MSE launch");
}

int launchAdam(float* w, const float* g, float* m, float* v, uint16_t* w16, size_t n, float lr, float b1, float b2,
               float eps, float c1, float c2, cudaStream_t s)
{
	const int blocks = (int)std::min<size_t>(2048, std::max<size_t>(1, (n + 255) / 256));
	adamKernel<<<blocks, 256, 0, s>>>(w, g, m, v, w16, n, lr, b1, b2, eps, c1, c2);
	countLaunches(1);
	return cudaCheck(cudaGetLastError(), "Adam launch");
}

int launchToBf16(const float* x, uint16_t* y, size_t n, cudaStream_t s)
{
	const int blocks = (int)std::min<size_t>(4096, std::max<size_t>(1, (n + 255) / 256));
	toBf16Kernel<<<blocks, 256, 0, s>>>(x, y, n);
	countLaunches(1);
	return cudaCheck(cudaGetLastError(), "bf16 conversion launch");
}

int launchGatherRows(const void* src, const uint32_t* idx, int rows, size_t rowBytes, void* dst, cudaStream_t s)
{
	const int blocks = std::min(4096, std::max(1, rows));
	gatherRowsKernel<<<blocks, 256, 0, s>>>(static_cast<const unsigned char*>(src), idx, rows, rowBytes,
	                                        static_cast<unsigned char*>(dst));
	countLaunches(1);
	return cudaCheck(cudaGetLastError(), "row gather launch");
}

}  // namespace pwa
