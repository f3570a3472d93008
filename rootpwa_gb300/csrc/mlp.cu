// mlp.cu -- the warm-start network: a 3-layer perceptron
//   h1 = relu(W1 x + b1), h2 = relu(W2 h1 + b2), y = W3 h2 + b3
// with BF16 weights and activations, FP32 accumulation, FP32 master weights,
// its backward pass and an Adam update, all as hand-written kernels.
//
// One tensor-core GEMM kernel serves every product: C[M][N] = sum_k A(m, k)
// B(k, n) with A and B read through strides (so that X W^T, dY W and dY^T X
// are the same kernel).  128 x 128 output tiles; per K step of 64 the four
// loader warps read both operand tiles from global memory (along whichever
// dimension is contiguous) and write them in the canonical K-major
// 128-byte-swizzled layout, one thread issues four tcgen05.mma kind::f16
// (BF16 operands, M = N = 128, K = 16) into an FP32 accumulator in tensor
// memory (128 columns), two operand stages alternate.  The product is split
// into K slices, one block per (tile, slice), so that the grid covers the
// GPU (the batch has 256 rows, the layers 102 to 512 columns); the loader
// warps then move the accumulator to the slice's FP32 partials, and a second
// kernel sums the slices in slice order (deterministic) and applies the
// epilogue: bias, relu or a relu mask, FP32 and/or BF16 stores.

#include "pwa_internal.h"
#include "tcgen05.cuh"

#include <cuda_bf16.h>

#include <algorithm>

namespace pwa {
namespace {

constexpr int kTcTile = 128;                       // output tile 128 x 128
constexpr int kTcK = 64;                           // K per stage: one 128-byte row of BF16
constexpr int kTcLoadWarps = 4;                    // loaders, then the drain (warp = lane quarter)
constexpr int kTcMmaWarp = kTcLoadWarps;           // warp 4
constexpr int kTcThreads = (kTcLoadWarps + 1) * 32;
constexpr int kTcStages = 2;
constexpr uint32_t kTcOpBytes = kTcTile * 128u;    // one operand tile: 128 rows x 64 BF16
constexpr uint32_t kTcCols = 128;                  // tensor-memory columns of the accumulator
constexpr size_t kTcSmem = 1024 + 2u * kTcStages * kTcOpBytes + 128;

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

// one 128 x 64 operand tile in the K-major swizzled layout: row r, k of
// element (r, k) = X[r * ldr + k * ldk] of rows r0.., k0.. (zero beyond
// nR rows or kEnd); 128 loader threads, each storing 16-byte chunks of 8 k
__device__ __forceinline__ void loadTile(unsigned char* dst, const uint16_t* X, size_t ldr, size_t ldk, int contigK,
                                         int r0, int nR, int k0, int kEnd, int t)
{
	if (contigK) {
		// thread t: chunks t, t + 128, ... (8 per thread): row c / 8, k-chunk c % 8
#pragma unroll 2
		for (int j = 0; j < 8; ++j) {
			const int c = t + 128 * j, r = c >> 3, kc = (c & 7) * 8;
			uint32_t w[4] = {0u, 0u, 0u, 0u};
			if (r0 + r < nR) {
				const uint16_t* src = X + (size_t)(r0 + r) * ldr;
#pragma unroll
				for (int i = 0; i < 8; ++i) {
					const int k = k0 + kc + i;
					const uint32_t v = k < kEnd ? src[k] : 0u;
					w[i >> 1] |= v << (16 * (i & 1));
				}
			}
			*reinterpret_cast<uint4*>(dst + swzOffset16(r, kc)) = make_uint4(w[0], w[1], w[2], w[3]);
		}
	} else {
		// thread t: row t, all 8 k-chunks (neighbouring threads read neighbouring rows)
		const int r = t;
		const bool in = r0 + r < nR;
#pragma unroll 2
		for (int kc = 0; kc < kTcK; kc += 8) {
			uint32_t w[4] = {0u, 0u, 0u, 0u};
			if (in) {
#pragma unroll
				for (int i = 0; i < 8; ++i) {
					const int k = k0 + kc + i;
					const uint32_t v = k < kEnd ? X[(size_t)(r0 + r) * ldr + (size_t)k * ldk] : 0u;
					w[i >> 1] |= v << (16 * (i & 1));
				}
			}
			*reinterpret_cast<uint4*>(dst + swzOffset16(r, kc)) = make_uint4(w[0], w[1], w[2], w[3]);
		}
	}
}

// C tile (blockIdx.y, blockIdx.x) over K slice blockIdx.z -> g.work[z][M][N]
__global__ void __launch_bounds__(kTcThreads) mlpGemmTcKernel(const MlpGemm g, int kPerSlice)
{
	extern __shared__ __align__(1024) unsigned char smemRaw[];
	unsigned char* smem =
	    reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smemRaw) + 1023) & ~uintptr_t(1023));
	unsigned char* opA = smem;                                 // [stages][128 x 128 B]
	unsigned char* opB = smem + kTcStages * kTcOpBytes;        // [stages][128 x 128 B]
	uint64_t* full = reinterpret_cast<uint64_t*>(opB + kTcStages * kTcOpBytes);
	uint64_t* empty = full + kTcStages;
	uint64_t* done = empty + kTcStages;
	uint32_t* tmemHolder = reinterpret_cast<uint32_t*>(done + 1);
	__shared__ unsigned sFail;

	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const int m0 = blockIdx.y * kTcTile, n0 = blockIdx.x * kTcTile;
	const int kBeg = (int)blockIdx.z * kPerSlice, kEnd = min(g.K, kBeg + kPerSlice);
	const int nSteps = kEnd > kBeg ? (kEnd - kBeg + kTcK - 1) / kTcK : 0;
	const uint16_t* A = g.A;
	const uint16_t* B = g.B;

	if (tid == 0) {
		for (int s = 0; s < kTcStages; ++s) {
			barInit(&full[s], kTcLoadWarps);
			barInit(&empty[s], 1);
		}
		barInit(done, 1);
		sFail = 0u;
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	if (warp == kTcMmaWarp) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sAddr(tmemHolder)),
		             "r"(kTcCols)
		             : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
	}
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
	__syncthreads();
	asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
	const uint32_t tmem = *tmemHolder;

	if (warp < kTcLoadWarps) {
		// ---- loaders: both operand tiles of every K step ----
		bool ok = true;
		for (int t = 0; t < nSteps; ++t) {
			const int s = t % kTcStages;
			if (t >= kTcStages && !barWait(&empty[s], (uint32_t)(((t / kTcStages) - 1) & 1))) {
				atomicOr(g.devErr, (unsigned)kDevErrTimeout);
				sFail = 1u;
				ok = false;
				break;
			}
			const int k0 = kBeg + t * kTcK;
			// A(m, k) = A[m lda_m + k lda_k]; B(k, n) = B[k ldb_k + n ldb_n] as rows n
			loadTile(opA + s * kTcOpBytes, A, g.lda_m, g.lda_k, g.aContigK, m0, g.M, k0, kEnd, tid);
			loadTile(opB + s * kTcOpBytes, B, g.ldb_n, g.ldb_k, g.bContigK, n0, g.N, k0, kEnd, tid);
			asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
			__syncwarp();
			if (lane == 0)
				barArrive(&full[s]);
		}
		// ---- drain: the accumulator rows of this warp's lane quarter ----
		if (ok && nSteps > 0 && !barWait(done, 0u)) {
			atomicOr(g.devErr, (unsigned)kDevErrTimeout);
			ok = false;
		}
		if (ok) {
			asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
			const int m = m0 + warp * 32 + lane;
			float* out = g.work + ((size_t)blockIdx.z * g.M + (size_t)(m < g.M ? m : 0)) * g.N;
			for (int c = 0; c < kTcTile; c += 16) {
				uint32_t r[16];
				if (nSteps > 0) {
					tmemLd16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, r);
					asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
				} else {
#pragma unroll
					for (int i = 0; i < 16; ++i)
						r[i] = 0u;
				}
				if (m < g.M)
#pragma unroll
					for (int i = 0; i < 16; ++i)
						if (n0 + c + i < g.N)
							out[n0 + c + i] = __uint_as_float(r[i]);
			}
		}
	} else if (lane == 0) {
		// ---- MMA issuer ----
		const uint32_t idesc = idescBf16(kTcTile, kTcTile);
		int t = 0;
		for (; t < nSteps; ++t) {
			const int s = t % kTcStages;
			if (!barWait(&full[s], (uint32_t)((t / kTcStages) & 1))) {
				atomicOr(g.devErr, (unsigned)kDevErrTimeout);
				sFail = 1u;
				break;
			}
			asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
			const uint64_t aD = smemDesc(sAddr(opA + s * kTcOpBytes)), bD = smemDesc(sAddr(opB + s * kTcOpBytes));
#pragma unroll
			for (uint32_t kk = 0; kk < 4; ++kk)
				mmaBf16(tmem, aD + 2 * kk, bD + 2 * kk, idesc, (t > 0 || kk > 0) ? 1u : 0u);
			mmaCommit(&empty[s]);
		}
		// all MMAs of this block complete before the drain reads tensor memory
		mmaCommit(done);
		if (t < nSteps || nSteps == 0)
			barWait(done, 0u);
	}
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
	__syncthreads();
	if (warp == kTcMmaWarp) {
		asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcCols) : "memory");
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
	// K slices of whole K steps, so that the blocks cover the SMs about twice
	const int tiles = ((g.N + kTcTile - 1) / kTcTile) * ((g.M + kTcTile - 1) / kTcTile);
	const int steps = (g.K + kTcK - 1) / kTcK;
	return std::max(1, std::min(steps, (2 * numSMs + tiles - 1) / tiles));
}

int launchMlpGemm(const MlpGemm& g, cudaStream_t s)
{
	if (g.M <= 0 || g.N <= 0 || g.K <= 0)
		return setError(kErrArg, "MLP GEMM: empty shape");
	if (!g.work || g.splitK < 1 || !g.devErr)
		return setError(kErrArg, "MLP GEMM: workspace, K slices and error flag required");
	const int steps = (g.K + kTcK - 1) / kTcK;
	const int kPerSlice = ((steps + g.splitK - 1) / g.splitK) * kTcK;
	const int slices = (g.K + kPerSlice - 1) / kPerSlice;
	static bool configured = false;
	if (!configured) {
		PWA_CHECK(cudaCheck(cudaFuncSetAttribute(mlpGemmTcKernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
		                                         (int)kTcSmem),
		                    "MLP GEMM smem attribute"));
		configured = true;
	}
	dim3 grid((g.N + kTcTile - 1) / kTcTile, (g.M + kTcTile - 1) / kTcTile, slices);
	mlpGemmTcKernel<<<grid, kTcThreads, kTcSmem, s>>>(g, kPerSlice);
	countLaunches(1);
	PWA_CHECK(cudaCheck(cudaGetLastError(), "MLP GEMM launch"));
	MlpGemm r = g;
	r.splitK = slices;
	const size_t total = (size_t)g.M * g.N;
	const int blocks = (int)std::min<size_t>(4096, (total + 255) / 256);
	mlpSplitReduceKernel<<<blocks, 256, 0, s>>>(r);
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
