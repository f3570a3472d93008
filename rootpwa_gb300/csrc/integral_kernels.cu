// integral_kernels.cu -- SIMT Gram kernels for the MC integral matrices.
//
// Computes the raw sums of ampIntegralMatrix::integrate
// (decayAmplitude/ampIntegralMatrix.cc:408-469)
//   I_ij = sum_k w_k A_{i,k} conj(A_{j,k})
// over K = events x sub-amplitudes, for the upper triangle of 64 x 64 output
// tiles.  Each CTA owns one output tile and one contiguous chunk of K; a
// 16 x 16 thread grid holds 4 x 4 complex accumulators per thread (FP32 or
// FP64).  Chunk partials are summed in FP64 by a second kernel, which also
// mirrors the upper triangle into the lower one (the reference's matrix is
// exactly Hermitian, since a conj(b) and b conj(a) round identically).
// The tensor-core variant lives in gram_tc.cu.

#include "pwa_internal.h"

#include <algorithm>

namespace pwa {
namespace {

constexpr int kTile = 64;
constexpr int kKT = 16;

template <typename In>
struct InTraits;
template <>
struct InTraits<float2> {
	__device__ static double2 load(const float2* p, uint64_t i)
	{
		const float2 v = p[i];
		return make_double2(v.x, v.y);
	}
};
template <>
struct InTraits<double2> {
	__device__ static double2 load(const double2* p, uint64_t i) { return p[i]; }
};

template <typename T>
struct Cplx {
	T x, y;
};

template <typename In, typename Acc>
__global__ void __launch_bounds__(256) gramSimtKernel(const In* __restrict__ amps, uint64_t K, uint64_t ldK, int W,
                                                      const double* __restrict__ weightK, double* partials,
                                                      int tilesPerSide, uint64_t chunkLen)
{
	__shared__ Cplx<Acc> sa[kKT][kTile + 1];
	__shared__ Cplx<Acc> sb[kKT][kTile + 1];
	// decode upper-triangle tile index (ti <= tj)
	int t = blockIdx.x, ti = 0;
	while (t >= tilesPerSide - ti) {
		t -= tilesPerSide - ti;
		++ti;
	}
	const int tj = ti + t;
	const int chunk = blockIdx.y;
	const uint64_t k0 = (uint64_t)chunk * chunkLen;
	const uint64_t k1 = min(K, k0 + chunkLen);
	const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
	const int i0 = ti * kTile, j0 = tj * kTile;

	Cplx<Acc> acc[4][4];
#pragma unroll
	for (int a = 0; a < 4; ++a)
#pragma unroll
		for (int b = 0; b < 4; ++b)
			acc[a][b] = Cplx<Acc>{Acc(0), Acc(0)};

	for (uint64_t kb = k0; kb < k1; kb += kKT) {
		// load 64 rows x 16 K of both operands; thread -> (row, k) pairs
		for (int idx = threadIdx.x; idx < kTile * kKT; idx += 256) {
			const int row = idx / kKT, kk = idx - row * kKT;
			const uint64_t k = kb + kk;
			Cplx<Acc> va{Acc(0), Acc(0)}, vb{Acc(0), Acc(0)};
			if (k < k1) {
				const int gi = i0 + row, gj = j0 + row;
				const Acc w = weightK ? (Acc)weightK[k] : Acc(1);
				if (gi < W) {
					const double2 v = InTraits<In>::load(amps, (uint64_t)gi * ldK + k);
					va = Cplx<Acc>{(Acc)v.x * w, (Acc)v.y * w};
				}
				if (gj < W) {
					const double2 v = InTraits<In>::load(amps, (uint64_t)gj * ldK + k);
					vb = Cplx<Acc>{(Acc)v.x, (Acc)v.y};
				}
			}
			sa[kk][row] = va;
			sb[kk][row] = vb;
		}
		__syncthreads();
#pragma unroll
		for (int kk = 0; kk < kKT; ++kk) {
			Cplx<Acc> a[4], b[4];
#pragma unroll
			for (int q = 0; q < 4; ++q) {
				a[q] = sa[kk][ty + 16 * q];
				b[q] = sb[kk][tx + 16 * q];
			}
#pragma unroll
			for (int p = 0; p < 4; ++p)
#pragma unroll
				for (int q = 0; q < 4; ++q) {
					// a conj(b)
					acc[p][q].x = fma(a[p].x, b[q].x, fma(a[p].y, b[q].y, acc[p][q].x));
					acc[p][q].y = fma(a[p].y, b[q].x, fma(-a[p].x, b[q].y, acc[p][q].y));
				}
		}
		__syncthreads();
	}
	double* out = partials + (size_t)chunk * W * W * 2;
#pragma unroll
	for (int p = 0; p < 4; ++p)
#pragma unroll
		for (int q = 0; q < 4; ++q) {
			const int gi = i0 + ty + 16 * p, gj = j0 + tx + 16 * q;
			if (gi < W && gj < W && gi <= gj) {
				out[((size_t)gi * W + gj) * 2] = (double)acc[p][q].x;
				out[((size_t)gi * W + gj) * 2 + 1] = (double)acc[p][q].y;
			}
		}
}

// Sums chunk partials (upper triangle) in FP64 and writes the full Hermitian
// matrix; the diagonal's imaginary part is exactly zero as in the reference.
__global__ void gramReduceKernel(const double* partials, int chunks, int W, double* out, int accumulate)
{
	const int n = W * W;
	for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
		const int i = e / W, j = e - i * W;
		if (i > j)
			continue;
		double re = 0., im = 0.;
		for (int c = 0; c < chunks; ++c) {
			re += partials[((size_t)c * n + e) * 2];
			im += partials[((size_t)c * n + e) * 2 + 1];
		}
		if (i == j)
			im = 0.;
		if (accumulate) {
			re += out[(size_t)e * 2];
			im += out[(size_t)e * 2 + 1];
		}
		out[(size_t)e * 2] = re;
		out[(size_t)e * 2 + 1] = im;
		out[((size_t)j * W + i) * 2] = re;
		out[((size_t)j * W + i) * 2 + 1] = -im;
	}
}

}  // namespace

int launchGramSimt(const GramArgs& a, int precision, cudaStream_t s)
{
	const int tps = (a.W + kTile - 1) / kTile;
	const int nTiles = tps * (tps + 1) / 2;
	const uint64_t chunkLen = ((a.K + a.chunks - 1) / a.chunks + kKT - 1) / kKT * kKT;
	dim3 grid(nTiles, a.chunks);
	if (precision == 0) {
		if (a.amps64)
			gramSimtKernel<double2, double><<<grid, 256, 0, s>>>(a.amps64, a.K, a.ldK, a.W, a.weightK, a.partials, tps,
			                                                     chunkLen);
		else
			gramSimtKernel<float2, double><<<grid, 256, 0, s>>>(a.amps, a.K, a.ldK, a.W, a.weightK, a.partials, tps,
			                                                    chunkLen);
	} else {
		gramSimtKernel<float2, float><<<grid, 256, 0, s>>>(a.amps, a.K, a.ldK, a.W, a.weightK, a.partials, tps,
		                                                   chunkLen);
	}
	countLaunches(1);
	return cudaCheck(cudaGetLastError(), "gram SIMT launch");
}

// out += the blocks of a Gram of two row groups: rows and columns i < G of
// blk belong to group a (global index a G + i), the others to group b
// (b G + i - G); the cross blocks are always added, the diagonal blocks of
// group a / b only when addAA / addBB (another pair may supply them);
// indices >= nOut are padding and skipped.  One group (G = n2) adds all.
__global__ void gramBlockAddKernel(const double* blk, int n2, int G, int a, int b, int nOut, int addAA, int addBB,
                                   double* out)
{
	const int n = n2 * n2;
	for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
		const int i = e / n2, j = e - i * n2;
		const bool ia = i < G, ja = j < G;
		if ((ia && ja && !addAA) || (!ia && !ja && !addBB))
			continue;
		const int gi = ia ? a * G + i : b * G + (i - G), gj = ja ? a * G + j : b * G + (j - G);
		if (gi >= nOut || gj >= nOut)
			continue;
		out[((size_t)gi * nOut + gj) * 2] += blk[(size_t)e * 2];
		out[((size_t)gi * nOut + gj) * 2 + 1] += blk[(size_t)e * 2 + 1];
	}
}

int launchGramBlockAdd(const double* blk, int n2, int G, int a, int b, int nOut, int addAA, int addBB, double* out,
                       cudaStream_t s)
{
	const int n = n2 * n2;
	const int blocks = std::max(1, std::min(1024, (n + 255) / 256));
	gramBlockAddKernel<<<blocks, 256, 0, s>>>(blk, n2, G, a, b, nOut, addAA, addBB, out);
	countLaunches(1);
	return cudaCheck(cudaGetLastError(), "gram block add launch");
}

int launchGramReduce(const double* partials, int chunks, int W, double* out, int accumulate, cudaStream_t s)
{
	const int n = W * W;
	const int blocks = std::max(1, std::min(1024, (n + 255) / 256));
	gramReduceKernel<<<blocks, 256, 0, s>>>(partials, chunks, W, out, accumulate);
	countLaunches(1);
	return cudaCheck(cudaGetLastError(), "gram reduce launch");
}

namespace {

// out[w] = sum_k a[w][k] (complex64 rows of stride ld): one block per row,
// compensated FP32 sums per thread (GB300's FP64 pipe is a small fraction
// of its FP32 rate, and one FP64 add per element made this kernel slower
// than the Gram itself), FP64 across the block's threads, a fixed reduction
// order (thread-strided partial sums, then a shared-memory tree), so the
// result does not depend on the run.
__global__ void __launch_bounds__(256) rowSumsKernel(const float2* __restrict__ a, uint64_t n, uint64_t ld,
                                                     double* out)
{
	__shared__ double sre[256], sim[256];
	const float2* row = a + (uint64_t)blockIdx.x * ld;
	float re = 0.f, im = 0.f, cre = 0.f, cim = 0.f;
	for (uint64_t k = threadIdx.x; k < n; k += 256) {
		const float2 v = row[k];
		const float yr = v.x - cre, tr = re + yr;
		cre = (tr - re) - yr;
		re = tr;
		const float yi = v.y - cim, ti = im + yi;
		cim = (ti - im) - yi;
		im = ti;
	}
	sre[threadIdx.x] = (double)re - (double)cre;
	sim[threadIdx.x] = (double)im - (double)cim;
	__syncthreads();
	for (int o = 128; o > 0; o >>= 1) {
		if ((int)threadIdx.x < o) {
			sre[threadIdx.x] += sre[threadIdx.x + o];
			sim[threadIdx.x] += sim[threadIdx.x + o];
		}
		__syncthreads();
	}
	if (threadIdx.x == 0) {
		out[2 * blockIdx.x] = sre[0];
		out[2 * blockIdx.x + 1] = sim[0];
	}
}

}  // namespace

int launchRowSums(const float2* a, uint64_t n, uint64_t ld, int W, double* out, cudaStream_t s)
{
	rowSumsKernel<<<W, 256, 0, s>>>(a, n, ld, out);
	countLaunches(1);
	return cudaCheck(cudaGetLastError(), "row sums launch");
}

}  // namespace pwa
