// hessian_kernels.cu -- per-event operands of the analytic Hessian.
//
// The event term of pwaLikelihood::Hessian (partialWaveFit/pwaLikelihood.cc:
// 676-735) is a sum over events of products of
//   d_s = S_{r(s),e(s)} conj(A_{w(s)})      (slot s = (rank, wave))
// weighted by f^2 (f = 2/L) plus a same-(rank, reflectivity) block of
// f A_i conj(A_j).  This kernel writes, for one slab of events, the complex
// columns [d; conj(d); 1] and [A; 1] with weights f^2 and f, so that two
// weighted complex Gram products (the tensor-core Gram of gram_tc.cu, TF32x3,
// in pairs of 48-row groups for the wide first set) yield
//   sum f^2 d_i conj(d_j), sum f^2 d_i d_j, sum f^2 d_i, sum f^2,
//   sum f A_i conj(A_j), sum f
// from which the host assembles the three real blocks the reference keeps
// per slot pair.  Coherent sums are FP32; the Gram sums FP32 in tensor
// memory per few tiles and FP64 across CTAs and slabs.

#include "pwa_internal.h"

#include <algorithm>

namespace pwa {
namespace {

constexpr int kMaxRW = 1024;  // rank x waves held in shared memory

__global__ void __launch_bounds__(256) hessPrepKernel(const float2* __restrict__ amps, uint64_t nEvents, uint32_t B,
                                                      uint64_t e0, uint64_t slab, int W0, int W, int R, int P,
                                                      const double* __restrict__ par, const int* __restrict__ slotRe,
                                                      const int* __restrict__ slotIm, float2* Y1, float2* Y2,
                                                      double* w1, double* w2)
{
	__shared__ float2 Vs[kMaxRW];
	const int nS = R * W;
	for (int k = threadIdx.x; k < nS; k += blockDim.x) {
		const int ir = slotRe[k], ii = slotIm[k];
		Vs[k] = make_float2(ir >= 0 ? (float)par[ir] : 0.f, ii >= 0 ? (float)par[ii] : 0.f);
	}
	__syncthreads();
	const double flat = par[P - 1];
	const float flat2 = (float)(flat * flat);
	for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < slab; t += (uint64_t)gridDim.x * blockDim.x) {
		const uint64_t ev = e0 + t;
		const bool valid = ev < nEvents;
		const uint64_t col = valid ? ev : 0;
		// L and f
		float L = flat2;
		for (int r = 0; r < R; ++r) {
			float2 S0 = make_float2(0.f, 0.f), S1 = make_float2(0.f, 0.f);
			for (int w = 0; w < W; ++w) {
				const float2 a = amps[storeIndex((uint32_t)w, col, (uint32_t)W, B)];
				const float2 v = Vs[r * W + w];
				float2& S = (w < W0) ? S0 : S1;
				S.x = fmaf(v.x, a.x, fmaf(-v.y, a.y, S.x));
				S.y = fmaf(v.x, a.y, fmaf(v.y, a.x, S.y));
			}
			L = fmaf(S0.x, S0.x, fmaf(S0.y, S0.y, L));
			L = fmaf(S1.x, S1.x, fmaf(S1.y, S1.y, L));
		}
		const float f = valid ? 2.f / L : 0.f;
		w1[t] = valid ? (double)f * (double)f : 0.;
		w2[t] = valid ? (double)f : 0.;
		// d_s and conj(d_s); recompute the coherent sums per rank
		for (int r = 0; r < R; ++r) {
			float2 S0 = make_float2(0.f, 0.f), S1 = make_float2(0.f, 0.f);
			for (int w = 0; w < W; ++w) {
				const float2 a = amps[storeIndex((uint32_t)w, col, (uint32_t)W, B)];
				const float2 v = Vs[r * W + w];
				float2& S = (w < W0) ? S0 : S1;
				S.x = fmaf(v.x, a.x, fmaf(-v.y, a.y, S.x));
				S.y = fmaf(v.x, a.y, fmaf(v.y, a.x, S.y));
			}
			for (int w = 0; w < W; ++w) {
				const float2 a = amps[storeIndex((uint32_t)w, col, (uint32_t)W, B)];
				const float2 S = (w < W0) ? S0 : S1;
				// S conj(a)
				const float2 d = make_float2(S.x * a.x + S.y * a.y, S.y * a.x - S.x * a.y);
				Y1[(size_t)(r * W + w) * slab + t] = d;
				Y1[(size_t)(nS + r * W + w) * slab + t] = make_float2(d.x, -d.y);
			}
		}
		Y1[(size_t)(2 * nS) * slab + t] = make_float2(1.f, 0.f);
		for (int w = 0; w < W; ++w)
			Y2[(size_t)w * slab + t] = amps[storeIndex((uint32_t)w, col, (uint32_t)W, B)];
		Y2[(size_t)W * slab + t] = make_float2(1.f, 0.f);
	}
}

}  // namespace

int launchHessPrep(const float2* amps, uint64_t nEvents, uint32_t B, uint64_t e0, uint64_t slab, int W0, int W,
                   int R, int P, const double* par, const int* slotRe, const int* slotIm, float2* Y1, float2* Y2,
                   double* w1, double* w2, cudaStream_t s)
{
	if (R * W > kMaxRW)
		return setError(kErrUnsupported, "Hessian kernel supports rank x waves <= 1024");
	const int threads = 256;
	const int blocks = (int)std::max<uint64_t>(1, std::min<uint64_t>((slab + threads - 1) / threads, 8192));
	hessPrepKernel<<<blocks, threads, 0, s>>>(amps, nEvents, B, e0, slab, W0, W, R, P, par, slotRe, slotIm, Y1, Y2,
	                                          w1, w2);
	countLaunches(1);
	return cudaCheck(cudaGetLastError(), "hessian prep launch");
}

}  // namespace pwa
