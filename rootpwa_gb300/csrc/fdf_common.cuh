// fdf_common.cuh -- pieces shared by the FdF kernels (fdf_kernels.cu,
// fdf_fused.cu): block shape, the exact fixed-point cross-block sums, the
// normalisation/prior terms and the last block's tail.
#pragma once

#include "pwa_internal.h"
#include "device_common.cuh"

namespace pwa {
namespace {


constexpr int kThreads = 512;
constexpr int kWarps = kThreads / 32;

// Exact cross-block sums: a value x is truncated to a 128-bit two's-
// complement fixed-point number X = trunc(x * 2^64) (64 integer, 64 fraction
// bits), split into four 32-bit limbs; each limb is added to its own 64-bit
// counter with a fire-and-forget atomic (no carries: a counter cannot
// overflow for fewer than 2^32 additions).  Integer addition is associative,
// so the totals do not depend on the order in which blocks arrive (bitwise
// reproducible).  The conversion uses integer operations on the IEEE-754
// fields only.  The last block propagates the carries once.
//
// Layout of the accumulators: [replica][limb][value] (the last block reads a
// limb of consecutive values with coalesced loads).
constexpr int kLimbs = 4;

// Number of replicas of the accumulators: block b adds into replica
// b % kReplicas, which divides the atomic contention per address.
constexpr int kReplicas = 8;

// Adds x to value slot `acc` (limb stride `ls` words).  Values outside the
// fixed-point range (|x| >= 2^63, inf, NaN) go to an FP64 accumulator
// instead: inf and NaN propagate the same way in any order.
__device__ __forceinline__ void fixedAdd(unsigned long long* acc, size_t ls, double* nf, double x)
{
	const unsigned long long b = (unsigned long long)__double_as_longlong(x);
	const int e = (int)((b >> 52) & 0x7ffull);
	if (e >= 1023 + 63) {  // |x| >= 2^63, inf or NaN
		atomicAdd(nf, x);
		return;
	}
	// |x| = m 2^(e - 1075); X = m 2^sh with sh = e - 1075 + 64
	const unsigned long long m = (b & 0xfffffffffffffull) | 0x10000000000000ull;
	const int sh = e - 1011;
	if (e == 0 || sh <= -53)  // zero, subnormal or below 2^-64
		return;
	unsigned long long lo, hi;
	if (sh >= 64) {
		lo = 0ull;
		hi = m << (sh - 64);
	} else if (sh > 0) {
		lo = m << sh;
		hi = m >> (64 - sh);
	} else {
		lo = m >> (-sh);
		hi = 0ull;
	}
	if (b >> 63) {  // two's-complement negation of hi:lo
		lo = ~lo + 1ull;
		hi = ~hi + (lo == 0ull ? 1ull : 0ull);
	}
	const unsigned long long l0 = lo & 0xffffffffull, l1 = lo >> 32, l2 = hi & 0xffffffffull, l3 = hi >> 32;
	if (l0)
		atomicAdd(acc, l0);
	if (l1)
		atomicAdd(acc + ls, l1);
	if (l2)
		atomicAdd(acc + 2 * ls, l2);
	if (l3)
		atomicAdd(acc + 3 * ls, l3);
}

// Exact sum of the kReplicas replicas (replica stride `rs`, limb stride `ls`
// words) of one value slot with the carries propagated, converted to FP64,
// plus its out-of-range part; clears the slot for the next launch.
__device__ __forceinline__ double fixedTake(unsigned long long* acc, size_t rs, size_t ls, double* nf)
{
	unsigned long long l[kLimbs] = {0ull, 0ull, 0ull, 0ull};
#pragma unroll
	for (int q = 0; q < kReplicas; ++q)
#pragma unroll
		for (int k = 0; k < kLimbs; ++k) {
			unsigned long long* p = acc + q * rs + k * ls;
			l[k] += __ldcg(p);
			__stcg(p, 0ull);
		}
	// carries: the value is limb3:limb2:limb1:limb0 in base 2^32
	l[1] += l[0] >> 32;
	l[2] += l[1] >> 32;
	l[3] += l[2] >> 32;
	const unsigned long long lo = (l[0] & 0xffffffffull) | (l[1] << 32);
	const unsigned long long hi = (l[2] & 0xffffffffull) | (l[3] << 32);
	const double out = __ldcg(nf);
	__stcg(nf, 0.);
	return ((double)(long long)hi + (double)lo * 5.42101086242752217e-20) + out;  // lo * 2^-64
}

// Normalisation and prior terms (pwaLikelihood.cc:254-297) of a share of
// the slots in FP64: D = sum_j V_j conj(I_ij) over the same reflectivity and
// the half-Cauchy value and gradient; nEvt Re(V_i conj(D)) + prior goes into
// value slot 0 (LL) and 2 nEvt D - prior gradient into the slot's gradient
// values, so that the exact cross-block sums carry them.  The slots go to the
// blocks with one tile fewer than the others (they finish a tile earlier), or
// to all blocks when every block has the same number of tiles; warp j of a
// block takes its j-th slot.
__device__ __forceinline__ void fdfNormTerms(const FdfArgs& a, const double2* V64, uint64_t nTiles,
                                             unsigned long long* myAcc, size_t ls, int warp, int lane)
{
	const int W = a.W, W0 = a.W0, R = a.R;
	const int nSlots = R * W;
	const int grid = (int)gridDim.x;
	const int rem = (int)(nTiles % (uint64_t)grid);
	// blocks b >= rem have one tile fewer when rem > 0
	const int first = (rem > 0 && nTiles > (uint64_t)grid) ? rem : 0;
	const int nb = grid - first;
	if ((int)blockIdx.x < first)
		return;
	const int me = (int)blockIdx.x - first;
	const double g2 = a.cauchyWidth * a.cauchyWidth;
	for (int j = warp; me + j * nb < nSlots; j += kWarps) {
		const int sl = me + j * nb;
		const int r = sl / W, g = sl - r * W;
		const int pos = (g >= W0) ? 1 : 0;
		const int off = pos ? W0 : 0, We = pos ? W - W0 : W0, i = g - off;
		const double* Ib = a.accI + (pos ? 2 * (size_t)W0 * W0 : 0) + 2 * (size_t)i * We;
		double dre = 0., dim = 0.;
#pragma unroll 4
		for (int q = lane; q < We; q += 32) {
			const double2 u = V64[r * W + off + q];
			const double Ir = __ldg(Ib + 2 * q), Ii = __ldg(Ib + 2 * q + 1);
			dre += u.x * Ir + u.y * Ii;  // V_q conj(I_iq)
			dim += u.y * Ir - u.x * Ii;
		}
		dre = warpSumD(dre);
		dim = warpSumD(dim);
		if (lane == 0) {
			const double2 v = V64[sl];
			double priorv = 0., pre = 0., pim = 0.;
			if (a.prior == 1) {
				const double rr = hypot(v.x, v.y);
				const double cf = 1. / (1. + (rr * rr) / g2);
				const double cd = (-2. * rr * g2) / ((g2 + rr * rr) * (g2 + rr * rr));
				const double fac = (1. / (rr * cf)) * cd;
				priorv = -log(cf);
				pre = fac * v.x;
				pim = fac * v.y;
			}
			const double twice = 2. * a.nEvt;
			// Re(V_i conj(D_i))
			fixedAdd(myAcc, ls, a.nfAcc, a.nEvt * (v.x * dre + v.y * dim) + priorv);
			if (a.withGrad) {
				fixedAdd(myAcc + 2 + 2 * sl, ls, a.nfAcc + 2 + 2 * sl, twice * dre - pre);
				fixedAdd(myAcc + 3 + 2 * sl, ls, a.nfAcc + 3 + 2 * sl, twice * dim - pim);
			}
		}
	}
}

// The last block to arrive reads the exact totals and writes f and the
// gradient in the parameter layout (pwaLikelihood.cc:300-304, :1716-1731),
// clearing the accumulators for the next launch as it reads them: one value
// slot per thread.  Value slot 0 holds LL plus the normalisation and prior
// terms, 1 sum c, 2 + 2 s (+1) the gradient re (im) of production-amplitude
// slot s.
__device__ __forceinline__ void fdfTail(const FdfArgs& a, unsigned* sLast, double flatD, int tid)
{
	__threadfence();
	__syncthreads();
	if (tid == 0)
		*sLast = (atomicAdd(a.counter, 1u) == gridDim.x - 1) ? 1u : 0u;
	__syncthreads();
	if (!*sLast)
		return;
	__threadfence();
	const size_t ls = (size_t)a.nPartial, rs = (size_t)kLimbs * ls;
	const double twice = 2. * a.nEvt;
	const int nVals = a.withGrad ? a.nPartial : 2;
	for (int v = tid; v < nVals; v += kThreads) {
		const unsigned err = (v == 0) ? *(const volatile unsigned*)a.devErr : 0u;
		const int idx = (v < 2) ? -1 : (((v & 1) == 0) ? a.slotRe[(v - 2) >> 1] : a.slotIm[(v - 2) >> 1]);
		const double x = fixedTake(a.fixAcc + v, rs, ls, a.nfAcc + v);
		if (v == 0) {
			a.out[0] = x + a.nEvt * flatD * flatD * a.totAcc;
			a.out[a.P + 1] = (double)err;
			*a.counter = 0u;
		} else if (v == 1) {
			if (a.withGrad)
				a.out[a.P] = flatD * x + twice * flatD * a.totAcc;
		} else if (idx >= 0) {
			a.out[1 + idx] = x;
		}
	}
}

}  // namespace
}  // namespace pwa
