// multibin.cu -- batched FdF over many kinematic bins x many start points,
// its per-problem finish (cross-item sums, normalisation and prior terms) and
// a batched L-BFGS step, for whole multibin multi-start fits on the GPU.
//
// A "problem" is one (bin, start point) pair with its own parameter vector in
// the pwaLikelihood layout (partialWaveFit/pwaLikelihood.cc:1487-1556).  All
// bins share the wave set.  For rank 1 with one reflectivity and at most 64
// waves one sweep evaluates every active problem at its trial point with the
// start-packed kernels below; other layouts (any rank, both reflectivities)
// evaluate each problem with its bin's own FdF kernel (fdf_kernels.cu,
// returning at once for converged problems) and gatherEvalKernel.  Packed
// layouts:
//   fdfBatchKernel   -- persistent blocks walk a list of work items
//                       (bin, group of SG starts, range of 128-event tiles);
//                       each tile is loaded once by a bulk copy and used for all
//                       SG starts: phase 1 forms S_{s,e} = sum_w V_{s,w} A_{w,e},
//                       L = |S|^2 + V_flat^2, -ln L and c S (c = -2/L); phase 2
//                       G_{s,w} += sum_e c S_{s,e} conj(A_{w,e});
//                       per-thread FP32 (compensated for -ln L and c) over up
//                       to 8 tiles, then FP64; FP64 partials per item.
//                       Groups of 32 starts: two tile stages, one block per SM;
//   fdfBatch8Kernel  -- the same for groups of 8 starts (little work per
//                       tile): register-blocked phases over a quarter of the
//                       waves or events per thread, combined by shuffles; one
//                       stage, several blocks per SM taking turns;
//   batchFinishKernel -- one warp per problem: sums the items' partials in item
//                       order (deterministic), adds nEvt (Re V^H I^acc V +
//                       V_flat^2 eta) and the half-Cauchy prior in FP64
//                       (pwaLikelihood.cc:254-297) and writes f and the gradient;
//   lbfgsKernel      -- one warp per problem: backtracking line search
//                       (Armijo, or the approximate Wolfe conditions of Hager
//                       and Zhang near the rounding floor of f) and the L-BFGS
//                       two-loop recursion in FP64.
// The launches of one sweep are stream-ordered and capture into a CUDA graph;
// converged problems drop out (their items exit at once).

#include "pwa_internal.h"
#include "device_common.cuh"

#include <algorithm>

namespace pwa {
namespace {

constexpr int kBThreads = 256;
constexpr int kBE = 128;     // events per tile (the amplitude store's block)
constexpr int kBFold = 8;    // tiles summed in FP32 before the FP64 fold

struct BatchSmem {
	size_t stages, vs, ts, flat, bars, total;
};

__host__ __device__ inline BatchSmem batchSmem(int W, int SG, int NST)
{
	BatchSmem L{};
	auto up = [](size_t x) { return (x + 127) & ~size_t(127); };
	L.stages = 0;
	L.vs = up((size_t)NST * W * kBE * 8);
	L.ts = up(L.vs + (size_t)W * SG * 16);
	L.flat = up(L.ts + (size_t)2 * kBE * SG * 8);
	L.bars = up(L.flat + (size_t)SG * 4);
	L.total = L.bars + 2 * 8 + 128;
	return L;
}

// SG starts per group; phase 1: SPT starts x EPT events per thread;
// phase 2: SPT2 starts x WPT waves per thread (waves < 64).  NST tile stages
// per block: 2 (the next tile loads while this one is used) or 1 (MINB
// blocks per SM take turns instead).  Instantiated for groups of 32 starts
// (two stages, one block per SM); groups of 8 use fdfBatch8Kernel below.
template <int SG, int SPT, int EPT, int SPT2, int WPT, int NST, int MINB>
__global__ void __launch_bounds__(kBThreads, MINB) fdfBatchKernel(const BatchArgs a)
{
	static_assert(NST == 1 || NST == 2, "one or two tile stages");
	static_assert((SG / SPT) * (kBE / EPT) == kBThreads, "phase-1 mapping");
	static_assert((SG / SPT2) * (64 / WPT) == kBThreads, "phase-2 mapping");
	static_assert(EPT % 2 == 0 && SPT2 % 2 == 0 && SPT % 2 == 0, "paired loads");
	static_assert(SPT == SPT2, "both phases group the starts in the same quads");
	constexpr int NQ = SG / SPT;  // start groups of SPT (phase-1 sq, phase-2 sp)
	extern __shared__ __align__(128) unsigned char smem[];
	const int W = a.W, P = a.P;
	const BatchSmem lay = batchSmem(W, SG, NST);
	float2* stages = reinterpret_cast<float2*>(smem + lay.stages);  // [NST][W][kBE]
	// V of start s = q * SPT + i at [w][i][q] (vx, vx, vy, vy): a quarter-warp
	// (q = 0..7) reads 128 contiguous bytes
	float4* Vs = reinterpret_cast<float4*>(smem + lay.vs);
	// c S of the start pair (q * SPT + 2h, +1) of event e at 16-byte chunk
	// e * SG / 2 + h * NQ + q: again contiguous over q for both phases
	float2* Ts = reinterpret_cast<float2*>(smem + lay.ts);          // [2][kBE][SG]
	float* flat2 = reinterpret_cast<float*>(smem + lay.flat);       // [SG]
	uint64_t* bars = reinterpret_cast<uint64_t*>(smem + lay.bars);
	__shared__ double redLL[kBThreads / 32][SG], redC[kBThreads / 32][SG];

	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const uint32_t tileBytes = (uint32_t)W * kBE * 8u;
	// phase-1 role
	const int sq = tid % (SG / SPT), eq = tid / (SG / SPT);
	const int s1 = sq * SPT, e1 = eq * EPT;
	// phase-2 role
	const int sp = tid % (SG / SPT2), wg = tid / (SG / SPT2);
	const int s2 = sp * SPT2, w2 = wg * WPT;

	if (tid == 0) {
		mbarInit(&bars[0], 1);
		mbarInit(&bars[1], 1);
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	__syncthreads();
	uint32_t phase[2] = {0u, 0u};
	bool failed = false;

	for (int item = blockIdx.x; item < a.nItems && !failed; item += gridDim.x) {
		const BatchItem it = a.items[item];
		const BinDesc bin = a.bins[it.bin];
		const int q0 = bin.q0 + it.group * SG;
		const int ns = min(SG, bin.nStarts - it.group * SG);
		const int act = (tid < ns) ? a.active[q0 + tid] : 0;
		if (!__syncthreads_or(act))
			continue;
		// production amplitudes of the group's starts
		for (int k = tid; k < W * SG; k += kBThreads) {
			const int w = k / SG, s = k - w * SG;
			float vr = 0.f, vi = 0.f;
			if (s < ns) {
				const double* x = a.x + (size_t)(q0 + s) * P;
				const int ir = a.slotRe[w], ii = a.slotIm[w];
				vr = ir >= 0 ? (float)x[ir] : 0.f;
				vi = ii >= 0 ? (float)x[ii] : 0.f;
			}
			Vs[w * SG + (s % SPT) * NQ + s / SPT] = make_float4(vr, vr, vi, vi);
		}
		for (int s = tid; s < SG; s += kBThreads) {
			const double f = (s < ns) ? a.x[(size_t)(q0 + s) * P + P - 1] : 0.;
			flat2[s] = (float)(f * f);
		}
		const int nt = (int)(it.t1 - it.t0);
		const uint32_t ph0[2] = {phase[0], phase[1]};
		if (tid == 0) {
			fenceProxyAsync();
			for (int k = 0; k < NST && k < nt; ++k) {
				mbarArriveExpectTx(&bars[k], tileBytes);
				bulkCopyG2S(stages + (size_t)k * W * kBE, bin.amps + (size_t)(it.t0 + k) * W * kBE, tileBytes,
				            &bars[k]);
			}
		}
		__syncthreads();

		// accumulators
		double llD[SPT], csD[SPT];
		float llF[SPT], csF[SPT], llK[SPT], csK[SPT];  // compensated FP32 sums
#pragma unroll
		for (int i = 0; i < SPT; ++i) {
			llD[i] = csD[i] = 0.;
			llF[i] = csF[i] = llK[i] = csK[i] = 0.f;
		}
		double gD[SPT2][WPT][2];
		float2 Pp[SPT2][WPT], Qp[SPT2][WPT];
#pragma unroll
		for (int i = 0; i < SPT2; ++i)
#pragma unroll
			for (int j = 0; j < WPT; ++j) {
				gD[i][j][0] = gD[i][j][1] = 0.;
				Pp[i][j] = Qp[i][j] = make_float2(0.f, 0.f);
			}

		int k = 0;
		for (; k < nt; ++k) {
			const int st = (NST == 2) ? (k & 1) : 0;
			const bool ok = mbarWaitBounded(&bars[st], phase[st]);
			phase[st] ^= 1u;
			const float2* tile = stages + (size_t)st * W * kBE;
			const uint32_t tileAddr = smemAddr(tile);
			float2* T = Ts + (size_t)(k & 1) * kBE * SG;
			const uint64_t ev0 = (uint64_t)(it.t0 + k) * kBE;

			// ---- phase 1: S, L, -ln L, c S ----
			{
				float2 U[SPT][EPT], Z[SPT][EPT];
#pragma unroll
				for (int i = 0; i < SPT; ++i)
#pragma unroll
					for (int j = 0; j < EPT; ++j)
						U[i][j] = Z[i][j] = make_float2(0.f, 0.f);
				const uint32_t vAddr = smemAddr(Vs) + (uint32_t)sq * 16u;
				for (int w = 0; w < W; ++w) {
					const int pos = (e1 + (int)storeRot((uint32_t)w, kBE)) & (kBE - 1);
					float2 av[EPT];
#pragma unroll
					for (int j = 0; j < EPT; j += 2) {
						const float4 q = lds128(tileAddr + (uint32_t)(w * kBE + pos + j) * 8u);
						av[j] = make_float2(q.x, q.y);
						av[j + 1] = make_float2(q.z, q.w);
					}
#pragma unroll
					for (int i = 0; i < SPT; ++i) {
						const float4 v = lds128(vAddr + (uint32_t)(w * SG + i * NQ) * 16u);
						const float2 vx = make_float2(v.x, v.y), vy = make_float2(v.z, v.w);
#pragma unroll
						for (int j = 0; j < EPT; ++j) {
							U[i][j] = ffma2(av[j], vx, U[i][j]);
							Z[i][j] = ffma2(av[j], vy, Z[i][j]);
						}
					}
				}
#pragma unroll
				for (int j = 0; j < EPT; ++j) {
					const bool valid = ev0 + (uint64_t)(e1 + j) < bin.nEvents;
#pragma unroll
					for (int i = 0; i < SPT; i += 2) {
						float2 ts[2];
#pragma unroll
						for (int h = 0; h < 2; ++h) {
							const float sx = U[i + h][j].x - Z[i + h][j].y, sy = U[i + h][j].y + Z[i + h][j].x;
							const float L = fmaf(sx, sx, fmaf(sy, sy, flat2[s1 + i + h]));
							const float c = valid ? -2.f / L : 0.f;
							if (valid)
								kahanAdd(llF[i + h], llK[i + h], -logf(L));
							kahanAdd(csF[i + h], csK[i + h], c);
							ts[h] = make_float2(c * sx, c * sy);
						}
						*reinterpret_cast<float4*>(&T[2 * ((e1 + j) * (SG / 2) + (i / 2) * NQ + sq)]) =
						    make_float4(ts[0].x, ts[0].y, ts[1].x, ts[1].y);
					}
				}
			}
			// T complete; phase 2 of the previous tile is done by every thread
			if (__syncthreads_or(!ok)) {
				failed = true;
				break;
			}
			if (NST == 2 && tid == 0 && k >= 1 && k + 1 < nt) {
				fenceProxyAsync();
				const int ns2 = (k + 1) & 1;
				mbarArriveExpectTx(&bars[ns2], tileBytes);
				bulkCopyG2S(stages + (size_t)ns2 * W * kBE, bin.amps + (size_t)(it.t0 + k + 1) * W * kBE, tileBytes,
				            &bars[ns2]);
			}

			// ---- phase 2: G += sum_e c S conj(A) ----
			if (w2 < W) {
				const uint32_t tAddr = smemAddr(T) + (uint32_t)sp * 16u;
				int rot[WPT];
#pragma unroll
				for (int j = 0; j < WPT; ++j)
					rot[j] = (int)storeRot((uint32_t)(w2 + j), kBE);
				for (int e = 0; e < kBE; ++e) {
					float2 t[SPT2];
#pragma unroll
					for (int i = 0; i < SPT2; i += 2) {
						const float4 q = lds128(tAddr + (uint32_t)(e * (SG / 2) + (i / 2) * NQ) * 16u);
						t[i] = make_float2(q.x, q.y);
						t[i + 1] = make_float2(q.z, q.w);
					}
#pragma unroll
					for (int j = 0; j < WPT; ++j) {
						const int w = min(w2 + j, W - 1);
						const float2 av = lds64(tileAddr + (uint32_t)(w * kBE + ((e + rot[j]) & (kBE - 1))) * 8u);
						const float2 aw = make_float2(av.y, av.x);
#pragma unroll
						for (int i = 0; i < SPT2; ++i) {
							Pp[i][j] = ffma2(t[i], av, Pp[i][j]);  // (tx ax, ty ay)
							Qp[i][j] = ffma2(t[i], aw, Qp[i][j]);  // (tx ay, ty ax)
						}
					}
				}
			}
			// one stage: the next tile loads once every thread is done with this one
			if (NST == 1) {
				__syncthreads();
				if (tid == 0 && k + 1 < nt) {
					fenceProxyAsync();
					mbarArriveExpectTx(&bars[0], tileBytes);
					bulkCopyG2S(stages, bin.amps + (size_t)(it.t0 + k + 1) * W * kBE, tileBytes, &bars[0]);
				}
			}
			// fold the FP32 partials into FP64
			if ((k + 1) % kBFold == 0 || k + 1 == nt) {
#pragma unroll
				for (int i = 0; i < SPT; ++i) {
					llD[i] += (double)llF[i] - (double)llK[i];
					csD[i] += (double)csF[i] - (double)csK[i];
					llF[i] = csF[i] = llK[i] = csK[i] = 0.f;
				}
#pragma unroll
				for (int i = 0; i < SPT2; ++i)
#pragma unroll
					for (int j = 0; j < WPT; ++j) {
						gD[i][j][0] += (double)(Pp[i][j].x + Pp[i][j].y);
						gD[i][j][1] += (double)(Qp[i][j].y - Qp[i][j].x);
						Pp[i][j] = Qp[i][j] = make_float2(0.f, 0.f);
					}
			}
		}
		if (failed) {
			if (tid == 0) {
				atomicOr(a.devErr, (unsigned)kDevErrTimeout);
				// copies of this item still in flight land before the block
				// exits: with two stages tiles k .. max(1, k) were issued and
				// not consumed, with one stage tile k
				if (NST == 2) {
					for (int j = k; j <= max(1, k) && j < nt; ++j)
						mbarWaitBounded(&bars[j & 1], ph0[j & 1] ^ (uint32_t)((j >> 1) & 1));
				} else if (k < nt) {
					mbarWaitBounded(&bars[0], ph0[0] ^ (uint32_t)(k & 1));
				}
			}
			break;
		}

		// ---- partials of this item: [SG][2 + 2W] FP64 ----
		const int NV = 2 + 2 * W;
		double* out = a.partials + (size_t)item * SG * NV;
		// LL and sum c per start: lanes that share sq differ in eq
#pragma unroll
		for (int i = 0; i < SPT; ++i) {
			double l = llD[i], c = csD[i];
			for (int o = SG / SPT; o < 32; o <<= 1) {
				l += __shfl_xor_sync(0xffffffffu, l, o);
				c += __shfl_xor_sync(0xffffffffu, c, o);
			}
			if (lane < SG / SPT) {
				redLL[warp][s1 + i] = l;
				redC[warp][s1 + i] = c;
			}
		}
		if (w2 < W) {
#pragma unroll
			for (int i = 0; i < SPT2; ++i)
#pragma unroll
				for (int j = 0; j < WPT; ++j)
					if (w2 + j < W) {
						out[(size_t)(s2 + i) * NV + 2 + 2 * (w2 + j)] = gD[i][j][0];
						out[(size_t)(s2 + i) * NV + 3 + 2 * (w2 + j)] = gD[i][j][1];
					}
		}
		__syncthreads();
		for (int s = tid; s < SG; s += kBThreads) {
			double l = 0., c = 0.;
			for (int wv = 0; wv < kBThreads / 32; ++wv) {
				l += redLL[wv][s];
				c += redC[wv][s];
			}
			out[(size_t)s * NV] = l;
			out[(size_t)s * NV + 1] = c;
		}
		__syncthreads();
	}
}

// ---- start groups of 8: register-blocked phases ----
// With 8 starts a tile holds little work for 256 threads.  Mapped like the
// 32-start kernel (2 starts x 2 events per thread in phase 1, 2 starts x 1
// wave in phase 2) every complex product needs 12 bytes of shared-memory
// loads, and the shared-memory pipe bounds the kernel.  Here a thread forms
// 4 starts x 4 events over a quarter of the waves in phase 1 (6 bytes per
// product) and 4 starts x 2 waves over a quarter of the events in phase 2
// (6 bytes); the four lanes that split the same products combine them with a
// two-step shuffle reduce-scatter.  Partial sums are compensated FP32 over
// the item's tiles and FP64 per item, so the FP64 accumulators do not hold
// registers during the tile loop (three blocks per SM, 80 registers).
struct Batch8Smem {
	size_t stage, vs, ts, flat, bar, total;
};

__host__ __device__ inline Batch8Smem batch8Smem(int W)
{
	auto up = [](size_t x) { return (x + 127) & ~size_t(127); };
	Batch8Smem L{};
	L.stage = 0;
	L.vs = up((size_t)W * kBE * 8);
	L.ts = up(L.vs + (size_t)W * 8 * 16);
	L.flat = up(L.ts + (size_t)kBE * 8 * 8);
	L.bar = up(L.flat + 8 * 4);
	L.total = L.bar + 8 + 128;
	return L;
}

// V of start s at wave w: 16-byte slot w * 8 + ((s + 2 (w & 3)) & 7), holding
// (vx, vx, -vy, vy); c S of start s at event e: 8-byte slot
// e * 8 + 2 ((s / 2 + ((e >> 1) & 1)) & 3) + (s & 1).  With these skews the
// phase-1 V loads and the phase-2 c S loads of a quarter-warp hit distinct
// 16-byte bank groups (the tile's own rotation, storeRot, does the same for
// the amplitude loads).
__device__ __forceinline__ int b8VSlot(int w, int s) { return w * 8 + ((s + 2 * (w & 3)) & 7); }
__device__ __forceinline__ int b8TSlot(int e, int s) { return e * 8 + 2 * ((s / 2 + ((e >> 1) & 1)) & 3) + (s & 1); }

__global__ void __launch_bounds__(kBThreads, 3) fdfBatch8Kernel(const BatchArgs a)
{
	extern __shared__ __align__(128) unsigned char smem[];
	constexpr int SG = 8;
	const int W = a.W, P = a.P;
	const Batch8Smem lay = batch8Smem(W);
	float4* Vs = reinterpret_cast<float4*>(smem + lay.vs);
	float2* Ts = reinterpret_cast<float2*>(smem + lay.ts);
	float* flat2 = reinterpret_cast<float*>(smem + lay.flat);
	uint64_t* bar = reinterpret_cast<uint64_t*>(smem + lay.bar);
	__shared__ double redLL[kBThreads / 32][4], redC[kBThreads / 32][4];

	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const uint32_t tileBytes = (uint32_t)W * kBE * 8u;
	const uint32_t tileAddr = smemAddr(smem + lay.stage), vAddr = smemAddr(Vs), tAddr = smemAddr(Ts);
	// phase-1 role: waves w = kq (mod 4), events 4 eg .. 4 eg + 3, starts
	// 4 sq .. 4 sq + 3; after the reduce-scatter the lane holds starts
	// 4 sq + 2 b1 + {0, 1} of events eb + {0, 1}
	const int kq = lane & 3, b0 = kq & 1, b1 = kq >> 1;
	const int eg = (lane >> 2) | ((warp & 3) << 3), sq = warp >> 2;
	const int eb = 4 * eg + 2 * (b0 ^ (eg & 1));
	// the lane's rows all have rotation 4 kq; odd event groups load their
	// upper 16 bytes first, so that a quarter-warp covers all 32 banks
	const uint32_t col = (uint32_t)((4 * eg + 4 * kq) & (kBE - 1)) * 8u;
	const uint32_t c0 = col + 16u * (uint32_t)(eg & 1), c1 = col + 16u * (uint32_t)(1 - (eg & 1));
	const int vBase = 4 * sq + 2 * kq;  // V slot of start 4 sq + i: (vBase + i) & 7
	// phase-2 role: events 4 i + eq, starts 4 sg .. 4 sg + 3, waves 2 wp and
	// 2 wp + 1; after the reduce-scatter the lane holds starts
	// 4 sg + 2 (eq >> 1) + {0, 1} of wave 2 wp + (eq & 1)
	const int eq = lane & 3, sg = (lane >> 2) & 1, wp = (lane >> 3) | (warp << 2);
	const bool p2 = 2 * wp < W;
	const int wa = min(2 * wp, W - 1), wb = min(2 * wp + 1, W - 1);
	const int ra = (int)storeRot((uint32_t)wa, kBE), rb = (int)storeRot((uint32_t)wb, kBE);
	const uint32_t tq0 = (uint32_t)(2 * ((2 * sg + (eq >> 1)) & 3)) * 8u;      // starts 4 sg, +1
	const uint32_t tq1 = (uint32_t)(2 * ((2 * sg + 1 + (eq >> 1)) & 3)) * 8u;  // starts 4 sg + 2, +3

	if (tid == 0) {
		mbarInit(bar, 1);
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	__syncthreads();
	uint32_t phase = 0u;
	bool failed = false;

	for (int item = blockIdx.x; item < a.nItems && !failed; item += gridDim.x) {
		const BatchItem it = a.items[item];
		const BinDesc bin = a.bins[it.bin];
		const int q0 = bin.q0 + it.group * SG;
		const int ns = min(SG, bin.nStarts - it.group * SG);
		const int act = (tid < ns) ? a.active[q0 + tid] : 0;
		if (!__syncthreads_or(act))
			continue;
		for (int k = tid; k < W * SG; k += kBThreads) {
			const int w = k / SG, s = k - w * SG;
			float vr = 0.f, vi = 0.f;
			if (s < ns) {
				const double* x = a.x + (size_t)(q0 + s) * P;
				const int ir = a.slotRe[w], ii = a.slotIm[w];
				vr = ir >= 0 ? (float)x[ir] : 0.f;
				vi = ii >= 0 ? (float)x[ii] : 0.f;
			}
			Vs[b8VSlot(w, s)] = make_float4(vr, vr, -vi, vi);
		}
		if (tid < SG) {
			const double f = (tid < ns) ? a.x[(size_t)(q0 + tid) * P + P - 1] : 0.;
			flat2[tid] = (float)(f * f);
		}
		const int nt = (int)(it.t1 - it.t0);
		if (tid == 0 && nt > 0) {
			fenceProxyAsync();
			mbarArriveExpectTx(bar, tileBytes);
			bulkCopyG2S(smem + lay.stage, bin.amps + (size_t)it.t0 * W * kBE, tileBytes, bar);
		}
		__syncthreads();

		float llF[2], llK[2], csF[2], csK[2], gF[4], gK[4];
#pragma unroll
		for (int x = 0; x < 2; ++x)
			llF[x] = llK[x] = csF[x] = csK[x] = 0.f;
#pragma unroll
		for (int x = 0; x < 4; ++x)
			gF[x] = gK[x] = 0.f;

		int k = 0;
		for (; k < nt; ++k) {
			const bool ok = mbarWaitBounded(bar, phase);
			phase ^= 1u;
			const uint64_t ev0 = (uint64_t)(it.t0 + k) * kBE;

			// ---- phase 1: S = V A over the lane's waves, 4 starts x 4 events ----
			{
				float2 S[4][4];  // [start][event of the lane's order]
#pragma unroll
				for (int i = 0; i < 4; ++i)
#pragma unroll
					for (int j = 0; j < 4; ++j)
						S[i][j] = make_float2(0.f, 0.f);
#pragma unroll 1
				for (int w = kq; w < W; w += 4) {
					const uint32_t row = tileAddr + (uint32_t)w * (uint32_t)(kBE * 8);
					const float4 p0 = lds128(row + c0), p1 = lds128(row + c1);
					const float2 av[4] = {make_float2(p0.x, p0.y), make_float2(p0.z, p0.w), make_float2(p1.x, p1.y),
					                      make_float2(p1.z, p1.w)};
					const uint32_t vRow = vAddr + (uint32_t)w * 128u;
#pragma unroll
					for (int i = 0; i < 4; ++i) {
						const float4 v = lds128(vRow + (uint32_t)((vBase + i) & 7) * 16u);
						const float2 vx = make_float2(v.x, v.y), vy = make_float2(v.z, v.w);
						// (vx, vx) (ax, ay) + (-vy, vy) (ay, ax) = V A
#pragma unroll
						for (int j = 0; j < 4; ++j) {
							S[i][j] = ffma2(vx, av[j], S[i][j]);
							S[i][j] = ffma2(vy, make_float2(av[j].y, av[j].x), S[i][j]);
						}
					}
				}
				// reduce-scatter over the four wave slices: lane bit 2 keeps
				// starts 2 b1, 2 b1 + 1, lane bit 1 the events 2 b0, 2 b0 + 1
				float2 R1[2][4];
#pragma unroll
				for (int x = 0; x < 2; ++x)
#pragma unroll
					for (int j = 0; j < 4; ++j) {
						const float2 keep = b1 ? S[2 + x][j] : S[x][j];
						const float2 send = b1 ? S[x][j] : S[2 + x][j];
						R1[x][j] = make_float2(keep.x + __shfl_xor_sync(0xffffffffu, send.x, 2),
						                       keep.y + __shfl_xor_sync(0xffffffffu, send.y, 2));
					}
				float2 T[2][2];  // [start 4 sq + 2 b1 + x][event eb + y]
#pragma unroll
				for (int y = 0; y < 2; ++y) {
					const bool valid = ev0 + (uint64_t)(eb + y) < bin.nEvents;
#pragma unroll
					for (int x = 0; x < 2; ++x) {
						const float2 keep = b0 ? R1[x][2 + y] : R1[x][y];
						const float2 send = b0 ? R1[x][y] : R1[x][2 + y];
						const float sx = keep.x + __shfl_xor_sync(0xffffffffu, send.x, 1);
						const float sy = keep.y + __shfl_xor_sync(0xffffffffu, send.y, 1);
						const float L = fmaf(sx, sx, fmaf(sy, sy, flat2[4 * sq + 2 * b1 + x]));
						const float c = valid ? -2.f / L : 0.f;
						if (valid)
							kahanAdd(llF[x], llK[x], -logf(L));
						kahanAdd(csF[x], csK[x], c);
						T[x][y] = make_float2(c * sx, c * sy);
					}
				}
				// the two events' stores in an order that alternates with
				// the event group (halves the bank conflicts of the stores)
#pragma unroll
				for (int t = 0; t < 2; ++t) {
					const int y = (eg & 1) ^ t;
					*reinterpret_cast<float4*>(&Ts[b8TSlot(eb + y, 4 * sq + 2 * b1)]) =
					    make_float4(T[0][y].x, T[0][y].y, T[1][y].x, T[1][y].y);
				}
			}
			// c S complete
			if (__syncthreads_or(!ok)) {
				failed = true;
				break;
			}

			// ---- phase 2: G += sum_e c S conj(A), 4 starts x 2 waves over a quarter of the events ----
			{
				float2 Pp[4][2], Qp[4][2];
#pragma unroll
				for (int i = 0; i < 4; ++i)
#pragma unroll
					for (int j = 0; j < 2; ++j)
						Pp[i][j] = Qp[i][j] = make_float2(0.f, 0.f);
				if (p2) {
					const uint32_t rowA = tileAddr + (uint32_t)wa * (uint32_t)(kBE * 8);
					const uint32_t rowB = tileAddr + (uint32_t)wb * (uint32_t)(kBE * 8);
#pragma unroll 1
					for (int i = 0; i < kBE / 4; ++i) {
						const int e = 4 * i + eq;
						const uint32_t tRow = tAddr + (uint32_t)e * 64u;
						const float4 t01 = lds128(tRow + tq0), t23 = lds128(tRow + tq1);
						const float2 t[4] = {make_float2(t01.x, t01.y), make_float2(t01.z, t01.w),
						                     make_float2(t23.x, t23.y), make_float2(t23.z, t23.w)};
						const float2 xa = lds64(rowA + (uint32_t)((e + ra) & (kBE - 1)) * 8u);
						const float2 xb = lds64(rowB + (uint32_t)((e + rb) & (kBE - 1)) * 8u);
						const float2 xaS = make_float2(xa.y, xa.x), xbS = make_float2(xb.y, xb.x);
#pragma unroll
						for (int i4 = 0; i4 < 4; ++i4) {
							Pp[i4][0] = ffma2(t[i4], xa, Pp[i4][0]);  // (tx ax, ty ay)
							Qp[i4][0] = ffma2(t[i4], xaS, Qp[i4][0]);  // (tx ay, ty ax)
							Pp[i4][1] = ffma2(t[i4], xb, Pp[i4][1]);
							Qp[i4][1] = ffma2(t[i4], xbS, Qp[i4][1]);
						}
					}
				}
				// G = (P.x + P.y, Q.y - Q.x); reduce-scatter over the four
				// event residues: lane bit 2 keeps starts 2 (eq >> 1) + {0, 1},
				// lane bit 1 the wave 2 wp + (eq & 1)
				const int e1 = eq >> 1, e0 = eq & 1;
				float2 H[2][2];  // [start x][wave j]
#pragma unroll
				for (int x = 0; x < 2; ++x)
#pragma unroll
					for (int j = 0; j < 2; ++j) {
						const int ik = e1 ? 2 + x : x, is = e1 ? x : 2 + x;
						const float2 keep = make_float2(Pp[ik][j].x + Pp[ik][j].y, Qp[ik][j].y - Qp[ik][j].x);
						const float2 send = make_float2(Pp[is][j].x + Pp[is][j].y, Qp[is][j].y - Qp[is][j].x);
						H[x][j] = make_float2(keep.x + __shfl_xor_sync(0xffffffffu, send.x, 2),
						                      keep.y + __shfl_xor_sync(0xffffffffu, send.y, 2));
					}
#pragma unroll
				for (int x = 0; x < 2; ++x) {
					const float2 keep = e0 ? H[x][1] : H[x][0];
					const float2 send = e0 ? H[x][0] : H[x][1];
					kahanAdd(gF[2 * x], gK[2 * x], keep.x + __shfl_xor_sync(0xffffffffu, send.x, 1));
					kahanAdd(gF[2 * x + 1], gK[2 * x + 1], keep.y + __shfl_xor_sync(0xffffffffu, send.y, 1));
				}
			}
			// the next tile loads once every thread is done with this one
			__syncthreads();
			if (tid == 0 && k + 1 < nt) {
				fenceProxyAsync();
				mbarArriveExpectTx(bar, tileBytes);
				bulkCopyG2S(smem + lay.stage, bin.amps + (size_t)(it.t0 + k + 1) * W * kBE, tileBytes, bar);
			}
		}
		if (failed) {
			// the copy of tile k (the one whose wait expired) lands before
			// the block exits
			if (tid == 0) {
				atomicOr(a.devErr, (unsigned)kDevErrTimeout);
				mbarWaitBounded(bar, phase ^ 1u);
			}
			break;
		}

		// ---- partials of this item: [SG][2 + 2W] FP64 ----
		const int NV = 2 + 2 * W;
		double* out = a.partials + (size_t)item * SG * NV;
		// -ln L and sum c: the lanes with equal b1 hold the same starts
#pragma unroll
		for (int x = 0; x < 2; ++x) {
			double l = (double)llF[x] - (double)llK[x], c = (double)csF[x] - (double)csK[x];
#pragma unroll
			for (int o = 1; o < 32; o <<= 1) {
				if (o == 2)
					continue;
				l += __shfl_xor_sync(0xffffffffu, l, o);
				c += __shfl_xor_sync(0xffffffffu, c, o);
			}
			if ((lane & ~2) == 0) {
				redLL[warp][2 * b1 + x] = l;
				redC[warp][2 * b1 + x] = c;
			}
		}
		{
			const int w = 2 * wp + (eq & 1);
			if (w < W) {
#pragma unroll
				for (int x = 0; x < 2; ++x) {
					const int s = 4 * sg + 2 * (eq >> 1) + x;
					out[(size_t)s * NV + 2 + 2 * w] = (double)gF[2 * x] - (double)gK[2 * x];
					out[(size_t)s * NV + 3 + 2 * w] = (double)gF[2 * x + 1] - (double)gK[2 * x + 1];
				}
			}
		}
		__syncthreads();
		if (tid < SG) {
			// warps 4 (s / 4) .. 4 (s / 4) + 3 hold start s, in a fixed order
			double l = 0., c = 0.;
			for (int wv = 4 * (tid >> 2); wv < 4 * (tid >> 2) + 4; ++wv) {
				l += redLL[wv][tid & 3];
				c += redC[wv][tid & 3];
			}
			out[(size_t)tid * NV] = l;
			out[(size_t)tid * NV + 1] = c;
		}
		__syncthreads();
	}
}

__device__ __forceinline__ double warpAllSum(double v)
{
#pragma unroll
	for (int o = 16; o > 0; o >>= 1)
		v += __shfl_xor_sync(0xffffffffu, v, o);
	return v;
}

// One warp per problem: f and gradient from the items' partials plus the
// normalisation and prior terms.
__global__ void batchFinishKernel(const FinishBatchArgs a)
{
	const int q = (int)((blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5);
	const int lane = threadIdx.x & 31;
	if (q >= a.Q || !a.active[q])
		return;
	const int W = a.W, P = a.P, NV = 2 + 2 * W;
	const ProblemDesc pd = a.problems[q];
	const BinDesc bin = a.bins[pd.bin];
	const double* x = a.x + (size_t)q * P;
	double* g = a.g + (size_t)q * P;
	const double nEvt = bin.nEvt, twice = 2. * bin.nEvt;
	const double flat = x[P - 1];
	// event sums, in item order
	double fLL = 0., fC = 0.;
	for (int v = lane; v < NV; v += 32) {
		double acc = 0.;
		for (int i = pd.item0; i < pd.item1; ++i)
			acc += a.partials[((size_t)i * a.SG + pd.slot) * NV + v];
		if (v == 0)
			fLL = acc;
		else if (v == 1)
			fC = acc;
		else {
			const int w = (v - 2) >> 1, comp = (v - 2) & 1;
			const int idx = comp ? a.slotIm[w] : a.slotRe[w];
			if (idx >= 0)
				g[idx] = acc;
		}
	}
	fLL = __shfl_sync(0xffffffffu, fLL, 0);
	fC = __shfl_sync(0xffffffffu, fC, 1);
	__syncwarp();
	// normalisation: D_i = sum_j V_j conj(I_ij); prior
	double norm = 0., prior = 0.;
	const double g2 = a.cauchyWidth * a.cauchyWidth;
	for (int i = lane; i < W; i += 32) {
		const int ri = a.slotRe[i], ii = a.slotIm[i];
		const double vr = ri >= 0 ? x[ri] : 0., vi = ii >= 0 ? x[ii] : 0.;
		double dre = 0., dim = 0.;
		const double* Ib = bin.accI + (size_t)2 * i * W;
		for (int j = 0; j < W; ++j) {
			const int rj = a.slotRe[j], ij = a.slotIm[j];
			const double ur = rj >= 0 ? x[rj] : 0., ui = ij >= 0 ? x[ij] : 0.;
			const double Ir = Ib[2 * j], Ii = Ib[2 * j + 1];
			dre += ur * Ir + ui * Ii;
			dim += ui * Ir - ur * Ii;
		}
		norm += vr * dre + vi * dim;
		double pre = 0., pim = 0.;
		if (a.prior == 1) {
			const double rr = hypot(vr, vi);
			const double cf = 1. / (1. + (rr * rr) / g2);
			const double cd = (-2. * rr * g2) / ((g2 + rr * rr) * (g2 + rr * rr));
			const double fac = (1. / (rr * cf)) * cd;
			prior += -log(cf);
			pre = fac * vr;
			pim = fac * vi;
		}
		if (ri >= 0)
			g[ri] += twice * dre - pre;
		if (ii >= 0)
			g[ii] += twice * dim - pim;
	}
	norm = warpAllSum(norm);
	prior = warpAllSum(prior);
	if (lane == 0) {
		a.f[q] = fLL + nEvt * (norm + flat * flat * bin.totAcc) + prior;
		g[P - 1] = flat * fC + twice * flat * bin.totAcc;
	}
	// parameters the layout holds fixed do not move: their gradient
	// components are 0 to the minimiser (the reference strips them,
	// highLevelInterface/pwaNloptFit.cc:383-401)
	__syncwarp();
	const unsigned char* fx = a.fixed + (size_t)pd.bin * P;
	for (int i = lane; i < P; i += 32)
		if (fx[i])
			g[i] = 0.;
}

// General-layout batches: problem q's FdF launch wrote [f, gradient, device
// status] to out[q]; copy f and the gradient (fixed components 0) into the
// L-BFGS buffers.  One warp per problem.
__global__ void gatherEvalKernel(const GatherEvalArgs a)
{
	const int q = (int)((blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5);
	const int lane = threadIdx.x & 31;
	if (q >= a.Q || !a.active[q])
		return;
	const int P = a.P;
	const double* o = a.out + (size_t)q * (P + 2);
	const unsigned char* fx = a.fixed + (size_t)a.problems[q].bin * P;
	double* g = a.g + (size_t)q * P;
	for (int i = lane; i < P; i += 32)
		g[i] = fx[i] ? 0. : o[1 + i];
	if (lane == 0) {
		a.f[q] = o[0];
		if (o[P + 1] != 0.)
			atomicOr(a.devErr, (unsigned)o[P + 1]);
	}
}

// ---------------------------------------------------------------------------
// batched L-BFGS (one warp per problem, FP64)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double wdot(const double* a, const double* b, int n, int lane)
{
	double s = 0.;
	for (int i = lane; i < n; i += 32)
		s += a[i] * b[i];
	return warpAllSum(s);
}

__global__ void lbfgsKernel(const LbfgsArgs a)
{
	const int q = (int)((blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5);
	const int lane = threadIdx.x & 31;
	if (q >= a.Q)
		return;
	const int st = a.status[q];
	if (st != kLbfgsInit && st != kLbfgsSearch)
		return;
	const int P = a.P, m = a.m;
	double* x = a.x + (size_t)q * P;    // accepted point
	double* g = a.g + (size_t)q * P;
	double* d = a.d + (size_t)q * P;
	double* xt = a.xt + (size_t)q * P;  // trial point (evaluated in this sweep)
	const double* gt = a.gt + (size_t)q * P;
	double* S = a.S + (size_t)q * m * P;
	double* Y = a.Y + (size_t)q * m * P;
	double* rho = a.rho + (size_t)q * m;
	double* alph = a.alphaBuf + (size_t)q * m;
	const double ft = a.ft[q];
	bool accept = false;
	if (st == kLbfgsInit) {
		accept = isfinite(ft);
		if (!accept) {
			if (lane == 0)
				a.status[q] = kLbfgsFailed;
			return;
		}
	} else {
		// sufficient decrease (Armijo), or the approximate Wolfe conditions of
		// Hager and Zhang (value within a relative 1e-8 of f, directional
		// derivative between 0.9 g.d and -0.8 g.d), which stay decisive when
		// the decrease is below the rounding noise of f near a minimum
		const double gd = wdot(g, d, P, lane);
		const double gtd = wdot(gt, d, P, lane);
		const double f0 = a.f[q];
		const bool armijo = ft <= f0 + 1e-4 * a.step[q] * gd;
		const bool approxWolfe = ft <= f0 + 1e-8 * fmax(1., fabs(f0)) && gtd >= 0.9 * gd && gtd <= -0.8 * gd;
		accept = isfinite(ft) && (armijo || approxWolfe);
	}
	if (!accept) {
		// backtrack
		const int nb = a.nBack[q] + 1;
		const double step = a.step[q] * 0.5;
		if (nb > 40) {
			if (a.hist[q] > 0) {
				// restart once from steepest descent at the accepted point
				const double gn = sqrt(wdot(g, g, P, lane));
				for (int i = lane; i < P; i += 32) {
					d[i] = -g[i] / fmax(gn, 1e-300);
					xt[i] = x[i] + d[i];
				}
				if (lane == 0) {
					a.hist[q] = 0;
					a.head[q] = 0;
					a.nBack[q] = 0;
					a.step[q] = 1.;
				}
				return;
			}
			if (lane == 0)
				a.status[q] = kLbfgsStalled;
			return;
		}
		for (int i = lane; i < P; i += 32)
			xt[i] = x[i] + step * d[i];
		if (lane == 0) {
			a.nBack[q] = nb;
			a.step[q] = step;
		}
		return;
	}
	// accept the trial point: update the history with s = xt - x, y = gt - g
	int hist = a.hist[q], head = a.head[q];
	if (st == kLbfgsSearch) {
		double sy = 0., yy = 0., ss = 0.;
		for (int i = lane; i < P; i += 32) {
			const double si = xt[i] - x[i], yi = gt[i] - g[i];
			sy += si * yi;
			yy += yi * yi;
			ss += si * si;
		}
		sy = warpAllSum(sy);
		yy = warpAllSum(yy);
		ss = warpAllSum(ss);
		if (sy > 1e-12 * sqrt(ss * yy)) {
			const int slot = (head + hist) % m;
			for (int i = lane; i < P; i += 32) {
				S[(size_t)slot * P + i] = xt[i] - x[i];
				Y[(size_t)slot * P + i] = gt[i] - g[i];
			}
			if (lane == 0) {
				rho[slot] = 1. / sy;
				a.gamma[q] = sy / yy;
			}
			if (hist < m)
				++hist;
			else
				head = (head + 1) % m;
		}
	}
	__syncwarp();
	for (int i = lane; i < P; i += 32) {
		x[i] = xt[i];
		g[i] = gt[i];
	}
	__syncwarp();
	const double fNew = ft;
	const double gnorm = sqrt(wdot(g, g, P, lane));
	const int iter = a.iter[q] + (st == kLbfgsSearch ? 1 : 0);
	if (lane == 0) {
		a.f[q] = fNew;
		a.gnorm[q] = gnorm;
		a.iter[q] = iter;
		a.hist[q] = hist;
		a.head[q] = head;
	}
	if (gnorm <= a.gtolAbs + a.gtolRel * fmax(1., fabs(fNew))) {
		if (lane == 0)
			a.status[q] = kLbfgsConverged;
		return;
	}
	// rounding floor: the gradient norm has not improved by 1% for
	// floorWindow iterations (FP32 contractions bound how small it gets)
	if (a.floorWindow > 0) {
		if (st == kLbfgsInit || gnorm < 0.99 * a.gBest[q]) {
			if (lane == 0) {
				a.gBest[q] = gnorm;
				a.itBest[q] = iter;
			}
		} else if (iter - a.itBest[q] >= a.floorWindow) {
			if (lane == 0)
				a.status[q] = kLbfgsFloor;
			return;
		}
	}
	if (iter >= a.maxIter) {
		if (lane == 0)
			a.status[q] = kLbfgsMaxIter;
		return;
	}
	// two-loop recursion: d = -H g
	for (int i = lane; i < P; i += 32)
		d[i] = -g[i];
	__syncwarp();
	for (int k = hist - 1; k >= 0; --k) {
		const int slot = (head + k) % m;
		const double al = rho[slot] * wdot(S + (size_t)slot * P, d, P, lane);
		if (lane == 0)
			alph[k] = al;
		for (int i = lane; i < P; i += 32)
			d[i] -= al * Y[(size_t)slot * P + i];
		__syncwarp();
	}
	const double gamma = hist > 0 ? a.gamma[q] : 1. / fmax(gnorm, 1e-300);
	for (int i = lane; i < P; i += 32)
		d[i] *= gamma;
	__syncwarp();
	for (int k = 0; k < hist; ++k) {
		const int slot = (head + k) % m;
		const double be = rho[slot] * wdot(Y + (size_t)slot * P, d, P, lane);
		const double al = __shfl_sync(0xffffffffu, lane == 0 ? alph[k] : 0., 0);
		for (int i = lane; i < P; i += 32)
			d[i] += (al - be) * S[(size_t)slot * P + i];
		__syncwarp();
	}
	const double gd = wdot(g, d, P, lane);
	if (!(gd < 0.)) {
		// not a descent direction: restart from steepest descent
		for (int i = lane; i < P; i += 32)
			d[i] = -g[i] / fmax(gnorm, 1e-300);
		if (lane == 0) {
			a.hist[q] = 0;
			a.head[q] = 0;
		}
		__syncwarp();
	}
	for (int i = lane; i < P; i += 32)
		xt[i] = x[i] + d[i];
	if (lane == 0) {
		a.step[q] = 1.;
		a.nBack[q] = 0;
		a.status[q] = kLbfgsSearch;
	}
}

__global__ void countActiveKernel(const int* status, int Q, int* active, unsigned* nActive)
{
	for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < Q; q += gridDim.x * blockDim.x) {
		const int a = (status[q] == kLbfgsInit || status[q] == kLbfgsSearch) ? 1 : 0;
		active[q] = a;
		if (a)
			atomicAdd(nActive, 1u);
	}
}

template <int SG, int SPT, int EPT, int SPT2, int WPT, int NST, int MINB>
int configureBatchT(int W)
{
	const BatchSmem lay = batchSmem(W, SG, NST);
	return cudaCheck(cudaFuncSetAttribute(fdfBatchKernel<SG, SPT, EPT, SPT2, WPT, NST, MINB>,
	                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lay.total),
	                 "batch smem attribute");
}

// persistent grid: numSMs x the blocks of this variant that fit on an SM
template <int SG, int SPT, int EPT, int SPT2, int WPT, int NST, int MINB>
int launchBatchT(const BatchArgs& a, int numSMs, cudaStream_t s)
{
	auto kern = fdfBatchKernel<SG, SPT, EPT, SPT2, WPT, NST, MINB>;
	const BatchSmem lay = batchSmem(a.W, SG, NST);
	int perSM = 1;
	if (NST == 1) {
		const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kern, kBThreads, lay.total);
		if (e != cudaSuccess)
			return cudaCheck(e, "batch FdF occupancy");
		perSM = std::max(1, std::min(perSM, MINB));
	}
	kern<<<numSMs * perSM, kBThreads, lay.total, s>>>(a);
	countLaunches(1);
	return cudaCheck(cudaGetLastError(), "batch FdF launch");
}

// persistent grid: numSMs x the blocks that fit on an SM (at most three)
int launchBatch8(const BatchArgs& a, int numSMs, cudaStream_t s)
{
	const size_t smemBytes = batch8Smem(a.W).total;
	int perSM = 1;
	const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, fdfBatch8Kernel, kBThreads, smemBytes);
	if (e != cudaSuccess)
		return cudaCheck(e, "batch FdF occupancy");
	perSM = std::max(1, std::min(perSM, 3));
	fdfBatch8Kernel<<<numSMs * perSM, kBThreads, smemBytes, s>>>(a);
	countLaunches(1);
	return cudaCheck(cudaGetLastError(), "batch FdF launch");
}

}  // namespace

size_t batchSmemBytes(int W, int SG) { return SG == 8 ? batch8Smem(W).total : batchSmem(W, SG, 2).total; }

// start groups of 32: two stages, one block per SM; of 8: the
// register-blocked kernel, one stage, up to three blocks per SM
int configureBatchFdf(int W, int SG, size_t maxSmem)
{
	if (W < 1 || W > 64)
		return setError(kErrUnsupported, "batched FdF supports 1..64 waves");
	if (batchSmemBytes(W, SG) > maxSmem)
		return setError(kErrUnsupported, "batched FdF: shared memory too small for this wave set");
	if (SG == 32)
		return configureBatchT<32, 4, 4, 4, 2, 2, 1>(W);
	if (SG == 8)
		return cudaCheck(cudaFuncSetAttribute(fdfBatch8Kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
		                                      (int)batch8Smem(W).total),
		                 "batch smem attribute");
	return setError(kErrUnsupported, "batched FdF: start-group size must be 8 or 32");
}

int launchBatchFdf(const BatchArgs& a, int numSMs, cudaStream_t s)
{
	if (a.W < 1 || a.W > 64)
		return setError(kErrUnsupported, "batched FdF supports 1..64 waves");
	if (a.SG == 32)
		return launchBatchT<32, 4, 4, 4, 2, 2, 1>(a, numSMs, s);
	if (a.SG == 8)
		return launchBatch8(a, numSMs, s);
	return setError(kErrUnsupported, "batched FdF: start-group size must be 8 or 32");
}

int launchBatchFinish(const FinishBatchArgs& a, cudaStream_t s)
{
	const int threads = 256;
	const int blocks = (int)((a.Q * 32ull + threads - 1) / threads);
	batchFinishKernel<<<std::max(blocks, 1), threads, 0, s>>>(a);
	countLaunches(1);
	return cudaCheck(cudaGetLastError(), "batch finish launch");
}

int launchGatherEval(const GatherEvalArgs& a, cudaStream_t s)
{
	const int threads = 256;
	const int blocks = (int)((a.Q * 32ull + threads - 1) / threads);
	gatherEvalKernel<<<std::max(blocks, 1), threads, 0, s>>>(a);
	countLaunches(1);
	return cudaCheck(cudaGetLastError(), "gather launch");
}

int launchLbfgs(const LbfgsArgs& a, cudaStream_t s)
{
	const int threads = 256;
	const int blocks = (int)((a.Q * 32ull + threads - 1) / threads);
	lbfgsKernel<<<std::max(blocks, 1), threads, 0, s>>>(a);
	countLaunches(1);
	return cudaCheck(cudaGetLastError(), "L-BFGS launch");
}

int launchCountActive(const int* status, int Q, int* active, unsigned* nActive, cudaStream_t s)
{
	PWA_CHECK(cudaCheck(cudaMemsetAsync(nActive, 0, sizeof(unsigned), s), "memset"));
	const int threads = 256;
	const int blocks = std::min(1024, std::max(1, (Q + threads - 1) / threads));
	countActiveKernel<<<blocks, threads, 0, s>>>(status, Q, active, nActive);
	countLaunches(1);
	return cudaCheck(cudaGetLastError(), "count launch");
}

}  // namespace pwa
