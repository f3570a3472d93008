// fdf_kernels.cu -- fused extended-likelihood value + gradient for sm_103a.
//
// One pass over the complex64 amplitude store computes, for every data event i,
//   S_{r,e,i} = sum_{w in e} V_{r,w} A_{w,i}            (coherent sum, FP32)
//   L_i       = sum_{r,e} |S_{r,e,i}|^2 + V_flat^2
//   c_i       = -2 / L_i
//   G_{r,w}  += c_i S_{r,e(w),i} conj(A_{w,i})          (FP32 per tile, FP64 across tiles)
// plus -sum ln L_i and sum c_i, which is the event term of
// partialWaveFit/pwaLikelihood.cc:209-244 (FdF), :361-375 (DoEval) and
// :547-577 (Gradient).  The same kernel adds the normalisation term
// (:254-273) and the half-Cauchy prior (:278-297) in FP64, sums the blocks'
// partials in FP64 and writes f and the gradient in the parameter layout
// (:1714-1731): one launch per evaluation.
//
// Kernel structure (one persistent CTA per SM, 512 threads):
//   * the store keeps each block of E events contiguous (storeIndex), so one
//     cp.async.bulk copy moves a tile into shared memory, completing on an
//     mbarrier; `stages` tiles are in flight;
//   * after its event loop every CTA computes the normalisation and prior
//     terms of a few slots in FP64;
//   * phase 1: each warp owns E/16 events of the tile, 32/(E/16) lanes per
//     event sum interleaved slices of the waves and combine them with warp
//     shuffles, giving L_i, c_i and T_{r,e,i} = c_i S (double-buffered, so
//     one block barrier per tile suffices).  Variant NE = 2 gives each lane
//     two adjacent events (one 128-bit amplitude load and one V load per
//     wave serve both; 17 % fewer shared-memory wavefronts per tile);
//   * phase 2: warp j owns a contiguous range of waves of one reflectivity,
//     each lane a fixed set of event pairs; the lane sums conj(A) T over its
//     events with packed FP32x2 FMA for kFold tiles, then a warp
//     reduce-scatter leaves every lane one (slot, re/im) value, which it adds
//     to its FP64 (or compensated FP32) accumulator;
//   * the last warp to finish with a stage (shared-memory counter) refills it
//     with the tile `stages` ahead;
//   * the CTAs' partials are summed exactly in 128-bit fixed point with
//     integer atomics (order-independent, so results are bitwise
//     reproducible); the last CTA to arrive writes f and the gradient.
// Every mbarrier wait is bounded (about a second); on expiry the CTA sets a
// device error flag, waits (again bounded) for its own copies and completes
// the tail, and the host discards the result.

#include "pwa_internal.h"
#include "device_common.cuh"
#include "fdf_common.cuh"

#include <algorithm>

namespace pwa {
namespace {


// Shared-memory layout of the main kernel (byte offsets from the dynamic base).
// A stage holds one store block: W rows of E complex64 amplitudes, in the
// store's rotated order (storeIndex), moved by a single bulk copy.
struct SmemLayout {
	size_t rowStride;  // bytes per wave row
	size_t tiles, vs, v64, ts, bars, done, total;
};

__host__ __device__ inline SmemLayout smemLayout(int W, int R, int E, int stages)
{
	auto up = [](size_t x) { return (x + 127) & ~(size_t)127; };
	SmemLayout L;
	L.rowStride = (size_t)E * 8;
	L.tiles = 0;
	L.vs = up((size_t)stages * W * L.rowStride);
	L.v64 = up(L.vs + (size_t)W * R * 8);
	L.ts = up(L.v64 + (size_t)W * R * 16);
	L.bars = up(L.ts + 2 * (size_t)R * 2 * E * 8);
	L.done = L.bars + (size_t)stages * 8;
	L.total = L.done + (size_t)stages * 4;
	return L;
}

// Phase-2 wave ownership: nNeg warps share the W0 negative-reflectivity
// waves (wn each), the other warps the positive ones (wp each), so that every
// warp works on one reflectivity only; returns the largest per-warp count.
__host__ __device__ inline int waveSplit(int W0, int W, int* nNeg, int* wn, int* wp)
{
	const int W1 = W - W0;
	int best = 1 << 30, bn = 0;
	if (W0 == 0 || W1 == 0) {
		bn = (W0 == 0) ? 0 : kWarps;
		best = (W0 == 0) ? (W1 + kWarps - 1) / kWarps : (W0 + kWarps - 1) / kWarps;
	} else {
		for (int n = 1; n < kWarps; ++n) {
			const int m = max((W0 + n - 1) / n, (W1 + kWarps - n - 1) / (kWarps - n));
			if (m < best) {
				best = m;
				bn = n;
			}
		}
	}
	*nNeg = bn;
	*wn = bn ? (W0 + bn - 1) / bn : 0;
	*wp = (bn < kWarps) ? (W1 + kWarps - bn - 1) / (kWarps - bn) : 0;
	return best;
}

// Tiles whose gradient partials are summed in FP32 before the warp
// reduce-scatter folds them into the FP64 accumulators (a lane's FP32
// partial then covers 256 events of one wave; the LL and gradient errors
// against FP64 at 1 M events are the same as with 8).  The compensated mode
// folds every tile; the plain FP32 mode only after the last one.
constexpr int kFold = 64;
__device__ __forceinline__ int foldTiles(int reduction) { return reduction == 0 ? kFold : reduction == 1 ? 1 : 1 << 30; }


template <int R, int E, int WPW, int NE>
__global__ void __launch_bounds__(kThreads, 1) fdfMainKernel(const FdfArgs a, const int stages)
{
	extern __shared__ __align__(128) unsigned char smem[];
	constexpr int EPW = E / kWarps;          // events per warp in phase 1
	constexpr int H = 32 / EPW;              // lanes (wave slices) per event
	constexpr int NV = WPW * R * 2;          // phase-2 values per lane
	constexpr int NQ = (NV + 31) / 32;       // rounds of 32
	constexpr int NVP = NQ * 32;
	constexpr int EPAIRS = E / 64;           // event pairs per lane per tile
	static_assert(EPW * kWarps == E && H * EPW == 32 && H == 512 / E, "tile shape");

	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const int W = a.W, W0 = a.W0;
	const SmemLayout lay = smemLayout(W, R, E, stages);
	float2* tiles = reinterpret_cast<float2*>(smem + lay.tiles);
	float2* Vs = reinterpret_cast<float2*>(smem + lay.vs);      // [W][R] (vx, vy)
	double2* V64 = reinterpret_cast<double2*>(smem + lay.v64);  // [R][W] FP64, slot order
	float2* Ts = reinterpret_cast<float2*>(smem + lay.ts);      // [2][R][2][E] c S
	uint64_t* bars = reinterpret_cast<uint64_t*>(smem + lay.bars);
	unsigned* done = reinterpret_cast<unsigned*>(smem + lay.done);

	const uint64_t nTiles = (a.nEvents + E - 1) / E;
	const uint64_t first = blockIdx.x, stride = gridDim.x;
	const uint64_t myTiles = (first < nTiles) ? (nTiles - 1 - first) / stride + 1 : 0;
	const uint32_t stageBytes = (uint32_t)W * E * 8u;

	// batched fits: the launch of a problem that no longer iterates does
	// nothing (the flag is written by the preceding grid; uniform over the grid)
	if (a.active) {
		gridDependencyWait();
		if (*(const volatile int*)a.active == 0)
			return;
	}

	if (tid == 0) {
		for (int s = 0; s < stages; ++s) {
			mbarInit(&bars[s], 1);
			done[s] = 0u;
		}
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	__syncthreads();

	// issue store block (tile) k (local index) into stage s: one bulk copy
	auto issue = [&](uint64_t k, int s) {
		if (lane == 0) {
			const float2* src = a.amps + (first + k * stride) * (uint64_t)W * E;
			mbarArriveExpectTx(&bars[s], stageBytes);
			bulkCopyG2S(tiles + (size_t)s * W * E, src, stageBytes, &bars[s]);
		}
	};
	// the amplitude store does not change after finishInit (which
	// synchronises), so the first stages load while the preceding grid ends
	if (warp == 0) {
		for (int s = 0; s < stages && (uint64_t)s < myTiles; ++s)
			issue((uint64_t)s, s);
	}

	// the parameters may be written by the preceding grid (device-side minimiser)
	gridDependencyWait();
	gridDependencyTrigger();
	for (int k = tid; k < W * R; k += kThreads) {
		const int w = k / R, r = k - w * R;
		const int ir = a.slotRe[r * W + w], ii = a.slotIm[r * W + w];
		const double vr = ir >= 0 ? a.par[ir] : 0., vi = ii >= 0 ? a.par[ii] : 0.;
		Vs[k] = make_float2((float)vr, (float)vi);
		V64[r * W + w] = make_double2(vr, vi);
	}
	const double flatD = a.par[a.P - 1];
	const float flat2 = (float)(flatD * flatD);
	__syncthreads();

	// phase-1 role: event pe of the tile, wave slice ph (waves w = ph mod H)
	const int pm = lane / H, ph = lane - pm * H;
	const int pe = warp * EPW + pm;
	const int wStart1 = W0 + (((ph - W0) % H) + H) % H;  // first positive-reflectivity wave of this slice
	// phase-2 role: the warp owns waves [wBase, wBase + nWarpWaves) of reflectivity wRefl
	int nNegWarps, wn, wp;
	waveSplit(W0, W, &nNegWarps, &wn, &wp);
	const int wRefl = (warp < nNegWarps) ? 0 : 1;
	const int wBase = wRefl == 0 ? warp * wn : W0 + (warp - nNegWarps) * wp;
	const int wEnd = wRefl == 0 ? min(W0, wBase + wn) : min(W, wBase + wp);
	const int nWarpWaves = max(0, wEnd - wBase);
	// tile-invariant phase-2 addresses: byte offset of this lane's first event
	// pair in row wBase + wi of a stage (the second pair, 64 events on, is at
	// offset ^ 512: adding 64 modulo 128 flips one bit of the position), and
	// of its first pair in the T buffers
	static_assert(EPAIRS == 1 || (EPAIRS == 2 && E == 128), "phase-2 event pairs");
	uint32_t aOff[WPW];
#pragma unroll
	for (int wi = 0; wi < WPW; ++wi) {
		const int w = min(wBase + wi, W - 1);
		aOff[wi] = (uint32_t)(w * E + ((2 * lane + (int)storeRot((uint32_t)w, (uint32_t)E)) & (E - 1))) * 8u;
	}
	const uint32_t tOff = (uint32_t)(wRefl * E + 2 * lane) * 8u;

	double accLL = 0., accC = 0.;
	float kLL = 0.f, kLLc = 0.f, kC = 0.f, kCc = 0.f;
	float llPart = 0.f, cPart = 0.f;
	double accG[NQ];
	float kG[NQ], kGc[NQ];
#pragma unroll
	for (int q = 0; q < NQ; ++q) {
		accG[q] = 0.;
		kG[q] = 0.f;
		kGc[q] = 0.f;
	}
	// P = sum a (.) t, Q = sum a (.) t_swapped  ->  G = (P.x + P.y, Q.x - Q.y)
	// ranks 1-2: packed sums as above; ranks 3-4 keep (Gx, Gy) in Pp alone
	// (half the accumulator registers, twice the FMA instructions), which
	// keeps their larger accumulator sets out of local memory
	constexpr bool kPacked = R <= 2;
	float2 Pp[WPW][R], Qp[WPW][R];
#pragma unroll
	for (int wi = 0; wi < WPW; ++wi)
#pragma unroll
		for (int r = 0; r < R; ++r) {
			Pp[wi][r] = make_float2(0.f, 0.f);
			Qp[wi][r] = make_float2(0.f, 0.f);
		}

	bool failed = false;
	uint64_t k = 0;
	int foldLeft = foldTiles(a.reduction);
	// stage, phase parity and first event of tile k, advanced incrementally
	// (no division by the runtime stage count inside the loop)
	int s = 0;
	uint32_t parity = 0;
	uint64_t e0 = first * (uint64_t)E;
	for (; k < myTiles; ++k, e0 += stride * (uint64_t)E) {
		if (k != 0 && ++s == stages) {
			s = 0;
			parity ^= 1u;
		}
		const bool timedOut = !mbarWaitBounded(&bars[s], parity);
		const float2* tile = tiles + (size_t)s * W * E;
		// shared-memory regions for the debug build's bounds checks
		const uint32_t tLo = smemAddr(tile), tHi = tLo + stageBytes;
		float2* T = Ts + (size_t)(k & 1ull) * R * 2 * E;

		// ---- phase 1: coherent sums, combined across the lanes of an event ----
		{
			float2 S[R][2];
			int pe1;       // the event whose sums this lane holds after the combination
			bool writer;   // one lane per event writes its results
			const uint32_t vAddr = smemAddr(Vs);
			const uint32_t vHi = vAddr + (uint32_t)(W * R) * 8u;
			const uint32_t rowB = (uint32_t)lay.rowStride;
			// V of two consecutive ranks in one 128-bit load; the address
			// (w * R + r) * 8 is 16-byte aligned only for even R
			auto loadV = [&](int w, float2 (&v)[R]) {
				if ((R & 1) == 0) {
#pragma unroll
					for (int r = 0; r + 1 < R; r += 2) {
						const float4 q = lds128c(vAddr + (uint32_t)(w * R + r) * 8u, vAddr, vHi, a.devErr);
						v[r] = make_float2(q.x, q.y);
						v[r + 1] = make_float2(q.z, q.w);
					}
				} else {
#pragma unroll
					for (int r = 0; r < R; ++r)
						v[r] = lds64c(vAddr + (uint32_t)(w * R + r) * 8u, vAddr, vHi, a.devErr);
				}
			};
			if constexpr (NE == 1) {
				float2 Sa[R][2];
#pragma unroll
				for (int r = 0; r < R; ++r) {
					Sa[r][0] = make_float2(0.f, 0.f);
					Sa[r][1] = make_float2(0.f, 0.f);
				}
				// every row this lane reads has the same rotation (w = ph mod H)
				const int rot1 = (int)storeRot((uint32_t)ph, (uint32_t)E);  // 512 / E == H
				const uint32_t colAddr = smemAddr(tile + ((pe + rot1) & (E - 1)));
#pragma unroll 4
				for (int w = ph; w < W0; w += H) {
					const float2 av = lds64c(colAddr + (uint32_t)w * rowB, tLo, tHi, a.devErr);
					float2 v[R];
					loadV(w, v);
#pragma unroll
					for (int r = 0; r < R; ++r) {
						Sa[r][0].x = fmaf(v[r].x, av.x, fmaf(-v[r].y, av.y, Sa[r][0].x));
						Sa[r][0].y = fmaf(v[r].x, av.y, fmaf(v[r].y, av.x, Sa[r][0].y));
					}
				}
#pragma unroll 4
				for (int w = wStart1; w < W; w += H) {
					const float2 av = lds64c(colAddr + (uint32_t)w * rowB, tLo, tHi, a.devErr);
					float2 v[R];
					loadV(w, v);
#pragma unroll
					for (int r = 0; r < R; ++r) {
						Sa[r][1].x = fmaf(v[r].x, av.x, fmaf(-v[r].y, av.y, Sa[r][1].x));
						Sa[r][1].y = fmaf(v[r].x, av.y, fmaf(v[r].y, av.x, Sa[r][1].y));
					}
				}
#pragma unroll
				for (int r = 0; r < R; ++r)
#pragma unroll
					for (int e = 0; e < 2; ++e) {
						S[r][e] = Sa[r][e];
#pragma unroll
						for (int o = 1; o < H; o <<= 1) {
							S[r][e].x += __shfl_xor_sync(0xffffffffu, S[r][e].x, o);
							S[r][e].y += __shfl_xor_sync(0xffffffffu, S[r][e].y, o);
						}
					}
				pe1 = pe;
				writer = ph == 0;
			} else if constexpr (NE == 4) {
				// four consecutive events per lane, 16 wave slices per quad of
				// events: each V load serves four events.  A lane reads its
				// quad as two 16-byte halves; lanes of the second quad of the
				// warp read the upper half first, so that each quarter-warp
				// (2 quads x 4 slices with distinct store rotations) covers
				// all 32 banks once in both loads.
				static_assert(E == 128, "four events per lane need 128-event tiles");
				const int kLo = lane & 3, quad = (lane >> 2) & 1, sHi = (lane >> 3) & 3;
				const int ph4 = kLo + 4 * sHi;          // wave slice: waves w = ph4 mod 16
				const int pe0 = warp * EPW + 4 * quad;  // the quad's first event
				const int rot1 = (int)storeRot((uint32_t)ph4, (uint32_t)E);
				const uint32_t colA = smemAddr(tile + ((pe0 + rot1) & (E - 1)));
				// slot 0 = the half loaded first (events pe0 + 2 quad, + 1)
				const uint32_t off0 = colA + 16u * (uint32_t)quad, off1 = colA + 16u * (uint32_t)(1 - quad);
				auto mac4 = [&](int w, float2 (&Sx)[2][2][R]) {
					const float4 p0 = lds128c(off0 + (uint32_t)w * rowB, tLo, tHi, a.devErr);
					const float4 p1 = lds128c(off1 + (uint32_t)w * rowB, tLo, tHi, a.devErr);
					float2 v[R];
					loadV(w, v);
#pragma unroll
					for (int r = 0; r < R; ++r) {
						Sx[0][0][r].x = fmaf(v[r].x, p0.x, fmaf(-v[r].y, p0.y, Sx[0][0][r].x));
						Sx[0][0][r].y = fmaf(v[r].x, p0.y, fmaf(v[r].y, p0.x, Sx[0][0][r].y));
						Sx[0][1][r].x = fmaf(v[r].x, p0.z, fmaf(-v[r].y, p0.w, Sx[0][1][r].x));
						Sx[0][1][r].y = fmaf(v[r].x, p0.w, fmaf(v[r].y, p0.z, Sx[0][1][r].y));
						Sx[1][0][r].x = fmaf(v[r].x, p1.x, fmaf(-v[r].y, p1.y, Sx[1][0][r].x));
						Sx[1][0][r].y = fmaf(v[r].x, p1.y, fmaf(v[r].y, p1.x, Sx[1][0][r].y));
						Sx[1][1][r].x = fmaf(v[r].x, p1.z, fmaf(-v[r].y, p1.w, Sx[1][1][r].x));
						Sx[1][1][r].y = fmaf(v[r].x, p1.w, fmaf(v[r].y, p1.z, Sx[1][1][r].y));
					}
				};
				float2 SN[2][2][R], SP[2][2][R];  // [slot][event of the slot][rank], per reflectivity
#pragma unroll
				for (int q = 0; q < 2; ++q)
#pragma unroll
					for (int j = 0; j < 2; ++j)
#pragma unroll
						for (int r = 0; r < R; ++r)
							SN[q][j][r] = SP[q][j][r] = make_float2(0.f, 0.f);
#pragma unroll 1
				for (int w = ph4; w < W0; w += 16)
					mac4(w, SN);
				const int wS1 = W0 + (((ph4 - W0) % 16) + 16) % 16;
#pragma unroll 1
				for (int w = wS1; w < W; w += 16)
					mac4(w, SP);
				// reduce-scatter over lane bit 16 (slot) and bit 8 (event of
				// the slot), butterfly over bits 0-1: the lane ends with the
				// sums of event pe0 + 2 (bs ^ quad) + be
				const int bs = (lane >> 4) & 1, be = (lane >> 3) & 1;
#pragma unroll
				for (int r = 0; r < R; ++r)
#pragma unroll
					for (int e = 0; e < 2; ++e) {
						const float2 (&Se)[2][2][R] = e ? SP : SN;
						float2 k0 = bs ? Se[1][0][r] : Se[0][0][r];
						float2 k1 = bs ? Se[1][1][r] : Se[0][1][r];
						const float2 s0 = bs ? Se[0][0][r] : Se[1][0][r];
						const float2 s1 = bs ? Se[0][1][r] : Se[1][1][r];
						k0.x += __shfl_xor_sync(0xffffffffu, s0.x, 16);
						k0.y += __shfl_xor_sync(0xffffffffu, s0.y, 16);
						k1.x += __shfl_xor_sync(0xffffffffu, s1.x, 16);
						k1.y += __shfl_xor_sync(0xffffffffu, s1.y, 16);
						float2 keep = be ? k1 : k0;
						const float2 send = be ? k0 : k1;
						keep.x += __shfl_xor_sync(0xffffffffu, send.x, 8);
						keep.y += __shfl_xor_sync(0xffffffffu, send.y, 8);
#pragma unroll
						for (int o = 1; o < 4; o <<= 1) {
							keep.x += __shfl_xor_sync(0xffffffffu, keep.x, o);
							keep.y += __shfl_xor_sync(0xffffffffu, keep.y, o);
						}
						S[r][e] = keep;
					}
				pe1 = pe0 + 2 * (bs ^ quad) + be;
				writer = kLo == 0;
			} else {
				// two consecutive events per lane: one 128-bit load brings a
				// wave's amplitudes of both, and each V load serves both.
				// Quarter-warp q holds PQ adjacent event pairs x QPH wave
				// slices with distinct rotations, so its eight 16-byte loads
				// cover all 32 banks once.
				constexpr int PPW = EPW / 2;  // event pairs per warp
				constexpr int H2 = 32 / PPW;  // lanes (wave slices) per pair
				constexpr int PQ = E / 64;    // pairs per quarter-warp
				constexpr int QPH = 8 / PQ;   // wave slices per quarter-warp
				static_assert(PQ * QPH == 8 && 2 * PQ == PPW && 2 * QPH == H2, "two-event phase-1 shape");
				const int phLo = lane & (QPH - 1);
				const int pm2 = ((lane >> 3) & 1) * PQ + ((lane / QPH) & (PQ - 1));
				const int ph2 = phLo + QPH * (lane >> 4);
				const int pe0 = warp * EPW + 2 * pm2;
				// H2 is a multiple of 512 / E: one rotation for all rows of the slice
				const int rot1 = (int)storeRot((uint32_t)ph2, (uint32_t)E);
				const uint32_t colAddr = smemAddr(tile + ((pe0 + rot1) & (E - 1)));
				// coherent sums of both events, FP32 FMA chains as in the
				// one-event variant: S[r][ev] per reflectivity
				auto mac = [&](int w, float2 (&Sx)[R][2]) {
					const float4 av = lds128c(colAddr + (uint32_t)w * rowB, tLo, tHi, a.devErr);
					float2 v[R];
					loadV(w, v);
#pragma unroll
					for (int r = 0; r < R; ++r) {
						Sx[r][0].x = fmaf(v[r].x, av.x, fmaf(-v[r].y, av.y, Sx[r][0].x));
						Sx[r][0].y = fmaf(v[r].x, av.y, fmaf(v[r].y, av.x, Sx[r][0].y));
						Sx[r][1].x = fmaf(v[r].x, av.z, fmaf(-v[r].y, av.w, Sx[r][1].x));
						Sx[r][1].y = fmaf(v[r].x, av.w, fmaf(v[r].y, av.z, Sx[r][1].y));
					}
				};
				float2 S0[R][2], S1[R][2];
#pragma unroll
				for (int r = 0; r < R; ++r)
#pragma unroll
					for (int j = 0; j < 2; ++j)
						S0[r][j] = S1[r][j] = make_float2(0.f, 0.f);
#pragma unroll 2
				for (int w = ph2; w < W0; w += H2)
					mac(w, S0);
				const int wS1 = W0 + (((ph2 - W0) % H2) + H2) % H2;
#pragma unroll 4
				for (int w = wS1; w < W; w += H2)
					mac(w, S1);
				// a reduce-scatter over the slice bit 16 (lanes with that bit
				// keep the second event) and a butterfly over the remaining
				// slice bits
				const int mine = (lane >> 4) & 1;
#pragma unroll
				for (int r = 0; r < R; ++r)
#pragma unroll
					for (int e = 0; e < 2; ++e) {
						const float2 (&Se)[R][2] = e ? S1 : S0;
						float2 keep = mine ? Se[r][1] : Se[r][0];
						const float2 send = mine ? Se[r][0] : Se[r][1];
						keep.x += __shfl_xor_sync(0xffffffffu, send.x, 16);
						keep.y += __shfl_xor_sync(0xffffffffu, send.y, 16);
#pragma unroll
						for (int o = 1; o < QPH; o <<= 1) {
							keep.x += __shfl_xor_sync(0xffffffffu, keep.x, o);
							keep.y += __shfl_xor_sync(0xffffffffu, keep.y, o);
						}
						S[r][e] = keep;
					}
				pe1 = pe0 + mine;
				writer = phLo == 0;
			}
			float L = flat2;
#pragma unroll
			for (int r = 0; r < R; ++r)
#pragma unroll
				for (int e = 0; e < 2; ++e)
					L = fmaf(S[r][e].x, S[r][e].x, fmaf(S[r][e].y, S[r][e].y, L));
			const bool valid = (e0 + (uint64_t)pe1) < a.nEvents;
			const float c = valid ? eventWeight(L) : 0.f;
			if (writer) {
				if (valid)
					llPart += -eventLog(L);
				cPart += c;
				if (a.withGrad) {
#pragma unroll
					for (int r = 0; r < R; ++r)
#pragma unroll
						for (int e = 0; e < 2; ++e) {
							const float tx = c * S[r][e].x, ty = c * S[r][e].y;
							const int ti = (r * 2 + e) * E + pe1;
							if (smemInBounds(smemAddr(T + ti), 8u, smemAddr(T), smemAddr(T + R * 2 * E), a.devErr)) {
								T[ti] = make_float2(tx, ty);
							}
						}
				}
			}
		}
		// the only block barrier per tile: T complete (and a uniform exit on timeout)
		if (__syncthreads_or(timedOut)) {
			failed = true;
			break;
		}

		// ---- phase 2: gradient contraction over the tile, one reflectivity per warp ----
		if (a.withGrad) {
			const uint32_t tAddr = smemAddr(tile);
			const uint32_t tBase = smemAddr(T) + tOff;
#pragma unroll
			for (int pp = 0; pp < EPAIRS; ++pp) {
				float4 t[R];
#pragma unroll
				for (int r = 0; r < R; ++r) {
					t[r] = lds128c(tBase + (uint32_t)(r * 2 * E + 64 * pp) * 8u, smemAddr(T),
					               smemAddr(T + R * 2 * E), a.devErr);

				}
#pragma unroll
				for (int wi = 0; wi < WPW; ++wi) {
					if (wi < nWarpWaves) {
						const float4 av = lds128c(tAddr + (aOff[wi] ^ (uint32_t)(pp * 512)), tLo, tHi, a.devErr);
						const float2 a0 = make_float2(av.x, av.y), a1 = make_float2(av.z, av.w);
#pragma unroll
						for (int r = 0; r < R; ++r) {
							if constexpr (kPacked) {
								Pp[wi][r] = ffma2(a0, make_float2(t[r].x, t[r].y), Pp[wi][r]);
								Pp[wi][r] = ffma2(a1, make_float2(t[r].z, t[r].w), Pp[wi][r]);
								// the swapped (ty, tx) pairs come from registers
								Qp[wi][r] = ffma2(a0, make_float2(t[r].y, t[r].x), Qp[wi][r]);
								Qp[wi][r] = ffma2(a1, make_float2(t[r].w, t[r].z), Qp[wi][r]);
							} else {
								// G += conj(a) t: (ax tx + ay ty, ax ty - ay tx)
								Pp[wi][r].x = fmaf(a0.x, t[r].x, fmaf(a0.y, t[r].y, Pp[wi][r].x));
								Pp[wi][r].y = fmaf(a0.x, t[r].y, fmaf(-a0.y, t[r].x, Pp[wi][r].y));
								Pp[wi][r].x = fmaf(a1.x, t[r].z, fmaf(a1.y, t[r].w, Pp[wi][r].x));
								Pp[wi][r].y = fmaf(a1.x, t[r].w, fmaf(-a1.y, t[r].z, Pp[wi][r].y));
							}
						}
					}
				}
			}
		}

		// stage s is no longer read by this warp; the last warp to finish
		// with it refills it with tile k + stages
		__syncwarp();
		unsigned prev = 0;
		if (lane == 0) {
			__threadfence_block();
			prev = atomicAdd(&done[s], 1u);
		}
		prev = __shfl_sync(0xffffffffu, prev, 0);
		if (prev == (unsigned)(kWarps - 1)) {
			if (lane == 0)
				atomicExch(&done[s], 0u);
			if (k + (uint64_t)stages < myTiles) {
				fenceProxyAsync();
				issue(k + (uint64_t)stages, s);
			}
		}

		// fold the FP32 tile partials every foldTiles(reduction) tiles and after the last tile
		if (--foldLeft == 0 || k + 1 == myTiles) {
			foldLeft = foldTiles(a.reduction);
			const float ll = warpSum(llPart), cs = warpSum(cPart);
			llPart = 0.f;
			cPart = 0.f;
			if (lane == 0) {
				if (a.reduction == 0) {
					accLL += (double)ll;
					accC += (double)cs;
				} else if (a.reduction == 1) {
					kahanAdd(kLL, kLLc, ll);
					kahanAdd(kC, kCc, cs);
				} else {
					kLL += ll;
					kC += cs;
				}
			}
			if (a.withGrad) {
				float part[NVP];
#pragma unroll
				for (int wi = 0; wi < WPW; ++wi)
#pragma unroll
					for (int r = 0; r < R; ++r) {
						part[(wi * R + r) * 2 + 0] = kPacked ? Pp[wi][r].x + Pp[wi][r].y : Pp[wi][r].x;
						part[(wi * R + r) * 2 + 1] = kPacked ? Qp[wi][r].x - Qp[wi][r].y : Pp[wi][r].y;
						Pp[wi][r] = make_float2(0.f, 0.f);
						Qp[wi][r] = make_float2(0.f, 0.f);
					}
#pragma unroll
				for (int v = NV; v < NVP; ++v)
					part[v] = 0.f;
#pragma unroll
				for (int q = 0; q < NQ; ++q) {
					const float v = reduceScatter32(&part[q * 32], lane);
					if (a.reduction == 0)
						accG[q] += (double)v;
					else if (a.reduction == 1)
						kahanAdd(kG[q], kGc[q], v);
					else
						kG[q] += v;
				}
			}
		}
	}

	if (failed) {
		// let our own copies in flight land (bounded): tiles up to
		// k - 1 + stages have been issued; the partials of this block are
		// incomplete and the error flag tells the host to discard the result
		if (tid == 0) {
			atomicOr(a.devErr, (unsigned)kDevErrTimeout);
			for (uint64_t j = k; j < k + (uint64_t)stages && j < myTiles; ++j) {
				const int s = (int)(j % (uint64_t)stages);
				mbarWaitBounded(&bars[s], (uint32_t)((j / (uint64_t)stages) & 1ull));
			}
		}
	}

	// ---- epilogue: the block's partials go into the exact fixed-point
	// accumulators; the last block writes the results ----
	// (the previous launch's tail may still read the accumulators and the
	// slot scratch when this grid starts early under programmatic dependent
	// launch)
	gridDependencyWait();

	const size_t ls = (size_t)a.nPartial;
	unsigned long long* myAcc = a.fixAcc + (blockIdx.x % kReplicas) * (size_t)kLimbs * ls;
	// normalisation and prior terms do not depend on the events: blocks with
	// one tile fewer compute them after their event loop
	fdfNormTerms(a, V64, nTiles, myAcc, ls, warp, lane);
	if (lane == 0) {
		fixedAdd(myAcc + 0, ls, a.nfAcc + 0, (a.reduction == 0) ? accLL : (double)kLL - (double)kLLc);
		fixedAdd(myAcc + 1, ls, a.nfAcc + 1, (a.reduction == 0) ? accC : (double)kC - (double)kCc);
	}
	if (a.withGrad) {
#pragma unroll
		for (int q = 0; q < NQ; ++q) {
			const int vi = q * 32 + lane;
			if (vi < NV) {
				const int wi = vi / (2 * R);
				const int rem = vi - wi * 2 * R;
				const int r = rem >> 1, comp = rem & 1;
				if (wi < nWarpWaves) {
					const int w = wBase + wi;
					const double v = (a.reduction == 0) ? accG[q] : ((double)kG[q] - (double)kGc[q]);
					const int slotVal = 2 + (r * W + w) * 2 + comp;
					fixedAdd(myAcc + slotVal, ls, a.nfAcc + slotVal, v);
				}
			}
		}
	}
	__shared__ unsigned sLast;
	fdfTail(a, &sLast, flatD, tid);
}

__global__ void convertRowKernel(const void* src, int srcIsDouble, float2* store, uint32_t W, uint32_t w, uint32_t B,
                                 uint64_t n, double divisor, unsigned* nonzero)
{
	bool any = false;
	for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
		double re, im;
		if (srcIsDouble) {
			const double2 v = reinterpret_cast<const double2*>(src)[i];
			re = v.x;
			im = v.y;
		} else {
			const float2 v = reinterpret_cast<const float2*>(src)[i];
			re = v.x;
			im = v.y;
		}
		any = any || re != 0. || im != 0.;
		store[storeIndex(w, i, W, B)] = make_float2((float)(re / divisor), (float)(im / divisor));
	}
	if (__any_sync(0xffffffffu, any) && (threadIdx.x & 31) == 0)
		atomicOr(nonzero, 1u);
}

__global__ void convertPlainKernel(const double2* src, float2* dst, uint64_t n)
{
	for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
		const double2 v = src[i];
		dst[i] = make_float2((float)v.x, (float)v.y);
	}
}

template <int R, int E, int WPW, int NE>
int launchVariant(const FdfPlan& p, const FdfArgs& a, cudaStream_t s)
{
	auto kern = fdfMainKernel<R, E, WPW, NE>;
	// raise the dynamic shared-memory limit once per variant (not a stream
	// operation, so it is kept out of the launches captured into graphs)
	static size_t configured = 0;
	if (p.smemBytes > configured) {
		const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p.smemBytes);
		if (e != cudaSuccess)
			return cudaCheck(e, "cudaFuncSetAttribute(fdf)");
		configured = p.smemBytes;
	}
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3(p.blocks);
	cfg.blockDim = dim3(kThreads);
	cfg.dynamicSmemBytes = p.smemBytes;
	cfg.stream = s;
	cudaLaunchAttribute attr[1];
	attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
	attr[0].val.programmaticStreamSerializationAllowed = 1;
	cfg.attrs = attr;
	cfg.numAttrs = 1;
	const cudaError_t e = cudaLaunchKernelEx(&cfg, kern, a, p.stages);
	countLaunches(1);
	return cudaCheck(e, "fdf kernel launch");
}

template <int R, int NE>
int launchRN(const FdfPlan& p, const FdfArgs& a, cudaStream_t s)
{
	if (p.E == 128) {
		switch (p.wpw) {
		case 2: return launchVariant<R, 128, 2, NE>(p, a, s);
		case 4: return launchVariant<R, 128, 4, NE>(p, a, s);
		case 6: return launchVariant<R, 128, 6, NE>(p, a, s);
		case 8: return launchVariant<R, 128, 8, NE>(p, a, s);
		default: break;
		}
	} else if constexpr (NE != 4) {  // four events per lane: 128-event tiles only
		if (p.E == 64) {
			switch (p.wpw) {
			case 2: return launchVariant<R, 64, 2, NE>(p, a, s);
			case 4: return launchVariant<R, 64, 4, NE>(p, a, s);
			case 6: return launchVariant<R, 64, 6, NE>(p, a, s);
			case 8: return launchVariant<R, 64, 8, NE>(p, a, s);
			case 14: return launchVariant<R, 64, 14, NE>(p, a, s);
			default: break;
			}
		}
	}
	return setError(kErrUnsupported, "no FdF kernel variant for this tile/wave bucket");
}

template <int R>
int launchR(const FdfPlan& p, const FdfArgs& a, cudaStream_t s)
{
	if constexpr (R <= 2) {
		if (p.phase1Events == 4)
			return launchRN<R, 4>(p, a, s);
	}
	return p.phase1Events == 2 ? launchRN<R, 2>(p, a, s) : launchRN<R, 1>(p, a, s);
}

}  // namespace

int chooseStoreBlock(int W, int R, size_t maxSmem)
{
	return (smemLayout(W, R, 128, 2).total + 1024 <= maxSmem) ? 128 : 64;
}

int planCandidates(int W0, int W, int R, int B, uint64_t nEvents, int numSMs, size_t maxSmem,
                   std::vector<FdfPlan>* out)
{
	out->clear();
	if (R < 1 || R > 4)
		return setError(kErrUnsupported, "FdF kernel supports rank 1..4");
	if (W < 1)
		return setError(kErrArg, "no waves");
	int nNeg, wn, wp;
	const int wpwa = waveSplit(W0, W, &nNeg, &wn, &wp);
	int wpw;
	if (wpwa <= 2) wpw = 2;
	else if (wpwa <= 4) wpw = 4;
	else if (wpwa <= 6) wpw = 6;
	else if (wpwa <= 8) wpw = 8;
	else if (wpwa <= 14) wpw = 14;
	else return setError(kErrUnsupported, "FdF kernel supports at most 224 waves");
	if (R * wpw > 32)
		return setError(kErrUnsupported, "rank x waves-per-warp beyond the compiled register budget");
	if (B != 128 && B != 64)
		return setError(kErrArg, "store block must be 64 or 128 events");
	for (int st = 1; st <= 4; ++st) {
		if (smemLayout(W, R, B, st).total + 1024 > maxSmem)
			break;
		FdfPlan p;
		p.E = B;
		p.stages = st;
		p.wpw = wpw;
		const uint64_t nTiles = (nEvents + B - 1) / B;
		p.blocks = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)numSMs, nTiles));
		p.smemBytes = smemLayout(W, R, B, st).total;
		// the default without autotuning first: two events per lane up to
		// rank 2, one beyond (where two would spill registers); four events
		// per lane (128-event tiles, rank <= 2) is timed by the autotuner
		const int order[3] = {R <= 2 ? 2 : 1, R <= 2 ? 1 : 2, (R <= 2 && B == 128) ? 4 : 0};
		for (int ne : order) {
			if (ne == 0)
				continue;
			p.phase1Events = ne;
			out->push_back(p);
		}
	}
	if (out->empty())
		return setError(kErrUnsupported, "amplitude tile does not fit in shared memory");
	// a single stage does not overlap copy and compute: drop it when deeper pipelines fit
	const size_t perStage = (R <= 2 && B == 128) ? 3 : 2;
	if (out->size() > perStage)
		out->erase(out->begin(), out->begin() + perStage);
	// the fused-gradient variant, with two or more stages where it fits
	if (B == 128)
		for (int st = 2; st <= 4; ++st) {
			const size_t need = fusedFdfSmem(W0, W, R, st);
			if (need == 0 || need + 1024 > maxSmem)
				break;
			FdfPlan p;
			p.E = B;
			p.stages = st;
			p.wpw = wpw;
			p.phase1Events = 3;
			const uint64_t nTiles = (nEvents + B - 1) / B;
			p.blocks = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)numSMs, nTiles));
			p.smemBytes = need;
			out->push_back(p);
		}
	// the narrow variant for small wave sets, two to four stages where they fit
	if (B == 128)
		for (int st = 2; st <= 4; ++st) {
			const size_t need = narrowFdfSmem(W, R, st);
			if (need == 0 || need + 1024 > maxSmem)
				break;
			FdfPlan p;
			p.E = B;
			p.stages = st;
			p.wpw = wpw;
			p.phase1Events = 5;
			p.blocks = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)numSMs, narrowFdfTiles(nEvents)));
			p.smemBytes = need;
			out->push_back(p);
		}
	return kOk;
}

size_t fdfAccumulatorWords(int nPartial) { return (size_t)kReplicas * kLimbs * (size_t)nPartial; }

int launchFdf(const FdfPlan& p, const FdfArgs& a, cudaStream_t s)
{
	if (p.phase1Events == 5)
		return launchFdfNarrow(p, a, s);
	if (p.phase1Events == 3) {
		if (a.reduction == 0)
			return launchFdfFused(p, a, s);
		// the FP32 reduction modes are those of the main kernel (two events
		// per lane, the fused variant's pipeline depth)
		FdfPlan q = p;
		q.phase1Events = 2;
		q.smemBytes = smemLayout(a.W, a.R, q.E, q.stages).total;
		int nNeg, wn, wp;
		const int wpwa = waveSplit(a.W0, a.W, &nNeg, &wn, &wp);
		q.wpw = wpwa <= 2 ? 2 : wpwa <= 4 ? 4 : wpwa <= 6 ? 6 : wpwa <= 8 ? 8 : 14;
		switch (a.R) {
		case 1: return launchR<1>(q, a, s);
		case 2: return launchR<2>(q, a, s);
		default: return setError(kErrUnsupported, "fused FdF plan beyond rank 2");
		}
	}
	switch (a.R) {
	case 1: return launchR<1>(p, a, s);
	case 2: return launchR<2>(p, a, s);
	case 3: return launchR<3>(p, a, s);
	case 4: return launchR<4>(p, a, s);
	default: return setError(kErrUnsupported, "FdF kernel supports rank 1..4");
	}
}

int launchConvertPlain(const void* src, float2* dst, uint64_t n, cudaStream_t s)
{
	const int threads = 256;
	const int blocks = (int)std::min<uint64_t>((n + threads - 1) / threads, 4096);
	convertPlainKernel<<<std::max(blocks, 1), threads, 0, s>>>(static_cast<const double2*>(src), dst, n);
	countLaunches(1);
	return cudaCheck(cudaGetLastError(), "convert launch");
}

int launchConvertRow(const void* src, int srcIsDouble, float2* store, uint32_t W, uint32_t w, uint32_t B, uint64_t n,
                     double divisor, unsigned* nonzero, cudaStream_t s)
{
	const int threads = 256;
	const int blocks = (int)std::min<uint64_t>((n + threads - 1) / threads, 4096);
	convertRowKernel<<<std::max(blocks, 1), threads, 0, s>>>(src, srcIsDouble, store, W, w, B, n, divisor, nonzero);
	countLaunches(1);
	return cudaCheck(cudaGetLastError(), "convert row launch");
}

}  // namespace pwa
