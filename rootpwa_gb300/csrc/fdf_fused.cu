// fdf_fused.cu -- fused-gradient variant of the FdF kernel.
//
// Same result as fdfMainKernel (partialWaveFit/pwaLikelihood.cc:209-244,
// :254-297 and :1714-1731: -sum ln L_i, the normalisation and prior terms
// and the analytic gradient), with a different division of the work inside
// a block.  In fdfMainKernel the gradient contraction of a tile needs the
// coherent sums of all 128 events, so c S goes through shared memory and the
// block synchronises once per tile.  Here every warp finishes its own eight
// events of a tile by itself:
//   * each lane holds two adjacent events and a slice of the waves (waves
//     w = ph (mod 8)); one 128-bit load per wave brings both events'
//     amplitudes (a quarter-warp holds two event pairs x four slices with
//     distinct store rotations, so its loads hit all 32 banks once);
//   * the coherent sums S of the pair are combined over the 8 lanes of the
//     pair (a reduce-scatter over lane bit 16, a butterfly over bits 0-1);
//     each lane then has L, c and c S of one event and gets the other
//     event's c S with one shuffle;
//   * the lane reads the same amplitudes again (its waves, its two events)
//     and accumulates G_{r,w} += c S_{r,e(w)} conj(A_w) in FP32 registers;
//   * every kFoldF tiles the four lanes sharing a wave slice are summed by a
//     butterfly and added to the warp's FP64 partials in shared memory;
//     after the event loop the block sums its warps' partials in a fixed
//     order and adds them to the exact fixed-point accumulators.
// There is no block barrier per tile and no c S traffic through shared
// memory; the stage refill is the counter-driven one of fdfMainKernel.
// Every mbarrier wait is bounded; a warp that times out leaves its loop, the
// others time out in turn on the stage it no longer releases, and thread 0
// waits (bounded) for the last copy issued into each stage before the block
// exits.

#include "fdf_common.cuh"

#include <algorithm>

namespace pwa {
namespace {

constexpr int kE = 128;      // events per tile
constexpr int kFoldF = 16;   // tiles between the FP32 -> FP64 folds of the gradient

struct FusedLayout {
	size_t rowStride, tiles, vs, v64, g64, bars, done, issued, total;
};

__host__ __device__ inline FusedLayout fusedLayout(int W, int R, int stages)
{
	auto up = [](size_t x) { return (x + 127) & ~(size_t)127; };
	FusedLayout L;
	L.rowStride = (size_t)kE * 8;
	L.tiles = 0;
	L.vs = up((size_t)stages * W * L.rowStride);
	L.v64 = up(L.vs + (size_t)(W + 1) * R * 8);  // one zero wave after the last
	L.g64 = up(L.v64 + (size_t)W * R * 16);
	L.bars = up(L.g64 + (size_t)kWarps * 2 * R * W * 8);
	L.done = L.bars + (size_t)stages * 8;
	L.issued = L.done + (size_t)stages * 4;
	L.total = L.issued + (size_t)stages * 4;
	return L;
}

template <int R, int NEG, int POS>
__global__ void __launch_bounds__(kThreads, 1) fdfFusedKernel(const FdfArgs a, const int stages)
{
	extern __shared__ __align__(128) unsigned char smem[];
	constexpr int E = kE;
	constexpr int EPW = E / kWarps;  // events per warp
	constexpr int NGA = NEG > 0 ? NEG : 1;
	static_assert(EPW == 8, "two events per lane, four pairs per warp");

	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const int W = a.W, W0 = a.W0;
	const int nG = 2 * R * W;
	const FusedLayout lay = fusedLayout(W, R, stages);
	float2* tiles = reinterpret_cast<float2*>(smem + lay.tiles);
	float2* Vs = reinterpret_cast<float2*>(smem + lay.vs);      // [W][R] (vx, vy)
	double2* V64 = reinterpret_cast<double2*>(smem + lay.v64);  // [R][W] FP64, slot order
	double* G64 = reinterpret_cast<double*>(smem + lay.g64);    // [warp][2 R W] gradient partials
	uint64_t* bars = reinterpret_cast<uint64_t*>(smem + lay.bars);
	unsigned* done = reinterpret_cast<unsigned*>(smem + lay.done);
	unsigned* issued = reinterpret_cast<unsigned*>(smem + lay.issued);

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
			issued[s] = 0u;
		}
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	__syncthreads();

	// issue store block (tile) k (local index) into stage s: one bulk copy
	auto issue = [&](uint64_t k, int s) {
		if (lane == 0) {
			const float2* src = a.amps + (first + k * stride) * (uint64_t)W * E;
			issued[s] += 1u;
			mbarArriveExpectTx(&bars[s], stageBytes);
			bulkCopyG2S(tiles + (size_t)s * W * E, src, stageBytes, &bars[s]);
		}
	};
	// the amplitude store does not change after finishInit, so the first
	// stages load while the preceding grid ends
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
	if (tid < R)
		Vs[W * R + tid] = make_float2(0.f, 0.f);
	const double flatD = a.par[a.P - 1];
	const float flat2 = (float)(flatD * flatD);
	if (a.withGrad)
		for (int i = tid; i < kWarps * nG; i += kThreads)
			G64[i] = 0.;
	__syncthreads();

	// lane roles: event pair pm2 of the warp (events pe0, pe0 + 1), wave
	// slice ph2 (waves w = ph2 mod 8 of each reflectivity); after the
	// combination the lane holds event pe0 + mine
	const int phLo = lane & 3;
	const int pm2 = ((lane >> 3) & 1) * 2 + ((lane >> 2) & 1);
	const int ph2 = phLo + 4 * (lane >> 4);
	const int pe0 = warp * EPW + 2 * pm2;
	const int mine = (lane >> 4) & 1;
	const int n0 = ph2 < W0 ? (W0 - 1 - ph2) / 8 + 1 : 0;
	const int wS1 = W0 + (((ph2 - W0) % 8) + 8) % 8;
	const int n1 = wS1 < W ? (W - 1 - wS1) / 8 + 1 : 0;
	const uint32_t rowB = (uint32_t)lay.rowStride;
	// every row of the slice has the same store rotation (8 is a multiple of 512 / E)
	const uint32_t colOff = (uint32_t)((pe0 + (int)storeRot((uint32_t)ph2, (uint32_t)E)) & (E - 1)) * 8u;
	const uint32_t vBase = smemAddr(Vs);
	// every lane runs NEG = ceil(W0 / 8) and POS = ceil(W1 / 8) waves (the
	// warp's maximum) without branches.  Only the last wave of each kind can
	// be beyond a lane's share; that one reads a valid amplitude row (the
	// last) with the zero V after the last wave, so it adds nothing to the
	// coherent sums, and its gradient accumulator is never folded.  The other
	// waves are at fixed offsets from the lane's first row.
	const uint32_t aNeg = (uint32_t)ph2 * rowB + colOff, aPos = (uint32_t)wS1 * rowB + colOff;
	const uint32_t vNeg = vBase + (uint32_t)(ph2 * R) * 8u, vPos = vBase + (uint32_t)(wS1 * R) * 8u;
	constexpr int JN = NEG > 0 ? NEG - 1 : 0;
	const uint32_t aNegLast = (uint32_t)min(ph2 + 8 * JN, W - 1) * rowB + colOff;
	const uint32_t vNegLast = vBase + (uint32_t)(((ph2 + 8 * JN < W0) ? ph2 + 8 * JN : W) * R) * 8u;
	const uint32_t aPosLast = (uint32_t)min(wS1 + 8 * (POS - 1), W - 1) * rowB + colOff;
	const uint32_t vPosLast = vBase + (uint32_t)(min(wS1 + 8 * (POS - 1), W) * R) * 8u;
	auto rowNeg = [&](int j) { return j == NEG - 1 ? aNegLast : aNeg + (uint32_t)j * 8u * rowB; };
	auto vNegA = [&](int j) { return j == NEG - 1 ? vNegLast : vNeg + (uint32_t)(j * 8 * R) * 8u; };
	auto rowPos = [&](int j) { return j == POS - 1 ? aPosLast : aPos + (uint32_t)j * 8u * rowB; };
	auto vPosA = [&](int j) { return j == POS - 1 ? vPosLast : vPos + (uint32_t)(j * 8 * R) * 8u; };

	// V of two consecutive ranks in one 128-bit load where the address is
	// 16-byte aligned (even R)
	const uint32_t vHi = vBase + (uint32_t)((W + 1) * R) * 8u;  // debug-build bounds
	auto loadV = [&](uint32_t addr, float2 (&v)[R]) {
		if ((R & 1) == 0) {
#pragma unroll
			for (int r = 0; r + 1 < R; r += 2) {
				const float4 q = lds128c(addr + (uint32_t)r * 8u, vBase, vHi, a.devErr);
				v[r] = make_float2(q.x, q.y);
				v[r + 1] = make_float2(q.z, q.w);
			}
		} else {
#pragma unroll
			for (int r = 0; r < R; ++r)
				v[r] = lds64c(addr + (uint32_t)r * 8u, vBase, vHi, a.devErr);
		}
	};
	// S[r][j] += V_r A of event j of the pair
	auto mac = [&](const float4& av, const float2 (&v)[R], float2 (&S)[R][2]) {
#pragma unroll
		for (int r = 0; r < R; ++r) {
			S[r][0].x = fmaf(v[r].x, av.x, fmaf(-v[r].y, av.y, S[r][0].x));
			S[r][0].y = fmaf(v[r].x, av.y, fmaf(v[r].y, av.x, S[r][0].y));
			S[r][1].x = fmaf(v[r].x, av.z, fmaf(-v[r].y, av.w, S[r][1].x));
			S[r][1].y = fmaf(v[r].x, av.w, fmaf(v[r].y, av.z, S[r][1].y));
		}
	};
	// G_r += conj(A_j) T_j over the pair's events j
	auto gmac = [&](const float4& av, const float2* t0, const float2* t1, float2 (&G)[R]) {
#pragma unroll
		for (int r = 0; r < R; ++r) {
			G[r].x = fmaf(av.x, t0[r].x, fmaf(av.y, t0[r].y, G[r].x));
			G[r].y = fmaf(av.x, t0[r].y, fmaf(-av.y, t0[r].x, G[r].y));
			G[r].x = fmaf(av.z, t1[r].x, fmaf(av.w, t1[r].y, G[r].x));
			G[r].y = fmaf(av.z, t1[r].y, fmaf(-av.w, t1[r].x, G[r].y));
		}
	};

	float2 Gn[NGA][R], Gp[POS > 0 ? POS : 1][R];
#pragma unroll
	for (int j = 0; j < NGA; ++j)
#pragma unroll
		for (int r = 0; r < R; ++r)
			Gn[j][r] = make_float2(0.f, 0.f);
#pragma unroll
	for (int j = 0; j < (POS > 0 ? POS : 1); ++j)
#pragma unroll
		for (int r = 0; r < R; ++r)
			Gp[j][r] = make_float2(0.f, 0.f);
	double accLL = 0., accC = 0.;
	float kLL = 0.f, kLLc = 0.f, kC = 0.f, kCc = 0.f;
	float llPart = 0.f, cPart = 0.f;

	bool failed = false;
	uint64_t k = 0;
	int s = 0;
	uint32_t parity = 0;
	uint64_t e0 = first * (uint64_t)E;
	for (; k < myTiles; ++k, e0 += stride * (uint64_t)E) {
		if (k != 0 && ++s == stages) {
			s = 0;
			parity ^= 1u;
		}
		if (!mbarWaitBounded(&bars[s], parity)) {
			failed = true;
			break;
		}
		const uint32_t tAddr = smemAddr(tiles + (size_t)s * W * E);
		const uint32_t tHi = tAddr + stageBytes;  // debug-build bounds

		// ---- coherent sums of the pair over this lane's waves ----
		float2 S0[R][2], S1[R][2];
#pragma unroll
		for (int r = 0; r < R; ++r)
#pragma unroll
			for (int j = 0; j < 2; ++j)
				S0[r][j] = S1[r][j] = make_float2(0.f, 0.f);
#pragma unroll
		for (int j = 0; j < NEG; ++j) {
			const float4 av = lds128c(tAddr + rowNeg(j), tAddr, tHi, a.devErr);
			float2 v[R];
			loadV(vNegA(j), v);
			mac(av, v, S0);
		}
#pragma unroll
		for (int j = 0; j < POS; ++j) {
			const float4 av = lds128c(tAddr + rowPos(j), tAddr, tHi, a.devErr);
			float2 v[R];
			loadV(vPosA(j), v);
			mac(av, v, S1);
		}
		float2 S[R][2];
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
				for (int o = 1; o < 4; o <<= 1) {
					keep.x += __shfl_xor_sync(0xffffffffu, keep.x, o);
					keep.y += __shfl_xor_sync(0xffffffffu, keep.y, o);
				}
				S[r][e] = keep;
			}
		float L = flat2;
#pragma unroll
		for (int r = 0; r < R; ++r)
#pragma unroll
			for (int e = 0; e < 2; ++e)
				L = fmaf(S[r][e].x, S[r][e].x, fmaf(S[r][e].y, S[r][e].y, L));
		const bool valid = (e0 + (uint64_t)(pe0 + mine)) < a.nEvents;
		const float c = valid ? eventWeight(L) : 0.f;
		if (phLo == 0) {
			if (valid)
				llPart += -eventLog(L);
			cPart += c;
		}

		// ---- gradient contributions of the pair over the same waves ----
		if (a.withGrad) {
			float2 T0[2][R], T1[2][R];  // [reflectivity][rank]: c S of the pair's first, second event
#pragma unroll
			for (int r = 0; r < R; ++r)
#pragma unroll
				for (int e = 0; e < 2; ++e) {
					const float2 t = make_float2(c * S[r][e].x, c * S[r][e].y);
					const float2 o = make_float2(__shfl_xor_sync(0xffffffffu, t.x, 16),
					                             __shfl_xor_sync(0xffffffffu, t.y, 16));
					T0[e][r] = mine ? o : t;
					T1[e][r] = mine ? t : o;
				}
#pragma unroll
			for (int j = 0; j < NEG; ++j) {
				const float4 av = lds128c(tAddr + rowNeg(j), tAddr, tHi, a.devErr);
				gmac(av, T0[0], T1[0], Gn[j]);
			}
#pragma unroll
			for (int j = 0; j < POS; ++j) {
				const float4 av = lds128c(tAddr + rowPos(j), tAddr, tHi, a.devErr);
				gmac(av, T0[1], T1[1], Gp[j]);
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

		// fold the FP32 partials every kFoldF tiles and after the last tile
		if ((k + 1) % kFoldF == 0 || k + 1 == myTiles) {
			const float ll = warpSum(llPart), cs = warpSum(cPart);
			llPart = 0.f;
			cPart = 0.f;
			if (lane == 0) {
				if (a.reduction == 0) {
					accLL += (double)ll;
					accC += (double)cs;
				} else {
					kahanAdd(kLL, kLLc, ll);
					kahanAdd(kC, kCc, cs);
				}
			}
			if (a.withGrad) {
				// the four lanes of a wave slice (lane bits 2 and 3) hold the
				// same waves for different event pairs; the shuffles run on
				// all lanes, the shared-memory adds on the first lane of each
				// slice only
				double* Gw = G64 + (size_t)warp * nG;
#pragma unroll
				for (int j = 0; j < NGA; ++j)
#pragma unroll
					for (int r = 0; r < R; ++r) {
						float gx = Gn[j][r].x, gy = Gn[j][r].y;
						gx += __shfl_xor_sync(0xffffffffu, gx, 4);
						gy += __shfl_xor_sync(0xffffffffu, gy, 4);
						gx += __shfl_xor_sync(0xffffffffu, gx, 8);
						gy += __shfl_xor_sync(0xffffffffu, gy, 8);
						if (NEG > 0 && pm2 == 0 && j < n0 &&
						    smemInBounds(smemAddr(Gw + (r * W + ph2 + 8 * j) * 2), 16u, smemAddr(Gw), smemAddr(Gw + nG),
						                 a.devErr)) {
							const int w = ph2 + 8 * j;
							Gw[(r * W + w) * 2] += (double)gx;
							Gw[(r * W + w) * 2 + 1] += (double)gy;
						}
						Gn[j][r] = make_float2(0.f, 0.f);
					}
#pragma unroll
				for (int j = 0; j < (POS > 0 ? POS : 1); ++j)
#pragma unroll
					for (int r = 0; r < R; ++r) {
						float gx = Gp[j][r].x, gy = Gp[j][r].y;
						gx += __shfl_xor_sync(0xffffffffu, gx, 4);
						gy += __shfl_xor_sync(0xffffffffu, gy, 4);
						gx += __shfl_xor_sync(0xffffffffu, gx, 8);
						gy += __shfl_xor_sync(0xffffffffu, gy, 8);
						if (POS > 0 && pm2 == 0 && j < n1 &&
						    smemInBounds(smemAddr(Gw + (r * W + wS1 + 8 * j) * 2), 16u, smemAddr(Gw), smemAddr(Gw + nG),
						                 a.devErr)) {
							const int w = wS1 + 8 * j;
							Gw[(r * W + w) * 2] += (double)gx;
							Gw[(r * W + w) * 2 + 1] += (double)gy;
						}
						Gp[j][r] = make_float2(0.f, 0.f);
					}
			}
		}
	}

	// a block that timed out anywhere flags the error and lets the last copy
	// issued into each stage land before it exits (bounded)
	if (__syncthreads_or(failed)) {
		if (tid == 0) {
			atomicOr(a.devErr, (unsigned)kDevErrTimeout);
			for (int q = 0; q < stages; ++q)
				if (issued[q] > 0u)
					mbarWaitBounded(&bars[q], (issued[q] - 1u) & 1u);
		}
	}

	// ---- epilogue: the block's partials go into the exact fixed-point
	// accumulators; the last block writes the results ----
	gridDependencyWait();
	const size_t ls = (size_t)a.nPartial;
	unsigned long long* myAcc = a.fixAcc + (blockIdx.x % kReplicas) * (size_t)kLimbs * ls;
	fdfNormTerms(a, V64, nTiles, myAcc, ls, warp, lane);
	if (lane == 0) {
		fixedAdd(myAcc + 0, ls, a.nfAcc + 0, (a.reduction == 0) ? accLL : (double)kLL - (double)kLLc);
		fixedAdd(myAcc + 1, ls, a.nfAcc + 1, (a.reduction == 0) ? accC : (double)kC - (double)kCc);
	}
	if (a.withGrad) {
		__syncthreads();
		for (int v = tid; v < nG; v += kThreads) {
			double t = 0.;
			for (int q = 0; q < kWarps; ++q)
				t += G64[(size_t)q * nG + v];
			fixedAdd(myAcc + 2 + v, ls, a.nfAcc + 2 + v, t);
		}
	}
	__shared__ unsigned sLast;
	fdfTail(a, &sLast, flatD, tid);
}

// POS = ceil(W1 / 8) waves per lane, compiled for 1..13 (W1 <= 104)
constexpr int kMaxPos = 13;

int posCount(int W1) { return (W1 + 7) / 8; }

template <int R, int NEG, int POS>
int launchFused(const FdfPlan& p, const FdfArgs& a, cudaStream_t s)
{
	auto kern = fdfFusedKernel<R, NEG, POS>;
	static size_t configured = 0;
	if (p.smemBytes > configured) {
		const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p.smemBytes);
		if (e != cudaSuccess)
			return cudaCheck(e, "cudaFuncSetAttribute(fdf fused)");
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
	return cudaCheck(e, "fdf fused kernel launch");
}

template <int R, int NEG>
int launchFusedP(const FdfPlan& p, const FdfArgs& a, cudaStream_t s)
{
	switch (posCount(a.W - a.W0)) {
	case 1: return launchFused<R, NEG, 1>(p, a, s);
	case 2: return launchFused<R, NEG, 2>(p, a, s);
	case 3: return launchFused<R, NEG, 3>(p, a, s);
	case 4: return launchFused<R, NEG, 4>(p, a, s);
	case 5: return launchFused<R, NEG, 5>(p, a, s);
	case 6: return launchFused<R, NEG, 6>(p, a, s);
	case 7: return launchFused<R, NEG, 7>(p, a, s);
	case 8: return launchFused<R, NEG, 8>(p, a, s);
	case 9: return launchFused<R, NEG, 9>(p, a, s);
	case 10: return launchFused<R, NEG, 10>(p, a, s);
	case 11: return launchFused<R, NEG, 11>(p, a, s);
	case 12: return launchFused<R, NEG, 12>(p, a, s);
	case 13: return launchFused<R, NEG, 13>(p, a, s);
	default: return setError(kErrUnsupported, "no fused FdF variant for this positive-reflectivity wave count");
	}
}

template <int R>
int launchFusedR(const FdfPlan& p, const FdfArgs& a, cudaStream_t s)
{
	switch ((a.W0 + 7) / 8) {
	case 0: return launchFusedP<R, 0>(p, a, s);
	case 1: return launchFusedP<R, 1>(p, a, s);
	case 2: return launchFusedP<R, 2>(p, a, s);
	default: return setError(kErrUnsupported, "no fused FdF variant for this negative-reflectivity wave count");
	}
}

}  // namespace

size_t fusedFdfSmem(int W0, int W, int R, int stages)
{
	if (R < 1 || R > 2 || (W0 + 7) / 8 > 2 || posCount(W - W0) < 1 || posCount(W - W0) > kMaxPos)
		return 0;
	return fusedLayout(W, R, stages).total;
}

int launchFdfFused(const FdfPlan& p, const FdfArgs& a, cudaStream_t s)
{
	if (p.E != kE)
		return setError(kErrUnsupported, "the fused FdF variant needs 128-event tiles");
	switch (a.R) {
	case 1: return launchFusedR<1>(p, a, s);
	case 2: return launchFusedR<2>(p, a, s);
	default: return setError(kErrUnsupported, "the fused FdF variant supports rank 1 and 2");
	}
}

}  // namespace pwa
