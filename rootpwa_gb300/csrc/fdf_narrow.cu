// fdf_narrow.cu -- FdF variant for small wave sets (rank x waves <= 16).
//
// Same result as fdfMainKernel (the event term of
// partialWaveFit/pwaLikelihood.cc:209-244, the normalisation and prior terms
// of :254-297 and the gradient in the layout of :1714-1731), with the work
// of a tile divided for wave sets so small that the per-tile overheads of the
// main kernel (cross-lane combination of the coherent sums, a block barrier
// and c S through shared memory per 128 events) dominate its time:
//   * a tile is four consecutive store blocks (512 events), moved by one bulk
//     copy; thread t of the block owns event t of the tile: store block
//     t / 128, position t % 128 (the row rotation of the store keeps a warp's
//     32 consecutive positions on distinct banks);
//   * the thread sums all waves of its event itself: S_{r,e} = sum_w V_rw A_w
//     with V read by broadcast from shared memory, then L, c = -2/L, -ln L;
//   * it keeps its event's amplitudes in registers and accumulates
//     G_{r,w} += c S_{r,e(w)} conj(A_w) for all slots in FP32 registers;
//   * every few tiles (the reduction mode's fold interval) a warp
//     reduce-scatter folds the 32 threads' G into one value per lane, added to
//     FP64 (or compensated / plain FP32) accumulators;
//   * no block barrier per tile: the last warp done with a stage refills it.
// The epilogue (normalisation and prior terms, exact fixed-point cross-block
// sums, the last block's tail) is the main kernel's.  Every mbarrier wait is
// bounded; on expiry the block records kDevErrTimeout, waits (bounded) for
// the copies it issued and exits with the result discarded by the host.

#include "fdf_common.cuh"

#include <algorithm>

namespace pwa {
namespace {

constexpr int kNB = 4;             // store blocks (128 events) per tile
constexpr int kNE = 128 * kNB;     // events per tile: one per thread
constexpr int kFoldNarrow = 32;    // tiles between FP32 -> FP64 folds (FP64 reduction)
static_assert(kNE == kThreads, "one event per thread");

struct NarrowLayout {
	size_t tiles, vs, v64, bars, done, issued, total;
};

__host__ __device__ inline NarrowLayout narrowLayout(int W, int R, int stages)
{
	auto up = [](size_t x) { return (x + 127) & ~(size_t)127; };
	NarrowLayout L;
	L.tiles = 0;
	L.vs = up((size_t)stages * W * kNE * 8);
	L.v64 = up(L.vs + (size_t)W * R * 8);
	L.bars = up(L.v64 + (size_t)W * R * 16);
	L.done = L.bars + (size_t)stages * 8;
	L.issued = L.done + (size_t)stages * 4;
	L.total = L.issued + (size_t)stages * 4;
	return L;
}

__device__ __forceinline__ int narrowFold(int reduction)
{
	return reduction == 0 ? kFoldNarrow : reduction == 1 ? 1 : 1 << 30;
}

// R ranks, at most WMAX waves; TWO: waves of both reflectivities (W0 > 0)
template <int R, int WMAX, bool TWO>
__global__ void __launch_bounds__(kThreads, 1) fdfNarrowKernel(const FdfArgs a, const int stages)
{
	extern __shared__ __align__(128) unsigned char smem[];
	constexpr int NV = 2 * R * WMAX;     // gradient values per thread
	constexpr int NQ = (NV + 31) / 32;  // reduce-scatter rounds
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const int W = a.W, W0 = a.W0;
	const NarrowLayout lay = narrowLayout(W, R, stages);
	float2* tiles = reinterpret_cast<float2*>(smem + lay.tiles);
	float2* Vs = reinterpret_cast<float2*>(smem + lay.vs);      // [W][R]
	double2* V64 = reinterpret_cast<double2*>(smem + lay.v64);  // [R][W]
	uint64_t* bars = reinterpret_cast<uint64_t*>(smem + lay.bars);
	unsigned* done = reinterpret_cast<unsigned*>(smem + lay.done);
	unsigned* issued = reinterpret_cast<unsigned*>(smem + lay.issued);

	const uint64_t nBlocks = (a.nEvents + 127) / 128;  // store blocks
	const uint64_t nTiles = (nBlocks + kNB - 1) / kNB;
	const uint64_t first = blockIdx.x, stride = gridDim.x;
	const uint64_t myTiles = (first < nTiles) ? (nTiles - 1 - first) / stride + 1 : 0;
	const uint32_t blockBytes = (uint32_t)W * 128u * 8u;

	// batched fits: the launch of a problem that no longer iterates does nothing
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

	// tile k (local index) into stage s: its store blocks (fewer in the last tile)
	auto issue = [&](uint64_t k, int s) {
		if (lane == 0) {
			const uint64_t b0 = (first + k * stride) * kNB;
			const uint64_t nb = nBlocks - b0 < (uint64_t)kNB ? nBlocks - b0 : (uint64_t)kNB;
			const uint32_t bytes = (uint32_t)nb * blockBytes;
			mbarArriveExpectTx(&bars[s], bytes);
			bulkCopyG2S(tiles + (size_t)s * W * kNE, a.amps + b0 * (uint64_t)W * 128, bytes, &bars[s]);
			++issued[s];
		}
	};
	// the store does not change after finishInit: the first stages load
	// while the preceding grid ends
	if (warp == 0)
		for (int s = 0; s < stages && (uint64_t)s < myTiles; ++s)
			issue((uint64_t)s, s);

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

	// this thread's event: store block jb of the tile, position pp in it; the
	// byte offset of wave w's amplitude in a stage is base + 1024 w + rot[w % 4]
	const int jb = tid >> 7, pp = tid & 127;
	const uint32_t base = (uint32_t)jb * (uint32_t)W * 1024u;
	uint32_t rot[4];
#pragma unroll
	for (int m = 0; m < 4; ++m)
		rot[m] = (uint32_t)((pp + (int)storeRot((uint32_t)m, 128u)) & 127) * 8u;
	const uint32_t vAddr = smemAddr(Vs), vHi = vAddr + (uint32_t)(W * R) * 8u;

	float2 G[R][WMAX];
#pragma unroll
	for (int r = 0; r < R; ++r)
#pragma unroll
		for (int w = 0; w < WMAX; ++w)
			G[r][w] = make_float2(0.f, 0.f);
	double accLL = 0., accC = 0.;
	float kLL = 0.f, kLLc = 0.f, kC = 0.f, kCc = 0.f;
	float llPart = 0.f, cPart = 0.f;
	double accG[NQ];
	float kG[NQ], kGc[NQ];
#pragma unroll
	for (int q = 0; q < NQ; ++q) {
		accG[q] = 0.;
		kG[q] = kGc[q] = 0.f;
	}

	bool failed = false;
	int s = 0, foldLeft = narrowFold(a.reduction);
	uint32_t parity = 0;
	uint64_t k = 0;
	for (; k < myTiles; ++k) {
		if (k != 0 && ++s == stages) {
			s = 0;
			parity ^= 1u;
		}
		if (!mbarWaitBounded(&bars[s], parity)) {
			failed = true;
			break;
		}
		const uint32_t stLo = smemAddr(tiles + (size_t)s * W * kNE), stHi = stLo + (uint32_t)W * kNE * 8u;
		const uint32_t tAddr = stLo + base;
		const uint64_t ev = (first + k * stride) * (uint64_t)kNE + (uint64_t)tid;
		if (ev < a.nEvents) {
			// coherent sums over the event's waves
			float2 A[WMAX];
			float2 S[R][2];
#pragma unroll
			for (int r = 0; r < R; ++r)
				S[r][0] = S[r][1] = make_float2(0.f, 0.f);
#pragma unroll
			for (int w = 0; w < WMAX; ++w) {
				if (w < W) {
					A[w] = lds64c(tAddr + (uint32_t)w * 1024u + rot[w & 3], stLo, stHi, a.devErr);
					const int e = (TWO && w < W0) ? 0 : 1;
#pragma unroll
					for (int r = 0; r < R; ++r) {
						const float2 v = lds64c(vAddr + (uint32_t)(w * R + r) * 8u, vAddr, vHi, a.devErr);
						if (e == 0) {
							S[r][0].x = fmaf(v.x, A[w].x, fmaf(-v.y, A[w].y, S[r][0].x));
							S[r][0].y = fmaf(v.x, A[w].y, fmaf(v.y, A[w].x, S[r][0].y));
						} else {
							S[r][1].x = fmaf(v.x, A[w].x, fmaf(-v.y, A[w].y, S[r][1].x));
							S[r][1].y = fmaf(v.x, A[w].y, fmaf(v.y, A[w].x, S[r][1].y));
						}
					}
				}
			}
			float L = flat2;
#pragma unroll
			for (int r = 0; r < R; ++r)
#pragma unroll
				for (int e = 0; e < 2; ++e)
					L = fmaf(S[r][e].x, S[r][e].x, fmaf(S[r][e].y, S[r][e].y, L));
			const float c = eventWeight(L);
			llPart += -eventLog(L);
			cPart += c;
			if (a.withGrad) {
				// G += c S conj(A): (ax tx + ay ty, ax ty - ay tx)
#pragma unroll
				for (int w = 0; w < WMAX; ++w) {
					if (w < W) {
						const bool neg = TWO && w < W0;
#pragma unroll
						for (int r = 0; r < R; ++r) {
							// a select, not a runtime index (which would put S in local memory)
							const float2 Se = neg ? S[r][0] : S[r][1];
							const float tx = c * Se.x, ty = c * Se.y;
							G[r][w].x = fmaf(A[w].x, tx, fmaf(A[w].y, ty, G[r][w].x));
							G[r][w].y = fmaf(A[w].x, ty, fmaf(-A[w].y, tx, G[r][w].y));
						}
					}
				}
			}
		}

		// stage s is no longer read by this warp; the last warp refills it
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

		// fold the FP32 partials
		if (--foldLeft == 0 || k + 1 == myTiles) {
			foldLeft = narrowFold(a.reduction);
			const float ll = warpSum(llPart), cs = warpSum(cPart);
			llPart = cPart = 0.f;
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
				float part[NQ * 32];
#pragma unroll
				for (int r = 0; r < R; ++r)
#pragma unroll
					for (int w = 0; w < WMAX; ++w) {
						part[(r * WMAX + w) * 2] = G[r][w].x;
						part[(r * WMAX + w) * 2 + 1] = G[r][w].y;
						G[r][w] = make_float2(0.f, 0.f);
					}
#pragma unroll
				for (int v = NV; v < NQ * 32; ++v)
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

	// a block that timed out flags the error and lets the copies it issued
	// land before it exits (bounded)
	if (__syncthreads_or(failed)) {
		if (tid == 0) {
			atomicOr(a.devErr, (unsigned)kDevErrTimeout);
			for (int q = 0; q < stages; ++q)
				if (issued[q] > 0u)
					mbarWaitBounded(&bars[q], (issued[q] - 1u) & 1u);
		}
	}

	// ---- epilogue: exact fixed-point sums; the last block writes the results ----
	gridDependencyWait();
	const size_t ls = (size_t)a.nPartial;
	unsigned long long* myAcc = a.fixAcc + (blockIdx.x % kReplicas) * (size_t)kLimbs * ls;
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
				const int sw = vi >> 1, comp = vi & 1;
				const int r = sw / WMAX, w = sw - r * WMAX;
				if (w < W) {
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

template <int R, int WMAX, bool TWO>
int launchNarrowVariant(const FdfPlan& p, const FdfArgs& a, cudaStream_t s)
{
	auto kern = fdfNarrowKernel<R, WMAX, TWO>;
	static size_t configured = 0;
	if (p.smemBytes > configured) {
		const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p.smemBytes);
		if (e != cudaSuccess)
			return cudaCheck(e, "cudaFuncSetAttribute(fdf narrow)");
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
	return cudaCheck(e, "fdf narrow kernel launch");
}

}  // namespace

// largest wave count of the narrow variant for a rank (0: none)
int narrowMaxWaves(int R) { return R == 1 ? 16 : (R == 2 ? 8 : 0); }

size_t narrowFdfSmem(int W, int R, int stages)
{
	if (W < 1 || W > narrowMaxWaves(R))
		return 0;
	return narrowLayout(W, R, stages).total;
}

uint64_t narrowFdfTiles(uint64_t nEvents) { return ((nEvents + 127) / 128 + kNB - 1) / kNB; }

int launchFdfNarrow(const FdfPlan& p, const FdfArgs& a, cudaStream_t s)
{
	if (p.E != 128 || a.W > narrowMaxWaves(a.R))
		return setError(kErrUnsupported, "the narrow FdF variant needs 128-event store blocks and R x W <= 16");
	const bool two = a.W0 > 0;
	if (a.R == 1)
		return two ? launchNarrowVariant<1, 16, true>(p, a, s) : launchNarrowVariant<1, 16, false>(p, a, s);
	if (a.R == 2)
		return two ? launchNarrowVariant<2, 8, true>(p, a, s) : launchNarrowVariant<2, 8, false>(p, a, s);
	return setError(kErrUnsupported, "the narrow FdF variant supports rank 1 and 2");
}

}  // namespace pwa
