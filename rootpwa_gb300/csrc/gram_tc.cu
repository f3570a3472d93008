// gram_tc.cu -- tcgen05 tensor-core Gram kernel for the integral matrices.
//
// Computes the raw sums of ampIntegralMatrix::integrate
// (decayAmplitude/ampIntegralMatrix.cc:408-469)
//   I_ij = sum_k w_k A_{i,k} conj(A_{j,k})
// from real products of the planar parts Ar = Re A, Ai = Im A (one column per
// event k):
//   Re I = Ar Ar^T + Ai Ai^T,   Im I = D - D^T with D = Ai Ar^T.
// Weights enter as sqrt(w_k) on both sides (the host passes w_k >= 0).
//
// One persistent CTA per SM owns a contiguous range of events.  Per tile of
// 32 events (64 for BF16):
//   - one TMA load brings the complex64 rows [W][32] (interleaved re, im)
//     into a raw shared-memory stage (warp 8);
//   - eight converter warps split re / im into planar operands in the
//     canonical K-major 128-byte-swizzled layout (TF32: one plane rounded to
//     TF32; TF32x3: hi = tf32(x), lo = tf32(x - hi); BF16x3: the same with
//     bf16), weighted;
//   - one thread of warp 9 issues tcgen05.mma (M = 128, K = 32 bytes per
//     instruction) into FP32 accumulators in tensor memory;
//   - drain warps move the accumulators into round-to-nearest FP32 sums.
// The tensor cores add into FP32 accumulators with truncation, so a long
// chain of accumulations drifts towards zero by a fraction of an ulp per
// instruction; the accumulators therefore start from zero every `period`
// tiles and are drained.  A tcgen05.mma of M = 128 takes about the same time
// for any N up to 96, so the instruction count sets the speed.  Three kernels:
//   * hi/lo precisions up to 96 waves (gramTcHiLoKernel, described at the
//     kernel): the planes side by side so that one instruction multiplies a
//     plane by two (N = 2W), 16 instructions per tile instead of 36, the
//     symmetric products assembled from one orientation;
//   * TF32 up to 96 waves (gramTcKernel<true>): Ar Ar^T + Ai Ai^T and
//     Ai Ar^T into two working pairs (Re, D) in tensor memory, 4N <= 384
//     columns; the MMAs of period p go to pair p % 2 while sixteen drain
//     warps (10..25, four per lane quarter) add pair (p - 1) % 2 into sums
//     they keep in registers;
//   * wider sets (gramTcKernel<false>): one working pair, sums in tensor
//     memory (4N <= 512 columns), four drain warps (10..13); the MMA warp
//     waits for each drain before the next period.
// At the end the drain warps store the CTA's FP32 partials; a second kernel
// sums the partials of all CTAs in FP64 in a fixed order and assembles the
// Hermitian matrix.
//
// Every wait on an mbarrier is bounded (1 s of globaltimer): on expiry the
// CTA records kDevErrTimeout, stops issuing work, waits (bounded) for its own
// TMA copies and MMAs in flight and frees its tensor memory before it exits.

#include "pwa_internal.h"
#include "tcgen05.cuh"

#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <mutex>

namespace pwa {
namespace {

#define PWA_CHECK_RET(expr)     \
	do {                        \
		const int _st = (expr); \
		if (_st != kOk)         \
			return _st;         \
	} while (0)

constexpr int kKT = 32;                   // events per tile (128-byte swizzle row of TF32)
constexpr int kKTB = 64;                  // events per tile of the BF16 variant (128-byte row of BF16)
constexpr int kConvWarps = 8;             // converter warps 0..7
constexpr int kTmaWarp = kConvWarps;      // warp 8
constexpr int kMmaWarp = kConvWarps + 1;  // warp 9
constexpr int kDrainWarp0 = kConvWarps + 2;  // first drain warp (10..13, or 10..25 double-buffered)
constexpr int kThreadsTc = (kConvWarps + 6) * 32;
// double-buffered kernel: sixteen drain warps (10..25, four per lane
// quarter), sums in registers
constexpr int kDrainWarpsDB = 16;
constexpr int kThreadsDB = (kConvWarps + 2 + kDrainWarpsDB) * 32;
constexpr int kMaxNDB = 96;          // 2N / 8 = 24 chunks of 8 columns, 6 per drain warp
constexpr int kChunksPerWarpDB = 6;
constexpr int kOpBufs = 2;
constexpr int kTmemCols = 512;
constexpr uint32_t kPlaneBytes = 256u * 128u;  // Ar rows 0..127, Ai rows 128..255

struct TcArgs {
	uint64_t K;         // events (columns)
	int W;              // waves (<= 128)
	int N;              // MMA N: W rounded up to 16
	int planes;         // 1 (TF32) or 2 (TF32x3, BF16x3: hi, lo)
	int bf16;           // BF16 operands (kind::f16), 64-event tiles
	int kt;             // events per tile: kKT or kKTB
	int stages;         // raw TMA stages
	int period;         // tiles between drains of the accumulators
	int groups;         // 1, or 2 row groups of W / 2 rows loaded by one 3-D TMA copy
	uint64_t tilesTotal;
	const double* weightK;  // per event, or null
	float* partials;        // [grid][2 (Re, D)][128][N]
	unsigned* devErr;
};

template <bool DB>
__global__ void __launch_bounds__(DB ? kThreadsDB : kThreadsTc, 1)
    gramTcKernel(const __grid_constant__ CUtensorMap map, const TcArgs a)
{
	extern __shared__ __align__(1024) unsigned char smemRaw[];
	unsigned char* smem =
	    reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smemRaw) + 1023) & ~uintptr_t(1023));
	const int W = a.W, N = a.N;
	const uint32_t rawBytes = (uint32_t)W * (uint32_t)a.kt * 8u;
	const uint32_t rawStride = (rawBytes + 1023u) & ~1023u;
	unsigned char* ops = smem;                                            // [kOpBufs][planes][256 rows x 128 B]
	unsigned char* raw = ops + (size_t)kOpBufs * a.planes * kPlaneBytes;  // [stages][W][64 floats]
	uint64_t* bars = reinterpret_cast<uint64_t*>(raw + (size_t)a.stages * rawStride);
	uint64_t* rawFull = bars;
	uint64_t* rawEmpty = bars + a.stages;
	uint64_t* opFull = bars + 2 * a.stages;
	uint64_t* opEmpty = opFull + kOpBufs;
	uint64_t* drainReady = opEmpty + kOpBufs;  // [2]: a working pair complete for a drain
	uint64_t* drainDone = drainReady + 2;      // [2]: a working pair read by the drain
	uint64_t* mmaFinal = drainDone + 2;
	uint32_t* tmemHolder = reinterpret_cast<uint32_t*>(mmaFinal + 1);
	__shared__ unsigned sFail;

	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const uint64_t t0 = (uint64_t)blockIdx.x * a.tilesTotal / gridDim.x;
	const uint64_t t1 = (uint64_t)(blockIdx.x + 1) * a.tilesTotal / gridDim.x;
	const int nT = (int)(t1 - t0);
	const int nDrains = (nT + a.period - 1) / a.period;

	if (tid == 0) {
		for (int s = 0; s < a.stages; ++s) {
			barInit(&rawFull[s], 1);
			barInit(&rawEmpty[s], kConvWarps);
		}
		for (int b = 0; b < kOpBufs; ++b) {
			barInit(&opFull[b], kConvWarps);
			barInit(&opEmpty[b], 1);
		}
		for (int x = 0; x < 2; ++x) {
			barInit(&drainReady[x], 1);
			barInit(&drainDone[x], DB ? kDrainWarpsDB : 4);
		}
		barInit(mmaFinal, 1);
		sFail = 0u;
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	if (warp == kMmaWarp) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sAddr(tmemHolder)),
		             "r"(kTmemCols)
		             : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
	}
	// rows W..127 (Ar) and 128+W..255 (Ai) of every operand plane stay zero
	if (warp < kConvWarps) {
		const int padWords = (128 - W) * 32;
		for (int b = 0; b < kOpBufs * a.planes; ++b)
			for (int h = 0; h < 2; ++h) {
				uint32_t* p = reinterpret_cast<uint32_t*>(ops + (size_t)b * kPlaneBytes + (size_t)(h * 128 + W) * 128);
				for (int i = tid; i < padWords; i += kConvWarps * 32)
					p[i] = 0u;
			}
		asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
	}
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
	__syncthreads();
	asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
	const uint32_t tmem = *tmemHolder;
	// tensor-memory columns: working Re [0, N), D [N, 2N); sums Re [2N, 3N), D [3N, 4N)

	if (warp == kTmaWarp) {
		// ---- producer: one TMA load per tile ----
		if (lane == 0) {
			asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&map)) : "memory");
			int issued = 0;
			for (int t = 0; t < nT; ++t) {
				const int s = t % a.stages;
				if (t >= a.stages && !barWait(&rawEmpty[s], (uint32_t)(((t / a.stages) - 1) & 1))) {
					atomicOr(a.devErr, (unsigned)kDevErrTimeout);
					sFail = 1u;
					break;
				}
				if (*(volatile unsigned*)&sFail)
					break;
				barExpectTx(&rawFull[s], rawBytes);
				if (a.groups == 2)
					tmaLoad3d(raw + (size_t)s * rawStride, &map, (int)(2 * (t0 + t) * (uint64_t)a.kt), 0, 0, &rawFull[s]);
				else
					tmaLoad2d(raw + (size_t)s * rawStride, &map, (int)(2 * (t0 + t) * (uint64_t)a.kt), 0, &rawFull[s]);
				++issued;
			}
			// the copies of this CTA land before it exits
			for (int t = (issued > a.stages ? issued - a.stages : 0); t < issued; ++t)
				barWait(&rawFull[t % a.stages], (uint32_t)((t / a.stages) & 1));
		}
	} else if (warp == kMmaWarp) {
		// ---- MMA issuer ----
		if (lane == 0) {
			const uint32_t idesc = a.bf16 ? idescBf16(128, N) : idescTf32(128, N);
			const uint32_t opBase = sAddr(ops);
			bool freshRe = true, freshD = true;
			// one product over the tile: acc += A B^T, 4 instructions of 32
			// bytes of K (8 TF32 or 16 BF16 elements)
			auto product = [&](uint32_t acc, bool& fresh, uint32_t aOp, uint32_t bOp) {
				for (int kk = 0; kk < 4; ++kk) {
					if (a.bf16)
						mmaBf16(acc, smemDesc(aOp + (uint32_t)kk * 32u), smemDesc(bOp + (uint32_t)kk * 32u), idesc,
						        fresh ? 0u : 1u);
					else
						mmaTf32(acc, smemDesc(aOp + (uint32_t)kk * 32u), smemDesc(bOp + (uint32_t)kk * 32u), idesc,
						        fresh ? 0u : 1u);
					fresh = false;
				}
			};
			for (int t = 0; t < nT; ++t) {
				const int b = t % kOpBufs;
				// working pair of this period (double-buffered: period p uses pair p % 2)
				const int p = t / a.period, x = DB ? (p & 1) : 0;
				const uint32_t accRe = tmem + (uint32_t)(x * 2 * N), accD = accRe + (uint32_t)N;
				if (t % a.period == 0 && p >= (DB ? 2 : 1)) {
					// the drain of the last period that used this pair has read it
					const uint32_t k = DB ? (uint32_t)(p / 2 - 1) : (uint32_t)(p - 1);
					if (!barWait(&drainDone[x], k & 1u)) {
						atomicOr(a.devErr, (unsigned)kDevErrTimeout);
						sFail = 1u;
						break;
					}
					asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
				}
				if (t % a.period == 0)
					freshRe = freshD = true;
				if (!barWait(&opFull[b], (uint32_t)((t / kOpBufs) & 1))) {
					atomicOr(a.devErr, (unsigned)kDevErrTimeout);
					sFail = 1u;
					break;
				}
				asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
				const uint32_t hi = opBase + (uint32_t)b * a.planes * kPlaneBytes;
				const uint32_t arH = hi, aiH = hi + 16384u;
				if (a.planes == 2) {
					const uint32_t arL = hi + kPlaneBytes, aiL = arL + 16384u;
					product(accRe, freshRe, arH, arL);
					product(accRe, freshRe, arL, arH);
					product(accRe, freshRe, aiH, aiL);
					product(accRe, freshRe, aiL, aiH);
					product(accD, freshD, aiH, arL);
					product(accD, freshD, aiL, arH);
				}
				product(accRe, freshRe, arH, arH);
				product(accRe, freshRe, aiH, aiH);
				product(accD, freshD, aiH, arH);
				mmaCommit(&opEmpty[b]);
				if ((t + 1) % a.period == 0 || t + 1 == nT)
					mmaCommit(&drainReady[x]);
			}
			// all MMAs of this CTA complete before tensor memory is freed
			mmaCommit(mmaFinal);
			if (!barWait(mmaFinal, 0u))
				atomicOr(a.devErr, (unsigned)kDevErrTimeout);
		}
	} else if (DB && warp >= kDrainWarp0) {
		// ---- drain, double-buffered: register sums += working pair d % 2 ----
		// warp w reaches tensor-memory lanes 32 (w % 4) ..; the four drain
		// warps of a lane quarter take every fourth 8-column chunk of the pair
		const int q = warp & 3, sub = (warp - kDrainWarp0) >> 2;
		const uint32_t rowBase = tmem + ((uint32_t)(q * 32) << 16);
		const int nch = 2 * N / 8;  // chunks of a working pair (Re then D)
		float acc[kChunksPerWarpDB][8];
#pragma unroll
		for (int j = 0; j < kChunksPerWarpDB; ++j)
#pragma unroll
			for (int i = 0; i < 8; ++i)
				acc[j][i] = 0.f;
		bool ok = true;
		for (int d = 0; d < nDrains; ++d) {
			const int x = d & 1;
			if (!barWait(&drainReady[x], (uint32_t)((d >> 1) & 1))) {
				atomicOr(a.devErr, (unsigned)kDevErrTimeout);
				ok = false;
				break;
			}
			asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
			const uint32_t pair = rowBase + (uint32_t)(x * 2 * N);
#pragma unroll
			for (int j = 0; j < kChunksPerWarpDB; ++j) {
				const int c = sub + 4 * j;
				if (c < nch) {
					uint32_t w[8];
					tmemLd8(pair + (uint32_t)(8 * c), w);
					asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
					for (int i = 0; i < 8; ++i)
						acc[j][i] += __uint_as_float(w[i]);
				}
			}
			asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
			__syncwarp();
			if (lane == 0)
				barArrive(&drainDone[x]);
		}
		if (ok) {
			// partials of this CTA: [2][128][N], rows < W
			const int row = q * 32 + lane;
			if (row < W) {
#pragma unroll
				for (int j = 0; j < kChunksPerWarpDB; ++j) {
					const int c = sub + 4 * j;
					if (c < nch) {
						const int part = (8 * c) / N, col = 8 * c - part * N;
						float4* d4 = reinterpret_cast<float4*>(
						    a.partials + (((size_t)blockIdx.x * 2 + part) * 128 + row) * N + col);
						d4[0] = make_float4(acc[j][0], acc[j][1], acc[j][2], acc[j][3]);
						d4[1] = make_float4(acc[j][4], acc[j][5], acc[j][6], acc[j][7]);
					}
				}
			}
		}
	} else if (!DB && warp >= kDrainWarp0) {
		// ---- drain, single-buffered: sums += working accumulators (round to nearest) ----
		const int q = warp & 3;  // lane quarter of tensor memory
		const uint32_t rowBase = tmem + ((uint32_t)(q * 32) << 16);
		bool ok = true;
		for (int d = 0; d < nDrains; ++d) {
			if (!barWait(&drainReady[0], (uint32_t)(d & 1))) {
				atomicOr(a.devErr, (unsigned)kDevErrTimeout);
				ok = false;
				break;
			}
			asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
			for (int c = 0; c < 2 * N; c += 16) {
				uint32_t w[16], s[16];
				tmemLd16(rowBase + (uint32_t)c, w);
				if (d > 0)
					tmemLd16(rowBase + (uint32_t)(2 * N + c), s);
				asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
				if (d > 0)
#pragma unroll
					for (int i = 0; i < 16; ++i)
						w[i] = __float_as_uint(__uint_as_float(w[i]) + __uint_as_float(s[i]));
				tmemSt16(rowBase + (uint32_t)(2 * N + c), w);
			}
			asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
			asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
			__syncwarp();
			if (lane == 0)
				barArrive(&drainDone[0]);
		}
		if (ok) {
			// partials of this CTA: [2][128][N], rows < W
			const int row = q * 32 + lane;
			for (int c = 0; c < 2 * N; c += 16) {
				uint32_t r[16];
				tmemLd16(rowBase + (uint32_t)(2 * N + c), r);
				asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
				if (row < W) {
					const int part = c / N, col = c - part * N;
					float4* d4 = reinterpret_cast<float4*>(
					    a.partials + (((size_t)blockIdx.x * 2 + part) * 128 + row) * N + col);
#pragma unroll
					for (int i = 0; i < 4; ++i)
						d4[i] = make_float4(__uint_as_float(r[4 * i]), __uint_as_float(r[4 * i + 1]),
						                    __uint_as_float(r[4 * i + 2]), __uint_as_float(r[4 * i + 3]));
				}
			}
		}
	} else {
		// ---- converters: raw interleaved rows -> planar swizzled operand ----
		const int sub = lane >> 4, p = lane & 15;  // wave of the pair, event pair
		for (int t = 0; t < nT; ++t) {
			const int s = t % a.stages, b = t % kOpBufs;
			if (!barWait(&rawFull[s], (uint32_t)((t / a.stages) & 1)) ||
			    (t >= kOpBufs && !barWait(&opEmpty[b], (uint32_t)(((t / kOpBufs) - 1) & 1)))) {
				atomicOr(a.devErr, (unsigned)kDevErrTimeout);
				sFail = 1u;
				break;
			}
			const float* rs = reinterpret_cast<const float*>(raw + (size_t)s * rawStride);
			unsigned char* hiP = ops + (size_t)b * a.planes * kPlaneBytes;
			unsigned char* loP = hiP + kPlaneBytes;
			if (a.bf16) {
				// four events per lane: raw row of 64 (re, im) pairs -> BF16 hi, lo
				const uint64_t kb = (t0 + t) * (uint64_t)kKTB + 4u * p;
				float wq[4] = {1.f, 1.f, 1.f, 1.f};
				if (a.weightK)
#pragma unroll
					for (int q = 0; q < 4; ++q)
						wq[q] = (kb + q < a.K) ? sqrtf((float)a.weightK[kb + q]) : 0.f;
				for (int w = 2 * warp + sub; w < W; w += 2 * kConvWarps) {
					const float4 v0 = *reinterpret_cast<const float4*>(rs + w * 128 + 8 * p);
					const float4 v1 = *reinterpret_cast<const float4*>(rs + w * 128 + 8 * p + 4);
					const float re[4] = {v0.x * wq[0], v0.z * wq[1], v1.x * wq[2], v1.z * wq[3]};
					const float im[4] = {v0.y * wq[0], v0.w * wq[1], v1.y * wq[2], v1.w * wq[3]};
					uint32_t hr[4], hm[4], lr[4], lm[4];
#pragma unroll
					for (int q = 0; q < 4; ++q) {
						float br, bm, dummy;
						hr[q] = bf16Bits(re[q], &br);
						hm[q] = bf16Bits(im[q], &bm);
						lr[q] = bf16Bits(re[q] - br, &dummy);
						lm[q] = bf16Bits(im[q] - bm, &dummy);
					}
					const uint32_t oRe = swzOffset16(w, 4 * p), oIm = swzOffset16(128 + w, 4 * p);
					*reinterpret_cast<uint2*>(hiP + oRe) = make_uint2(hr[0] | (hr[1] << 16), hr[2] | (hr[3] << 16));
					*reinterpret_cast<uint2*>(hiP + oIm) = make_uint2(hm[0] | (hm[1] << 16), hm[2] | (hm[3] << 16));
					*reinterpret_cast<uint2*>(loP + oRe) = make_uint2(lr[0] | (lr[1] << 16), lr[2] | (lr[3] << 16));
					*reinterpret_cast<uint2*>(loP + oIm) = make_uint2(lm[0] | (lm[1] << 16), lm[2] | (lm[3] << 16));
				}
				asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
				__syncwarp();
				if (lane == 0) {
					barArrive(&rawEmpty[s]);
					barArrive(&opFull[b]);
				}
				continue;
			}
			const uint64_t k0 = (t0 + t) * (uint64_t)kKT + 2u * p;
			float w0 = 1.f, w1 = 1.f;
			if (a.weightK) {
				w0 = (k0 < a.K) ? sqrtf((float)a.weightK[k0]) : 0.f;
				w1 = (k0 + 1 < a.K) ? sqrtf((float)a.weightK[k0 + 1]) : 0.f;
			}
			for (int w = 2 * warp + sub; w < W; w += 2 * kConvWarps) {
				const float4 v = *reinterpret_cast<const float4*>(rs + w * 64 + 4 * p);
				const float re0 = v.x * w0, im0 = v.y * w0, re1 = v.z * w1, im1 = v.w * w1;
				const uint32_t oRe = swzOffset(w, 2 * p), oIm = swzOffset(128 + w, 2 * p);
				const float2 hre = make_float2(tf32Round(re0), tf32Round(re1));
				const float2 him = make_float2(tf32Round(im0), tf32Round(im1));
				*reinterpret_cast<float2*>(hiP + oRe) = hre;
				*reinterpret_cast<float2*>(hiP + oIm) = him;
				if (a.planes == 2) {
					*reinterpret_cast<float2*>(loP + oRe) =
					    make_float2(tf32Round(re0 - hre.x), tf32Round(re1 - hre.y));
					*reinterpret_cast<float2*>(loP + oIm) =
					    make_float2(tf32Round(im0 - him.x), tf32Round(im1 - him.y));
				}
			}
			asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
			__syncwarp();
			if (lane == 0) {
				barArrive(&rawEmpty[s]);
				barArrive(&opFull[b]);
			}
		}
	}
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
	__syncthreads();
	if (warp == kMmaWarp) {
		asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
	}
}

// ---- hi/lo kernel (TF32x3, BF16x3; N <= 96): wide products ----
// A tcgen05.mma of M = 128 costs about the same time for every N up to 96,
// so the products are made as wide as the operand layout allows.  The four
// planes of a tile sit one after another in one operand buffer, NB = N rows
// each: Ar_hi at row 0, Ar_lo at NB, Ai_lo at 2NB, Ai_hi at 3NB (plus 32
// rows of slack, so that an A operand of 128 rows starting at Ai_hi stays
// inside; the rows of A beyond NB produce accumulator lanes >= W that are
// never read).  Per K step four instructions:
//   [Hr | C]     += Ar_hi [Ar_hi; Ar_lo]^T      (N = 2NB)
//   [C | Hi]     += Ai_hi [Ai_lo; Ai_hi]^T      (N = 2NB)
//   [Dh | E]     += Ai_hi [Ar_hi; Ar_lo]^T      (N = 2NB)
//   E            += Ai_lo Ar_hi^T               (N = NB)
// in the tensor-memory blocks Hr, C, Hi (columns [0, 3NB)) and Dh, E
// ([3NB, 5NB)).  The three-product sums follow from symmetry: Re = Hr + Hi
// + C + C^T = (S + S^T) / 2 with S = Hr + Hi + 2C, and Im = D - D^T with
// D = Dh + E.  The drain warps keep S and D in registers (2N sums per row),
// the reduction kernel symmetrises.  The blocks collect `period` tiles
// between drains; the tensor cores add into them with truncation, so each
// block of large values (Hr, Hi, Dh) gets only four additions per tile.  At
// the first tile of a period the second instruction is issued as two of
// N = NB, so that Hi starts from zero while C keeps the first one's
// products.  The first three blocks (X) are drained while the MMAs of the
// last two (Y) run, and Y while the next tile's MMAs of X run.
constexpr int kDrainWarpsHL = 16;
constexpr int kThreadsHL = (kConvWarps + 2 + kDrainWarpsHL) * 32;
constexpr int kChunksPerWarpHL = 3;  // NB / 8 <= 12 chunks of a block, every fourth per drain warp

__host__ __device__ constexpr uint32_t hlOpBytes(int NB) { return (uint32_t)(3 * NB + 128) * 128u; }

// one MMA of the operand type of the kernel (descriptors precomputed)
template <bool BF16>
__device__ __forceinline__ void mmaOp(uint32_t d, uint64_t aDesc, uint64_t bDesc, uint32_t idesc, uint32_t acc)
{
	if (BF16)
		mmaBf16(d, aDesc, bDesc, idesc, acc);
	else
		mmaTf32(d, aDesc, bDesc, idesc, acc);
}

template <bool BF16>
__global__ void __launch_bounds__(kThreadsHL, 1) gramTcHiLoKernel(const __grid_constant__ CUtensorMap map, const TcArgs a)
{
	extern __shared__ __align__(1024) unsigned char smemRaw[];
	unsigned char* smem =
	    reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smemRaw) + 1023) & ~uintptr_t(1023));
	const int W = a.W, NB = a.N;
	const uint32_t rawBytes = (uint32_t)W * (uint32_t)a.kt * 8u;
	const uint32_t rawStride = (rawBytes + 1023u) & ~1023u;
	const uint32_t opBytes = hlOpBytes(NB);
	unsigned char* ops = smem;                                   // [kOpBufs][3NB + 128 rows x 128 B]
	unsigned char* raw = ops + (size_t)kOpBufs * opBytes;        // [stages][W][kt complex]
	uint64_t* bars = reinterpret_cast<uint64_t*>(raw + (size_t)a.stages * rawStride);
	uint64_t* rawFull = bars;
	uint64_t* rawEmpty = bars + a.stages;
	uint64_t* opFull = bars + 2 * a.stages;
	uint64_t* opEmpty = opFull + kOpBufs;
	uint64_t* drainReady = opEmpty + kOpBufs;  // [2]: X, Y complete for a drain
	uint64_t* drainDone = drainReady + 2;      // [2]: X, Y read by the drain
	uint64_t* mmaFinal = drainDone + 2;
	uint32_t* tmemHolder = reinterpret_cast<uint32_t*>(mmaFinal + 1);
	__shared__ unsigned sFail;

	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const uint64_t t0 = (uint64_t)blockIdx.x * a.tilesTotal / gridDim.x;
	const uint64_t t1 = (uint64_t)(blockIdx.x + 1) * a.tilesTotal / gridDim.x;
	const int nT = (int)(t1 - t0);
	const int nDrains = (nT + a.period - 1) / a.period;

	if (tid == 0) {
		for (int s = 0; s < a.stages; ++s) {
			barInit(&rawFull[s], 1);
			barInit(&rawEmpty[s], kConvWarps);
		}
		for (int b = 0; b < kOpBufs; ++b) {
			barInit(&opFull[b], kConvWarps);
			barInit(&opEmpty[b], 1);
		}
		for (int x = 0; x < 2; ++x) {
			barInit(&drainReady[x], 1);
			barInit(&drainDone[x], kDrainWarpsHL);
		}
		barInit(mmaFinal, 1);
		sFail = 0u;
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	if (warp == kMmaWarp) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sAddr(tmemHolder)),
		             "r"(kTmemCols)
		             : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
	}
	// the operand buffers start at zero: rows W..NB-1 of every plane and the
	// slack rows are never written
	if (warp < kConvWarps) {
		uint4* p = reinterpret_cast<uint4*>(ops);
		const int n16 = (int)(kOpBufs * opBytes / 16u);
		for (int i = tid; i < n16; i += kConvWarps * 32)
			p[i] = make_uint4(0u, 0u, 0u, 0u);
		asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
	}
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
	__syncthreads();
	asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
	const uint32_t tmem = *tmemHolder;

	if (warp == kTmaWarp) {
		// ---- producer: one TMA load per tile ----
		if (lane == 0) {
			asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&map)) : "memory");
			int issued = 0;
			for (int t = 0; t < nT; ++t) {
				const int s = t % a.stages;
				if (t >= a.stages && !barWait(&rawEmpty[s], (uint32_t)(((t / a.stages) - 1) & 1))) {
					atomicOr(a.devErr, (unsigned)kDevErrTimeout);
					sFail = 1u;
					break;
				}
				if (*(volatile unsigned*)&sFail)
					break;
				barExpectTx(&rawFull[s], rawBytes);
				if (a.groups == 2)
					tmaLoad3d(raw + (size_t)s * rawStride, &map, (int)(2 * (t0 + t) * (uint64_t)a.kt), 0, 0, &rawFull[s]);
				else
					tmaLoad2d(raw + (size_t)s * rawStride, &map, (int)(2 * (t0 + t) * (uint64_t)a.kt), 0, &rawFull[s]);
				++issued;
			}
			for (int t = (issued > a.stages ? issued - a.stages : 0); t < issued; ++t)
				barWait(&rawFull[t % a.stages], (uint32_t)((t / a.stages) & 1));
		}
	} else if (warp == kMmaWarp) {
		// ---- MMA issuer ----
		if (lane == 0) {
			const uint32_t id2 = BF16 ? idescBf16(128, 2 * NB) : idescTf32(128, 2 * NB);
			const uint32_t id1 = BF16 ? idescBf16(128, NB) : idescTf32(128, NB);
			const uint32_t tX = tmem, tY = tmem + (uint32_t)(3 * NB);
			// descriptors of the planes of buffer 0; a plane is NB x 128 B (NB * 8
			// in the descriptor's 16-byte address units), a buffer opBytes, a K
			// step of 32 bytes 2 units
			const uint64_t desc0 = smemDesc(sAddr(ops));
			const uint64_t planeD = (uint64_t)NB * 8u, bufD = (uint64_t)(opBytes >> 4);
			for (int t = 0; t < nT; ++t) {
				const int b = t % kOpBufs;
				const int p = t / a.period;
				const bool first = (t % a.period) == 0;
				const bool last = (t + 1) % a.period == 0 || t + 1 == nT;
				if (!barWait(&opFull[b], (uint32_t)((t / kOpBufs) & 1))) {
					atomicOr(a.devErr, (unsigned)kDevErrTimeout);
					sFail = 1u;
					break;
				}
				asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
				const uint64_t rh = desc0 + (uint64_t)b * bufD, il = rh + 2 * planeD, ih = rh + 3 * planeD;
				// X: the drain of the last period has read it
				if (first && p >= 1) {
					if (!barWait(&drainDone[0], (uint32_t)((p - 1) & 1))) {
						atomicOr(a.devErr, (unsigned)kDevErrTimeout);
						sFail = 1u;
						break;
					}
					asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
				}
#pragma unroll
				for (uint32_t kk = 0; kk < 4; ++kk)
					mmaOp<BF16>(tX, rh + 2 * kk, rh + 2 * kk, id2, (first && kk == 0) ? 0u : 1u);
				if (first) {
#pragma unroll
					for (uint32_t kk = 0; kk < 4; ++kk) {
						mmaOp<BF16>(tX + (uint32_t)NB, ih + 2 * kk, il + 2 * kk, id1, 1u);
						mmaOp<BF16>(tX + (uint32_t)(2 * NB), ih + 2 * kk, ih + 2 * kk, id1, kk == 0 ? 0u : 1u);
					}
				} else {
#pragma unroll
					for (uint32_t kk = 0; kk < 4; ++kk)
						mmaOp<BF16>(tX + (uint32_t)NB, ih + 2 * kk, il + 2 * kk, id2, 1u);
				}
				if (last)
					mmaCommit(&drainReady[0]);
				if (first && p >= 1) {
					if (!barWait(&drainDone[1], (uint32_t)((p - 1) & 1))) {
						atomicOr(a.devErr, (unsigned)kDevErrTimeout);
						sFail = 1u;
						break;
					}
					asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
				}
#pragma unroll
				for (uint32_t kk = 0; kk < 4; ++kk)
					mmaOp<BF16>(tY, ih + 2 * kk, rh + 2 * kk, id2, (first && kk == 0) ? 0u : 1u);
#pragma unroll
				for (uint32_t kk = 0; kk < 4; ++kk)
					mmaOp<BF16>(tY + (uint32_t)NB, il + 2 * kk, rh + 2 * kk, id1, 1u);
				mmaCommit(&opEmpty[b]);
				if (last)
					mmaCommit(&drainReady[1]);
			}
			mmaCommit(mmaFinal);
			if (!barWait(mmaFinal, 0u))
				atomicOr(a.devErr, (unsigned)kDevErrTimeout);
		}
	} else if (warp >= kDrainWarp0) {
		// ---- drain: S += Hr + Hi + 2 C, D += Dh + E ----
		const int q = warp & 3, sub = (warp - kDrainWarp0) >> 2;
		const uint32_t rowBase = tmem + ((uint32_t)(q * 32) << 16);
		const int nc = NB / 8;
		float S[kChunksPerWarpHL][8], D[kChunksPerWarpHL][8];
#pragma unroll
		for (int j = 0; j < kChunksPerWarpHL; ++j)
#pragma unroll
			for (int i = 0; i < 8; ++i)
				S[j][i] = D[j][i] = 0.f;
		bool ok = true;
		for (int d = 0; d < nDrains && ok; ++d) {
#pragma unroll
			for (int x = 0; x < 2; ++x) {
				if (!barWait(&drainReady[x], (uint32_t)(d & 1))) {
					atomicOr(a.devErr, (unsigned)kDevErrTimeout);
					ok = false;
					break;
				}
				asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
				for (int j = 0; j < kChunksPerWarpHL; ++j) {
					const int c = sub + 4 * j;
					if (c < nc) {
						uint32_t u[8], v[8];
						if (x == 0) {
							// Hr and Hi, then C
							tmemLd8(rowBase + (uint32_t)(8 * c), u);
							tmemLd8(rowBase + (uint32_t)(2 * NB + 8 * c), v);
							asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
							for (int i = 0; i < 8; ++i)
								S[j][i] += __uint_as_float(u[i]) + __uint_as_float(v[i]);
							tmemLd8(rowBase + (uint32_t)(NB + 8 * c), u);
							asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
							for (int i = 0; i < 8; ++i)
								S[j][i] += 2.f * __uint_as_float(u[i]);
						} else {
							tmemLd8(rowBase + (uint32_t)(3 * NB + 8 * c), u);
							tmemLd8(rowBase + (uint32_t)(4 * NB + 8 * c), v);
							asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
							for (int i = 0; i < 8; ++i)
								D[j][i] += __uint_as_float(u[i]) + __uint_as_float(v[i]);
						}
					}
				}
				asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
				__syncwarp();
				if (lane == 0)
					barArrive(&drainDone[x]);
			}
		}
		if (ok) {
			// partials of this CTA: [2 (S, D)][128][N], rows < W
			const int row = q * 32 + lane;
			if (row < W) {
#pragma unroll
				for (int j = 0; j < kChunksPerWarpHL; ++j) {
					const int c = sub + 4 * j;
					if (c < nc) {
						float4* s4 = reinterpret_cast<float4*>(a.partials + (((size_t)blockIdx.x * 2) * 128 + row) * NB + 8 * c);
						float4* d4 = reinterpret_cast<float4*>(a.partials + (((size_t)blockIdx.x * 2 + 1) * 128 + row) * NB + 8 * c);
						s4[0] = make_float4(S[j][0], S[j][1], S[j][2], S[j][3]);
						s4[1] = make_float4(S[j][4], S[j][5], S[j][6], S[j][7]);
						d4[0] = make_float4(D[j][0], D[j][1], D[j][2], D[j][3]);
						d4[1] = make_float4(D[j][4], D[j][5], D[j][6], D[j][7]);
					}
				}
			}
		}
	} else {
		// ---- converters: raw interleaved rows -> four planes of the operand buffer ----
		const int sub = lane >> 4, p = lane & 15;
		const uint32_t plane = (uint32_t)NB * 128u;
		for (int t = 0; t < nT; ++t) {
			const int s = t % a.stages, b = t % kOpBufs;
			if (!barWait(&rawFull[s], (uint32_t)((t / a.stages) & 1)) ||
			    (t >= kOpBufs && !barWait(&opEmpty[b], (uint32_t)(((t / kOpBufs) - 1) & 1)))) {
				atomicOr(a.devErr, (unsigned)kDevErrTimeout);
				sFail = 1u;
				break;
			}
			const float* rs = reinterpret_cast<const float*>(raw + (size_t)s * rawStride);
			unsigned char* op = ops + (size_t)b * opBytes;
			if (BF16) {
				const uint64_t kb = (t0 + t) * (uint64_t)kKTB + 4u * p;
				float wq[4] = {1.f, 1.f, 1.f, 1.f};
				if (a.weightK)
#pragma unroll
					for (int q = 0; q < 4; ++q)
						wq[q] = (kb + q < a.K) ? sqrtf((float)a.weightK[kb + q]) : 0.f;
				for (int w = 2 * warp + sub; w < W; w += 2 * kConvWarps) {
					const float4 v0 = *reinterpret_cast<const float4*>(rs + w * 128 + 8 * p);
					const float4 v1 = *reinterpret_cast<const float4*>(rs + w * 128 + 8 * p + 4);
					const float re[4] = {v0.x * wq[0], v0.z * wq[1], v1.x * wq[2], v1.z * wq[3]};
					const float im[4] = {v0.y * wq[0], v0.w * wq[1], v1.y * wq[2], v1.w * wq[3]};
					uint32_t hr[4], hm[4], lr[4], lm[4];
#pragma unroll
					for (int q = 0; q < 4; ++q) {
						float br, bm, dummy;
						hr[q] = bf16Bits(re[q], &br);
						hm[q] = bf16Bits(im[q], &bm);
						lr[q] = bf16Bits(re[q] - br, &dummy);
						lm[q] = bf16Bits(im[q] - bm, &dummy);
					}
					// planes NB rows apart (NB a multiple of 8: the same swizzle phase)
					unsigned char* o = op + swzOffset16(w, 4 * p);
					*reinterpret_cast<uint2*>(o) = make_uint2(hr[0] | (hr[1] << 16), hr[2] | (hr[3] << 16));
					*reinterpret_cast<uint2*>(o + plane) = make_uint2(lr[0] | (lr[1] << 16), lr[2] | (lr[3] << 16));
					*reinterpret_cast<uint2*>(o + 2 * plane) =
					    make_uint2(lm[0] | (lm[1] << 16), lm[2] | (lm[3] << 16));
					*reinterpret_cast<uint2*>(o + 3 * plane) =
					    make_uint2(hm[0] | (hm[1] << 16), hm[2] | (hm[3] << 16));
				}
			} else {
				const uint64_t k0 = (t0 + t) * (uint64_t)kKT + 2u * p;
				float w0 = 1.f, w1 = 1.f;
				if (a.weightK) {
					w0 = (k0 < a.K) ? sqrtf((float)a.weightK[k0]) : 0.f;
					w1 = (k0 + 1 < a.K) ? sqrtf((float)a.weightK[k0 + 1]) : 0.f;
				}
				for (int w = 2 * warp + sub; w < W; w += 2 * kConvWarps) {
					const float4 v = *reinterpret_cast<const float4*>(rs + w * 64 + 4 * p);
					const float re0 = v.x * w0, im0 = v.y * w0, re1 = v.z * w1, im1 = v.w * w1;
					const float2 hre = make_float2(tf32Round(re0), tf32Round(re1));
					const float2 him = make_float2(tf32Round(im0), tf32Round(im1));
					unsigned char* o = op + swzOffset(w, 2 * p);
					*reinterpret_cast<float2*>(o) = hre;
					*reinterpret_cast<float2*>(o + plane) = make_float2(tf32Round(re0 - hre.x), tf32Round(re1 - hre.y));
					*reinterpret_cast<float2*>(o + 2 * plane) =
					    make_float2(tf32Round(im0 - him.x), tf32Round(im1 - him.y));
					*reinterpret_cast<float2*>(o + 3 * plane) = him;
				}
			}
			asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
			__syncwarp();
			if (lane == 0) {
				barArrive(&rawEmpty[s]);
				barArrive(&opFull[b]);
			}
		}
	}
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
	__syncthreads();
	if (warp == kMmaWarp) {
		asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
	}
}

// FP64 sum of the CTAs' partials; assembles the Hermitian matrix (upper
// triangle from Re and D, lower mirrored, real diagonal).  sym: the first
// partial is S with Re = (S + S^T) / 2 (the hi/lo kernel).  One warp per
// element: lane l sums CTAs l, l + 32, ... in order, a fixed butterfly
// combines the lanes (the same order on every run).
__global__ void __launch_bounds__(256) gramTcReduceKernel(const float* partials, int grid, int W, int N, int sym,
                                                          double* out)
{
	const int lane = threadIdx.x & 31;
	const int nWarps = (int)((gridDim.x * blockDim.x) >> 5);
	const int n = W * W;
	for (int e = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); e < n; e += nWarps) {
		const int i = e / W, j = e - i * W;
		if (i > j)
			continue;
		double re = 0., im = 0.;
		for (int c = lane; c < grid; c += 32) {
			const float* Re = partials + (size_t)c * 2 * 128 * N;
			const float* D = Re + (size_t)128 * N;
			re += sym ? 0.5 * ((double)Re[(size_t)i * N + j] + (double)Re[(size_t)j * N + i])
			          : (double)Re[(size_t)i * N + j];
			im += (double)D[(size_t)i * N + j] - (double)D[(size_t)j * N + i];
		}
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) {
			re += __shfl_xor_sync(0xffffffffu, re, o);
			im += __shfl_xor_sync(0xffffffffu, im, o);
		}
		if (lane == 0) {
			if (i == j)
				im = 0.;
			out[(size_t)e * 2] = re;
			out[(size_t)e * 2 + 1] = im;
			out[((size_t)j * W + i) * 2] = re;
			out[((size_t)j * W + i) * 2 + 1] = -im;
		}
	}
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

int encodeTiled(EncodeTiledFn* fn)
{
	static std::mutex m;
	static EncodeTiledFn cached = nullptr;
	std::lock_guard<std::mutex> lock(m);
	if (!cached) {
		void* p = nullptr;
		cudaDriverEntryPointQueryResult q;
		const cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q);
		if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p)
			return setError(kErrCuda, "cuTensorMapEncodeTiled is not available from the driver");
		cached = reinterpret_cast<EncodeTiledFn>(p);
	}
	*fn = cached;
	return kOk;
}

}  // namespace

size_t gramTcScratchFloats(int W, int numSMs)
{
	const int N = ((W + 15) / 16) * 16;
	return (size_t)numSMs * 2 * 128 * N;
}

int launchGramTc(const GramArgs& g, int precision, int numSMs, cudaStream_t s, double* out, double* scratch,
                 size_t scratchDoubles)
{
	if (precision != 2 && precision != 3 && precision != 4)
		return setError(kErrUnsupported, "tensor-core Gram: precision must be TF32, TF32x3 or BF16x3");
	if (g.amps64 || !g.amps)
		return setError(kErrUnsupported, "tensor-core Gram: complex64 amplitudes required");
	if (g.W < 1 || g.W > 128)
		return setError(kErrUnsupported, "tensor-core Gram supports 1..128 waves");
	if ((g.ldK & 1ull) || (reinterpret_cast<uintptr_t>(g.amps) & 15u))
		return setError(kErrUnsupported, "tensor-core Gram needs an even row stride and a 16-byte aligned base");
	if (g.K == 0)
		return setError(kErrArg, "tensor-core Gram: no events");
	if (g.groupStride && ((g.W & 1) || (g.groupStride & 1ull)))
		return setError(kErrUnsupported, "tensor-core Gram: two row groups need an even wave count and group offset");
	int dev = 0;
	PWA_CHECK_RET(cudaCheck(cudaGetDevice(&dev), "cudaGetDevice"));
	int maxSmem = 0;
	PWA_CHECK_RET(cudaCheck(cudaDeviceGetAttribute(&maxSmem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev), "smem"));

	TcArgs a{};
	a.K = g.K;
	a.W = g.W;
	a.N = ((g.W + 15) / 16) * 16;
	a.planes = (precision == 2) ? 1 : 2;
	// hi/lo precisions up to 96 waves: the wide-product kernel, drained every
	// third tile (each accumulator element then collects as many tensor-core
	// additions between drains as the per-tile drain of the narrow kernel)
	const bool hiLo = a.planes == 2 && ((g.W + 15) / 16) * 16 <= kMaxNDB;
	a.period = (precision == 2) ? 8 : (hiLo ? 3 : 1);
	a.bf16 = (precision == 4) ? 1 : 0;
	a.kt = a.bf16 ? kKTB : kKT;
	a.tilesTotal = (g.K + a.kt - 1) / a.kt;
	a.groups = g.groupStride ? 2 : 1;
	a.weightK = g.weightK;
	a.devErr = g.devErr;
	const size_t rawStride = ((size_t)g.W * a.kt * 8 + 1023) & ~size_t(1023);
	const size_t opBytes = hiLo ? (size_t)hlOpBytes(((g.W + 15) / 16) * 16) : (size_t)a.planes * kPlaneBytes;
	const size_t fixed = 1024 /* alignment */ + (size_t)kOpBufs * opBytes + 256 /* barriers */;
	a.stages = 4;
	while (a.stages > 1 && fixed + a.stages * rawStride > (size_t)maxSmem)
		--a.stages;
	size_t smemBytes = fixed + a.stages * rawStride;
	if (smemBytes > (size_t)maxSmem)
		return setError(kErrUnsupported, "tensor-core Gram: shared memory too small for this wave count");
	// one CTA per SM: each CTA allocates all 512 tensor-memory columns
	smemBytes = std::max(smemBytes, (size_t)maxSmem / 2 + 2048);
	const int grid = (int)std::min<uint64_t>((uint64_t)numSMs, a.tilesTotal);
	const size_t need = (size_t)grid * 2 * 128 * a.N;
	if (need > scratchDoubles * 2)
		return setError(kErrArg, "tensor-core Gram: scratch too small");
	a.partials = reinterpret_cast<float*>(scratch);

	EncodeTiledFn enc = nullptr;
	PWA_CHECK_RET(encodeTiled(&enc));
	CUtensorMap map;
	// one group: (float x, row); two groups: (float x, row, group), the box
	// [2][W/2][64 floats] landing in shared memory as [W][64]
	const int G = a.groups == 2 ? g.W / 2 : g.W;
	const cuuint64_t dims[3] = {(cuuint64_t)(2 * g.K), (cuuint64_t)G, 2};
	const cuuint64_t strides[2] = {(cuuint64_t)(g.ldK * 8), (cuuint64_t)(g.groupStride * 8)};
	const cuuint32_t box[3] = {(cuuint32_t)(2 * a.kt), (cuuint32_t)G, 2};
	const cuuint32_t estr[3] = {1u, 1u, 1u};
	const CUresult cr = enc(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, a.groups == 2 ? 3 : 2, const_cast<float2*>(g.amps),
	                        dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
	                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
	if (cr != CUDA_SUCCESS)
		return setError(kErrCuda, "cuTensorMapEncodeTiled failed (" + std::to_string((int)cr) + ")");

	// the dynamic shared-memory limit of each variant is raised once to the
	// largest size asked for (a host call that per-bin batches would
	// otherwise repeat hundreds of times)
	static std::mutex attrMutex;
	static size_t configured[4] = {0, 0, 0, 0};
	auto ensureSmem = [&](const void* k, int variant) -> int {
		std::lock_guard<std::mutex> lock(attrMutex);
		if (smemBytes <= configured[variant])
			return kOk;
		PWA_CHECK_RET(cudaCheck(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smemBytes),
		                        "gram TC smem attribute"));
		configured[variant] = smemBytes;
		return kOk;
	};
	if (hiLo) {
		auto* k = a.bf16 ? gramTcHiLoKernel<true> : gramTcHiLoKernel<false>;
		PWA_CHECK_RET(ensureSmem((const void*)k, a.bf16 ? 1 : 0));
		k<<<grid, kThreadsHL, smemBytes, s>>>(map, a);
	} else if (a.N <= kMaxNDB) {
		PWA_CHECK_RET(ensureSmem((const void*)gramTcKernel<true>, 2));
		gramTcKernel<true><<<grid, kThreadsDB, smemBytes, s>>>(map, a);
	} else {
		PWA_CHECK_RET(ensureSmem((const void*)gramTcKernel<false>, 3));
		gramTcKernel<false><<<grid, kThreadsTc, smemBytes, s>>>(map, a);
	}
	countLaunches(1);
	PWA_CHECK_RET(cudaCheck(cudaGetLastError(), "gram TC launch"));
	const int n = g.W * g.W;
	const int blocks = std::max(1, std::min(4096, (n + 7) / 8));  // eight warps per block, one per element
	gramTcReduceKernel<<<blocks, 256, 0, s>>>(a.partials, grid, g.W, a.N, hiLo ? 1 : 0, out);
	countLaunches(1);
	return cudaCheck(cudaGetLastError(), "gram TC reduce launch");
}

}  // namespace pwa
