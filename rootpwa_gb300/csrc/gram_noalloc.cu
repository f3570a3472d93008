// gram_noalloc.cu -- Gram-matrix entry point that allocates no memory.
//
// pwa_gram_device_noalloc computes the raw integral sums of
// ampIntegralMatrix::integrate (decayAmplitude/ampIntegralMatrix.cc:408-469)
//   I_ij = sum_k w_k A_{i,k} conj(A_{j,k})
// of device-resident complex64 amplitudes into a caller-owned device matrix
// with the SIMT Gram kernels of integral_kernels.cu.  Their per-chunk
// partial sums live in a file-scope device array of fixed size rather than
// in a buffer from cudaMalloc, so a call allocates nothing, frees nothing
// (cudaFree synchronises the whole device) and makes no host round trip.
//
// Setup: the first call on a device (that device current) resolves the
// array's address with cudaGetSymbolAddress; that first call has to happen
// before any stream capture on the device.  The cached address is valid for
// the life of the device's primary context (a cudaDeviceReset invalidates
// it).  The partial sums need no
// initial value (every entry the reduction reads is written by the Gram
// kernel of the same call).  All calls on one device share the array, so
// calls that overlap in time (different streams or host threads without
// ordering between them) race on it.

#include "pwa_gb300.h"
#include "pwa_internal.h"

#include <algorithm>
#include <mutex>

namespace pwa {
namespace {

#define NOALLOC_TRY(expr)       \
	do {                        \
		const int _st = (expr); \
		if (_st != kOk)         \
			return _st;         \
	} while (0)

// 2^22 doubles = 32 MiB of chunk partials (chunks x W x W x 2 doubles):
// 32 chunks at the largest wave set, 270 at 88 waves
constexpr size_t kScratchDoubles = size_t(1) << 22;
constexpr uint32_t kMaxWaves = PWA_GRAM_NOALLOC_MAX_WAVES;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_gramScratch[kScratchDoubles];

std::mutex g_scratchMutex;
double* g_scratchPtr[kMaxDevices] = {};

int scratchFor(int dev, double** out)
{
	std::lock_guard<std::mutex> lock(g_scratchMutex);
	if (!g_scratchPtr[dev]) {
		void* p = nullptr;
		NOALLOC_TRY(cudaCheck(cudaGetSymbolAddress(&p, g_gramScratch), "cudaGetSymbolAddress(gram scratch)"));
		g_scratchPtr[dev] = static_cast<double*>(p);
	}
	*out = g_scratchPtr[dev];
	return kOk;
}

}  // namespace
}  // namespace pwa

using namespace pwa;

extern "C" int pwa_gram_device_noalloc(const void* amps, uint64_t nK, uint64_t ldK, uint32_t nWaves,
                                       const double* weights, int precision, double* out, void* stream)
{
	if (!amps || !out)
		return setError(kErrArg, "pwa_gram_device_noalloc: null amplitude or output pointer");
	if (nWaves == 0 || nWaves > kMaxWaves)
		return setError(kErrArg, "pwa_gram_device_noalloc: nWaves must be in 1.." + std::to_string(kMaxWaves) +
		                             " (got " + std::to_string(nWaves) + ")");
	if (nK == 0)
		return setError(kErrArg, "pwa_gram_device_noalloc: no events");
	if (ldK < nK)
		return setError(kErrArg, "pwa_gram_device_noalloc: row stride ldK is smaller than nK");
	if (precision != PWA_PRECISION_FP64 && precision != PWA_PRECISION_FP32)
		return setError(kErrUnsupported, "pwa_gram_device_noalloc: precision must be PWA_PRECISION_FP64 or "
		                                 "PWA_PRECISION_FP32 (SIMT kernels)");
	int dev = 0, sms = 0;
	NOALLOC_TRY(cudaCheck(cudaGetDevice(&dev), "cudaGetDevice"));
	if (dev < 0 || dev >= kMaxDevices)
		return setError(kErrUnsupported, "pwa_gram_device_noalloc: device index out of range");
	NOALLOC_TRY(cudaCheck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count"));
	double* scratch = nullptr;
	NOALLOC_TRY(scratchFor(dev, &scratch));

	// integrate()'s chunking: chunks of K per output tile so that the grid
	// fills the GPU, each a run of chunkLen events summed in the kernel's
	// accumulator type
	const size_t perChunk = (size_t)nWaves * nWaves * 2;
	const int tps = ((int)nWaves + 63) / 64;
	const int nTiles = tps * (tps + 1) / 2;
	uint64_t chunks = (uint64_t)std::max(1, (4 * sms + nTiles - 1) / nTiles);
	chunks = std::min<uint64_t>(chunks, std::max<uint64_t>(1, nK / 64));
	const uint64_t chunkLen = (nK + chunks - 1) / chunks;
	// the fixed array holds maxChunks chunk partials; a longer input is taken
	// in segments of maxChunks chunks of the same length, each reduced into
	// out in FP64 (the first segment overwrites out, the others add to it)
	const uint64_t maxChunks = kScratchDoubles / perChunk;
	const uint64_t segLen = maxChunks * chunkLen;
	cudaStream_t s = static_cast<cudaStream_t>(stream);
	for (uint64_t k0 = 0, seg = 0; k0 < nK; k0 += segLen, ++seg) {
		const uint64_t kSeg = std::min(segLen, nK - k0);
		GramArgs g{};
		g.amps = static_cast<const float2*>(amps) + k0;
		g.amps64 = nullptr;
		g.K = kSeg;
		g.ldK = ldK;
		g.W = (int)nWaves;
		g.weightK = weights ? weights + k0 : nullptr;
		g.partials = scratch;
		g.chunks = (int)((kSeg + chunkLen - 1) / chunkLen);
		g.devErr = nullptr;
		NOALLOC_TRY(launchGramSimt(g, precision == PWA_PRECISION_FP64 ? 0 : 1, s));
		NOALLOC_TRY(launchGramReduce(scratch, g.chunks, (int)nWaves, out, seg > 0 ? 1 : 0, s));
	}
	return kOk;
}
