// otf_kernels.cu -- on-the-fly event binning on the GPU.
//
// pwaLikelihood::setOnTheFlyBinning (partialWaveFit/pwaLikelihood.cc:1391-1440)
// drops an event of the data file when a binning variable v has x_v < lower_v
// or x_v >= upper_v and keeps the others in file order, and addAmplitude
// then reads only
// those events.  Here the selection is two passes over the per-event binning
// variables (stored [variable][event] in device memory):
//   otfCountKernel   -- events selected per block of kOtfChunk events;
//   (the host turns the counts into block offsets)
//   otfCompactKernel -- each block writes the indices of its selected events
//                       at its offset, in event order (warp ballots and a
//                       block-wide scan of the warps' counts);
// and otfGatherKernel copies the selected events of an amplitude row.

#include "pwa_internal.h"

#include <algorithm>

namespace pwa {
namespace {

constexpr int kOtfThreads = 256;

__device__ __forceinline__ bool otfSelected(const OtfArgs& a, uint64_t e)
{
	for (int v = 0; v < a.nVars; ++v) {
		const double x = a.vars[(size_t)v * a.n + e];
		// the reference's rejection test, so a NaN value keeps the event
		if (x < a.lower[v] || x >= a.upper[v])
			return false;
	}
	return true;
}

__global__ void otfCountKernel(const OtfArgs a, unsigned* counts)
{
	__shared__ unsigned warpCount[kOtfThreads / 32];
	const uint64_t b0 = (uint64_t)blockIdx.x * kOtfChunk;
	unsigned c = 0;
	for (int i = threadIdx.x; i < kOtfChunk; i += kOtfThreads) {
		const uint64_t e = b0 + i;
		if (e < a.n && otfSelected(a, e))
			++c;
	}
	for (int o = 16; o > 0; o >>= 1)
		c += __shfl_xor_sync(0xffffffffu, c, o);
	if ((threadIdx.x & 31) == 0)
		warpCount[threadIdx.x >> 5] = c;
	__syncthreads();
	if (threadIdx.x == 0) {
		unsigned t = 0;
		for (int w = 0; w < kOtfThreads / 32; ++w)
			t += warpCount[w];
		counts[blockIdx.x] = t;
	}
}

// the block's events in rounds of kOtfThreads consecutive events: a ballot
// per warp, the warps' counts scanned in shared memory, so the indices come
// out in event order
__global__ void otfCompactKernel(const OtfArgs a, const unsigned long long* offsets, unsigned long long* idx)
{
	__shared__ unsigned warpCount[kOtfThreads / 32];
	__shared__ unsigned long long base;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const uint64_t b0 = (uint64_t)blockIdx.x * kOtfChunk;
	if (threadIdx.x == 0)
		base = offsets[blockIdx.x];
	__syncthreads();
	for (int r = 0; r < kOtfChunk; r += kOtfThreads) {
		const uint64_t e = b0 + r + threadIdx.x;
		const bool sel = e < a.n && otfSelected(a, e);
		const unsigned m = __ballot_sync(0xffffffffu, sel);
		if (lane == 0)
			warpCount[warp] = __popc(m);
		__syncthreads();
		unsigned before = 0, total = 0;
		for (int w = 0; w < kOtfThreads / 32; ++w) {
			if (w < warp)
				before += warpCount[w];
			total += warpCount[w];
		}
		if (sel)
			idx[base + before + __popc(m & ((1u << lane) - 1u))] = e;
		__syncthreads();
		if (threadIdx.x == 0)
			base += total;
		__syncthreads();
	}
}

__global__ void otfGatherKernel(const unsigned char* src, const unsigned long long* idx, uint64_t n, int elemBytes,
                                unsigned char* dst)
{
	for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
		const unsigned char* s = src + idx[i] * (uint64_t)elemBytes;
		unsigned char* d = dst + i * (uint64_t)elemBytes;
		if (elemBytes == 16)
			*reinterpret_cast<double2*>(d) = *reinterpret_cast<const double2*>(s);
		else
			*reinterpret_cast<float2*>(d) = *reinterpret_cast<const float2*>(s);
	}
}

}  // namespace

int launchOtfCount(const OtfArgs& a, unsigned* counts, cudaStream_t s)
{
	const uint64_t blocks = (a.n + kOtfChunk - 1) / kOtfChunk;
	otfCountKernel<<<(unsigned)std::max<uint64_t>(1, blocks), kOtfThreads, 0, s>>>(a, counts);
	countLaunches(1);
	return cudaCheck(cudaGetLastError(), "OTF count launch");
}

int launchOtfCompact(const OtfArgs& a, const unsigned long long* offsets, unsigned long long* idx, cudaStream_t s)
{
	const uint64_t blocks = (a.n + kOtfChunk - 1) / kOtfChunk;
	otfCompactKernel<<<(unsigned)std::max<uint64_t>(1, blocks), kOtfThreads, 0, s>>>(a, offsets, idx);
	countLaunches(1);
	return cudaCheck(cudaGetLastError(), "OTF compaction launch");
}

int launchOtfGather(const void* src, const unsigned long long* idx, uint64_t n, int elemBytes, void* dst,
                    cudaStream_t s)
{
	const int blocks = (int)std::min<uint64_t>(4096, std::max<uint64_t>(1, (n + 255) / 256));
	otfGatherKernel<<<blocks, 256, 0, s>>>(static_cast<const unsigned char*>(src), idx, n, elemBytes,
	                                        static_cast<unsigned char*>(dst));
	countLaunches(1);
	return cudaCheck(cudaGetLastError(), "OTF gather launch");
}

}  // namespace pwa
