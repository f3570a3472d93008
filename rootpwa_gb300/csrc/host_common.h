// host_common.h -- pieces shared by the host translation units of the C ABI
// (host_common.cpp, host_integral.cpp, host_likelihood.cpp,
// host_multibin.cpp, host_mlp.cpp): device and pinned buffers owned by a
// handle, the status-propagation macro and the integral object, which the
// likelihood reads.
#pragma once

#include "../../include/pwa_gb300.h"
#include "pwa_internal.h"


#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <random>
#include <sstream>
#include <string>
#include <tuple>
#include <vector>

typedef std::complex<double> cplx;

namespace pwa {

// allocation-failure test hook (pwa_debug_fail_alloc_after)
extern std::atomic<long> g_failAllocAfter;

// device allocation owned by a handle
struct DevBuf {
	void* p = nullptr;
	size_t bytes = 0;
	DevBuf() = default;
	DevBuf(const DevBuf&) = delete;
	DevBuf& operator=(const DevBuf&) = delete;
	~DevBuf() { release(); }
	int alloc(size_t b, const char* what)
	{
		release();
		if (b == 0)
			return kOk;
		if (g_failAllocAfter.load() >= 0 && g_failAllocAfter.fetch_sub(1) <= 0) {
			g_failAllocAfter.store(0);
			return setError(kErrOom, std::string(what) + ": injected allocation failure");
		}
		const cudaError_t e = cudaMalloc(&p, b);
		if (e != cudaSuccess) {
			p = nullptr;
			return cudaCheck(e, what);
		}
		bytes = b;
		return kOk;
	}
	int ensure(size_t b, const char* what) { return (bytes >= b && p) ? kOk : alloc(b, what); }
	void release()
	{
		if (p)
			cudaFree(p);
		p = nullptr;
		bytes = 0;
	}
	template <typename T>
	T* as() const
	{
		return static_cast<T*>(p);
	}
};

// page-locked host staging buffer
struct PinnedBuf {
	void* p = nullptr;
	size_t bytes = 0;
	PinnedBuf() = default;
	PinnedBuf(const PinnedBuf&) = delete;
	PinnedBuf& operator=(const PinnedBuf&) = delete;
	~PinnedBuf() { release(); }
	void* dev = nullptr;  // device view of a mapped buffer
	int ensure(size_t b, const char* what, bool mapped = false)
	{
		if (p && bytes >= b && (!mapped || dev))
			return kOk;
		release();
		const cudaError_t e = mapped ? cudaHostAlloc(&p, b, cudaHostAllocMapped) : cudaMallocHost(&p, b);
		if (e != cudaSuccess) {
			p = nullptr;
			return cudaCheck(e, what);
		}
		bytes = b;
		if (mapped) {
			const cudaError_t e2 = cudaHostGetDevicePointer(&dev, p, 0);
			if (e2 != cudaSuccess) {
				release();
				return cudaCheck(e2, what);
			}
		}
		return kOk;
	}
	void release()
	{
		if (p)
			cudaFreeHost(p);
		p = nullptr;
		dev = nullptr;
		bytes = 0;
	}
	template <typename T>
	T* as() const
	{
		return static_cast<T*>(p);
	}
};

#define PWA_TRY(expr)                 \
	do {                              \
		const int _st = (expr);       \
		if (_st != kOk)               \
			return _st;               \
	} while (0)

int deviceInfo(int* dev, int* sms, size_t* smem);
// %.16e, the precision of the ASCII integral files
std::string fmtDouble(double v);
// monotonic wall-clock seconds
double seconds();

}  // namespace pwa

using namespace pwa;

// ===========================================================================
// ampIntegralMatrix: raw sums and the wave list
// ===========================================================================
// device buffers and stream of integrate(), kept by an integral between
// calls on one device (the output matrix, the error flag and the Gram
// partials: no allocation per call once they have their size)
struct GramScratch {
	int dev = -1;
	cudaStream_t stream = nullptr;
	DevBuf out, err, part;
	GramScratch() = default;
	GramScratch(const GramScratch&) = delete;
	GramScratch& operator=(const GramScratch&) = delete;
	~GramScratch() { reset(); }
	void reset()
	{
		out.release();
		err.release();
		part.release();
		if (stream)
			cudaStreamDestroy(stream);
		stream = nullptr;
		dev = -1;
	}
};

struct pwa_integral {
	uint32_t nWaves = 0;
	uint64_t nEvents = 0;
	std::vector<std::string> names;
	std::vector<cplx> sums;  // raw sums [i][j]
	// not part of the value: a copy starts without device buffers
	struct ScratchHolder {
		std::unique_ptr<GramScratch> p;
		ScratchHolder() = default;
		ScratchHolder(const ScratchHolder&) {}
		ScratchHolder& operator=(const ScratchHolder&) { return *this; }
	} scratch;

	int index(const std::string& n) const
	{
		for (size_t i = 0; i < names.size(); ++i)
			if (names[i] == n)
				return (int)i;
		return -1;
	}
	bool sameWaveSet(const pwa_integral& o) const
	{
		if (o.nWaves != nWaves)
			return false;
		for (const auto& n : names)
			if (o.index(n) < 0)
				return false;
		return true;
	}
};
