// host_common.cpp -- status codes and the last error message, the kernel
// launch counter, the allocation-failure test hook and small helpers shared
// by the host translation units.

#include "host_common.h"

namespace {
thread_local std::string g_lastError;
std::atomic<uint64_t> g_launches{0};
}  // namespace

namespace pwa {

std::atomic<long> g_failAllocAfter{-1};

int setError(int code, const std::string& msg)
{
	if (code != kOk)
		g_lastError = msg;
	return code;
}

int cudaCheck(cudaError_t e, const char* what)
{
	if (e == cudaSuccess)
		return kOk;
	cudaGetLastError();  // clear the sticky-free error state of the runtime
	return setError(e == cudaErrorMemoryAllocation ? kErrOom : kErrCuda,
	                std::string(what) + ": " + cudaGetErrorString(e));
}

void countLaunches(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

int deviceInfo(int* dev, int* sms, size_t* smem)
{
	PWA_TRY(cudaCheck(cudaGetDevice(dev), "cudaGetDevice"));
	PWA_TRY(cudaCheck(cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, *dev), "SM count"));
	int optin = 0;
	PWA_TRY(cudaCheck(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, *dev), "smem"));
	*smem = (size_t)optin;
	return kOk;
}

std::string fmtDouble(double v)
{
	char buf[64];
	std::snprintf(buf, sizeof(buf), "%.16e", v);
	return buf;
}

double seconds()
{
	return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace pwa

extern "C" {

int pwa_abi_version(void) { return PWA_GB300_ABI_VERSION; }
const char* pwa_last_error(void) { return g_lastError.c_str(); }
uint64_t pwa_kernel_launch_count(void) { return g_launches.load(); }

int pwa_debug_fail_alloc_after(int64_t n)
{
	g_failAllocAfter.store(n < 0 ? -1 : (long)n);
	return kOk;
}

}  // extern "C"
