// debug_wait.cu -- test hook for the device-side failure path: a bounded
// wait that runs out.
//
// Every spin-wait of the streaming kernels (mbarrier phases of bulk copies
// and tensor-core commits) gives up after a time limit, sets kDevErrTimeout in
// a device flag and returns, so that the host reports
// PWA_ERROR_DEVICE_TIMEOUT and the context stays usable.  This kernel takes
// the same route on purpose without any fault: one thread arms an mbarrier
// for 16 bytes of transfer that no copy ever delivers (no copy is issued, so
// nothing is in flight when the block exits), every thread of the warp waits
// on it with the production wait helper and a short limit, and the expiry is
// recorded in the flag.
#include "device_common.cuh"
#include "host_common.h"

namespace pwa {
namespace {

__device__ unsigned g_stalledWaitFlag;

__global__ void stalledWaitKernel(unsigned long long limitNs)
{
	__shared__ __align__(8) uint64_t bar;
	if (threadIdx.x == 0) {
		mbarInit(&bar, 1);
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	__syncwarp();
	if (threadIdx.x == 0)
		mbarArriveExpectTx(&bar, 16);
	__syncwarp();
	const bool done = mbarWaitBounded(&bar, 0, limitNs);
	if (!done && threadIdx.x == 0)
		atomicOr(&g_stalledWaitFlag, (unsigned)kDevErrTimeout);
}

}  // namespace
}  // namespace pwa

using namespace pwa;

extern "C" int pwa_debug_stalled_wait(uint32_t limitMicroseconds)
{
	if (limitMicroseconds == 0 || limitMicroseconds > 1000000u)
		return setError(kErrArg, "pwa_debug_stalled_wait: limit must be 1 us .. 1 s");
	const unsigned zero = 0;
	PWA_CHECK(cudaCheck(cudaMemcpyToSymbol(g_stalledWaitFlag, &zero, sizeof zero), "stalled wait: clear flag"));
	stalledWaitKernel<<<1, 32>>>(1000ull * limitMicroseconds);
	countLaunches(1);
	PWA_CHECK(cudaCheck(cudaGetLastError(), "stalled wait: launch"));
	unsigned flag = 0;
	PWA_CHECK(cudaCheck(cudaMemcpyFromSymbol(&flag, g_stalledWaitFlag, sizeof flag), "stalled wait: read flag"));
	if (flag & kDevErrTimeout)
		return setError(kErrTimeout, "pwa_debug_stalled_wait: bounded device wait expired (as intended)");
	return kOk;
}
