// device_common.cuh -- device helpers shared by the streaming kernels:
// mbarrier and bulk-copy wrappers (with waits bounded by %globaltimer),
// programmatic-dependent-launch controls, warp reductions, packed FP32x2 FMA
// and shared-window loads.
#pragma once

#include <cstdint>

namespace pwa {

// bound of every spin-wait on the device (1 s); on expiry the caller records
// kDevErrTimeout and returns
constexpr unsigned long long kWaitLimitNs = 1000000000ull;

__device__ __forceinline__ uint32_t smemAddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Bounds checks of shared-memory accesses for the debug build (compiled with
// -DPWA_DEBUG_CHECKS, the stand-in for a memory checker): an access of
// `bytes` at shared address `addr` must lie in [lo, hi); otherwise the flag
// kDevErrBounds (2) is set in *err and the caller skips the access.  In the
// release build the check is the constant true and costs nothing.
#ifdef PWA_DEBUG_CHECKS
__device__ __forceinline__ bool smemInBounds(uint32_t addr, uint32_t bytes, uint32_t lo, uint32_t hi, unsigned* err)
{
	if (addr >= lo && addr + bytes <= hi && (addr & (bytes - 1u)) == 0u)
		return true;
	atomicOr(err, 2u);
	return false;
}
#else
__device__ __forceinline__ bool smemInBounds(uint32_t, uint32_t, uint32_t, uint32_t, unsigned*) { return true; }
#endif

__device__ __forceinline__ void mbarInit(uint64_t* bar, uint32_t count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbarArriveExpectTx(uint64_t* bar, uint32_t bytes)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smemAddr(bar)), "r"(bytes)
	             : "memory");
}

__device__ __forceinline__ bool mbarTryWait(uint64_t* bar, uint32_t parity)
{
	uint32_t ok;
	asm volatile(
	    "{\n\t.reg .pred p;\n\t"
	    "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
	    "selp.u32 %0, 1, 0, p;\n\t}"
	    : "=r"(ok)
	    : "r"(smemAddr(bar)), "r"(parity)
	    : "memory");
	return ok != 0;
}

__device__ __forceinline__ unsigned long long globalTimer()
{
	unsigned long long t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}

// Bounded wait for the phase with the given parity to complete (false after
// limitNs of %globaltimer).
static __device__ bool mbarWaitBounded(uint64_t* bar, uint32_t parity, unsigned long long limitNs = kWaitLimitNs)
{
	if (mbarTryWait(bar, parity))
		return true;
	const unsigned long long t0 = globalTimer();
	while (true) {
		if (mbarTryWait(bar, parity))
			return true;
		if (globalTimer() - t0 > limitNs)
			return false;
	}
}

__device__ __forceinline__ void bulkCopyG2S(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
	                 smemAddr(dst)),
	             "l"(src), "r"(bytes), "r"(smemAddr(bar))
	             : "memory");
}

__device__ __forceinline__ void fenceProxyAsync() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Programmatic dependent launch: wait until the preceding grid in the stream
// has completed and its memory is visible; allow the next grid to launch.
__device__ __forceinline__ void gridDependencyWait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void gridDependencyTrigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Per-event c = -2 / L and ln L of the FdF kernels with the hardware
// reciprocal and base-2 logarithm (a few instructions each, where the IEEE
// division and the full-accuracy logf took about 30 per warp and event;
// 2.3 % of the 87-wave, 10^6-event FdF).  Relative errors are about 2^-21;
// the FdF's LL error against the FP64 oracle at 10^6 events went from 2.7e-9
// to 3.7e-8, the gradient's from 1.9e-8 to 2.6e-8.  The batched-fit kernels
// keep the IEEE forms: their line searches work near the rounding floor of
// f, where the faster forms changed the plain fit's convergence tail.
__device__ __forceinline__ float eventWeight(float L) { return __fdividef(-2.f, L); }
__device__ __forceinline__ float eventLog(float L) { return __logf(L); }

__device__ __forceinline__ float warpSum(float v)
{
#pragma unroll
	for (int o = 16; o > 0; o >>= 1)
		v += __shfl_xor_sync(0xffffffffu, v, o);
	return v;
}

__device__ __forceinline__ double warpSumD(double v)
{
#pragma unroll
	for (int o = 16; o > 0; o >>= 1)
		v += __shfl_xor_sync(0xffffffffu, v, o);
	return v;
}

// Warp reduce-scatter of 32 values held by every lane: afterwards x[0] of
// lane l holds the sum over all lanes of value index l.
__device__ __forceinline__ float reduceScatter32(float* x, int lane)
{
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) {
		const bool up = (lane & o) != 0;
#pragma unroll
		for (int k = 0; k < o; ++k) {
			const float send = up ? x[k] : x[k + o];
			const float keep = up ? x[k + o] : x[k];
			x[k] = keep + __shfl_xor_sync(0xffffffffu, send, o);
		}
	}
	return x[0];
}

__device__ __forceinline__ void kahanAdd(float& s, float& c, float x)
{
	const float y = x - c;
	const float t = s + y;
	c = (t - s) - y;
	s = t;
}

__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c)
{
	float2 d;
	asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\t"
	    "mov.b64 ra, {%2, %3};\n\t"
	    "mov.b64 rb, {%4, %5};\n\t"
	    "mov.b64 rc, {%6, %7};\n\t"
	    "fma.rn.f32x2 rd, ra, rb, rc;\n\t"
	    "mov.b64 {%0, %1}, rd;\n\t}"
	    : "=f"(d.x), "=f"(d.y)
	    : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
	return d;
}

// shared-memory loads through 32-bit shared-window addresses
__device__ __forceinline__ float2 lds64(uint32_t addr)
{
	float2 v;
	asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr));
	return v;
}
__device__ __forceinline__ float4 lds128(uint32_t addr)
{
	float4 v;
	asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(addr));
	return v;
}

// loads with the debug build's bounds check against [lo, hi)
__device__ __forceinline__ float2 lds64c(uint32_t addr, uint32_t lo, uint32_t hi, unsigned* err)
{
	return smemInBounds(addr, 8u, lo, hi, err) ? lds64(addr) : make_float2(0.f, 0.f);
}

__device__ __forceinline__ float4 lds128c(uint32_t addr, uint32_t lo, uint32_t hi, unsigned* err)
{
	return smemInBounds(addr, 16u, lo, hi, err) ? lds128(addr) : make_float4(0.f, 0.f, 0.f, 0.f);
}

}  // namespace pwa
