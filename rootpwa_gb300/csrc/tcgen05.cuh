// tcgen05.cuh -- device helpers of the tensor-core kernels (gram_tc.cu,
// mlp.cu): shared-memory addresses, bounded mbarrier waits, TMA and bulk
// tensor copies, tcgen05 matrix descriptors, MMAs, commits and tensor-memory
// loads and stores, and the canonical K-major 128-byte-swizzled layout.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cstdint>

namespace pwa {
namespace {

// bound of every mbarrier wait (1 s of globaltimer); on expiry the caller
// records a device error and winds down
constexpr unsigned long long kWaitNs = 1000000000ull;

__device__ __forceinline__ uint32_t sAddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long nowNs()
{
	unsigned long long t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}

__device__ __forceinline__ void barInit(uint64_t* b, uint32_t count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sAddr(b)), "r"(count) : "memory");
}

__device__ __forceinline__ void barArrive(uint64_t* b)
{
	asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(sAddr(b)) : "memory");
}

__device__ __forceinline__ void barExpectTx(uint64_t* b, uint32_t bytes)
{
	asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(sAddr(b)),
	             "r"(bytes)
	             : "memory");
}

__device__ __forceinline__ bool barTry(uint64_t* b, uint32_t parity)
{
	uint32_t ok;
	asm volatile(
	    "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
	    : "=r"(ok)
	    : "r"(sAddr(b)), "r"(parity)
	    : "memory");
	return ok != 0;
}

// bounded wait for the completion of phase `parity`
__device__ bool barWait(uint64_t* b, uint32_t parity)
{
	if (barTry(b, parity))
		return true;
	const unsigned long long t0 = nowNs();
	while (!barTry(b, parity))
		if (nowNs() - t0 > kWaitNs)
			return false;
	return true;
}

__device__ __forceinline__ void tmaLoad2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar)
{
	asm volatile(
	    "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
	        sAddr(dst)),
	    "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(sAddr(bar))
	    : "memory");
}

// the same for a map of two row groups (x, row, group)
__device__ __forceinline__ void tmaLoad3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar)
{
	asm volatile(
	    "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
	        sAddr(dst)),
	    "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(sAddr(bar))
	    : "memory");
}

__device__ __forceinline__ float tf32Round(float x)
{
	uint32_t r;
	asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
	return __uint_as_float(r);
}

// K-major, 128-byte swizzle shared-memory matrix descriptor (tcgen05 format):
// start address >> 4 at [0,14), leading byte offset >> 4 at [16,30) (unused
// for swizzled K-major layouts), stride byte offset >> 4 at [32,46) = 1024 B
// between groups of 8 rows, version 1 at [46,48), swizzle mode 2 (128 B) at
// [61,64).
__device__ __forceinline__ uint64_t smemDesc(uint32_t addr)
{
	return (uint64_t)((addr & 0x3ffffu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
	       ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// instruction descriptor of kind::tf32: D format F32 at [4,6), A and B
// format TF32 (2) at [7,10) and [10,13), both K-major, N >> 3 at [17,23),
// M >> 4 at [24,29)
__host__ __device__ constexpr uint32_t idescTf32(int M, int N)
{
	return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// instruction descriptor of kind::f16 with BF16 operands: D format F32 at
// [4,6), A and B format BF16 (1) at [7,10) and [10,13), both K-major,
// N >> 3 at [17,23), M >> 4 at [24,29)
__host__ __device__ constexpr uint32_t idescBf16(int M, int N)
{
	return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mmaBf16(uint32_t dTmem, uint64_t aDesc, uint64_t bDesc, uint32_t idesc, uint32_t acc)
{
	asm volatile(
	    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
	    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dTmem),
	    "l"(aDesc), "l"(bDesc), "r"(idesc), "r"(acc)
	    : "memory");
}

__device__ __forceinline__ void mmaTf32(uint32_t dTmem, uint64_t aDesc, uint64_t bDesc, uint32_t idesc, uint32_t acc)
{
	asm volatile(
	    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
	    "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(dTmem),
	    "l"(aDesc), "l"(bDesc), "r"(idesc), "r"(acc)
	    : "memory");
}

__device__ __forceinline__ void mmaCommit(uint64_t* bar)
{
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(sAddr(bar))
	             : "memory");
}

// byte offset of element (row r, column k < 32) in a K-major 128-byte
// swizzled TF32 tile: 8-row groups of 1024 B, 16-byte chunks XOR row % 8
__device__ __forceinline__ uint32_t swzOffset(int r, int k)
{
	return (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + ((((k >> 2) ^ (r & 7)) & 7) << 4) + (k & 3) * 4);
}

// the same for BF16 elements (k < 64): 8 elements per 16-byte chunk
__device__ __forceinline__ uint32_t swzOffset16(int r, int k)
{
	return (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + ((((k >> 3) ^ (r & 7)) & 7) << 4) + (k & 7) * 2);
}

// BF16 bits of x rounded to nearest even, and the FP32 value of those bits
__device__ __forceinline__ uint32_t bf16Bits(float x, float* back)
{
	const __nv_bfloat16 h = __float2bfloat16_rn(x);
	*back = __bfloat162float(h);
	return (uint32_t)__bfloat16_as_ushort(h);
}

__device__ __forceinline__ void tmemLd16(uint32_t taddr, uint32_t (&r)[16])
{
	asm volatile(
	    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
	    "%15}, [%16];"
	    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
	      "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
	    : "r"(taddr));
}

__device__ __forceinline__ void tmemSt16(uint32_t taddr, const uint32_t (&r)[16])
{
	asm volatile(
	    "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
	    "%15, %16};" ::"r"(taddr),
	    "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]),
	    "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
	    : "memory");
}

__device__ __forceinline__ void tmemLd8(uint32_t taddr, uint32_t (&r)[8])
{
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
	             : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
	             : "r"(taddr));
}

}  // namespace
}  // namespace pwa
