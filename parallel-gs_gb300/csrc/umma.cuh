// Blackwell (sm_100 family) tensor-core building blocks in inline PTX:
// tcgen05 MMA with accumulators in tensor memory (TMEM), shared-memory matrix
// descriptors, mbarriers with bounded waits, and TMA tensor loads.
//
// Operands are K-major BF16 in shared memory.  Two canonical layouts are used:
//  - no swizzle: 8 x 16-byte "core matrices" (8 rows x 8 elements), the next
//    core matrix along K at LBO bytes, along M/N at SBO bytes;
//  - 64-byte swizzle: rows of 64 bytes (32 BF16), 8-row groups of 512 bytes at
//    SBO; inside a group the 16-byte chunk index of row r is XORed with
//    (r >> 1) & 3 -- the pattern a TMA load with CU_TENSOR_MAP_SWIZZLE_64B
//    writes.  The group must start on a 512-byte boundary.
#pragma once

#include <cstdint>

namespace pgs_umma
{
// Bounded waits: an mbarrier that does not complete within this many polls
// sets an error flag instead of spinning on.
constexpr uint32_t WAIT_LIMIT = 1u << 26;

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return uint32_t(__cvta_generic_to_shared(p)); }

// Instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major,
// M rows x N columns (tcgen05.mma instruction descriptor).
__host__ __device__ constexpr uint32_t idesc_bf16_f32(uint32_t m, uint32_t n)
{
	return (1u << 4)            // D format: F32
	       | (1u << 7)          // A format: BF16
	       | (1u << 10)         // B format: BF16
	       | ((n >> 3) << 17)   // N / 8
	       | ((m >> 4) << 24);  // M / 16
}

enum : uint32_t
{
	LAYOUT_NONE = 0,
	LAYOUT_SWIZZLE_64B = 4,
};

// Shared-memory matrix descriptor (tcgen05 form: version 1 at bit 46).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo, uint32_t layout)
{
	uint64_t d = 0;
	d |= uint64_t((addr >> 4) & 0x3fffu);
	d |= uint64_t((lbo >> 4) & 0x3fffu) << 16;
	d |= uint64_t((sbo >> 4) & 0x3fffu) << 32;
	d |= uint64_t(1) << 46;
	d |= uint64_t(layout & 7u) << 61;
	return d;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count));
}

__device__ __forceinline__ void fence_barrier_init()
{
	asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async()
{
	asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes)
	             : "memory");
}

// Waits for phase `parity` of the barrier; false when the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity)
{
	const uint32_t a = smem_addr(bar);
	for (uint32_t i = 0; i < WAIT_LIMIT; i++)
	{
		uint32_t done;
		asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
		             : "=r"(done)
		             : "r"(a), "r"(parity)
		             : "memory");
		if (done)
			return true;
	}
	return false;
}

// Bounded wait with an explicit poll limit.
__device__ __forceinline__ bool mbar_wait_limit(uint64_t *bar, uint32_t parity, uint32_t limit)
{
	const uint32_t a = smem_addr(bar);
	for (uint32_t i = 0; i < limit; i++)
	{
		uint32_t done;
		asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
		             : "=r"(done)
		             : "r"(a), "r"(parity)
		             : "memory");
		if (done)
			return true;
	}
	return false;
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
	asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_addr(bar)) : "memory");
}

// Bounded wait that also gives up as soon as *abort is set by another warp.
__device__ __forceinline__ bool mbar_wait_or_abort(uint64_t *bar, uint32_t parity, volatile uint32_t *abort)
{
	const uint32_t a = smem_addr(bar);
	for (uint32_t i = 0; i < WAIT_LIMIT; i++)
	{
		uint32_t done;
		asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
		             : "=r"(done)
		             : "r"(a), "r"(parity)
		             : "memory");
		if (done)
			return true;
		if ((i & 255u) == 255u && *abort)
			return false;
	}
	return false;
}

// TMEM allocation by one full warp; the base address is written to *slot.
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t cols)
{
	asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_addr(slot)), "r"(cols)
	             : "memory");
	asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t cols)
{
	asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(cols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

// D[tmem] (+)= A[smem] x B[smem]^T, issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool accumulate)
{
	asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
	             " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
	             ::"r"(d_tmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(uint32_t(accumulate))
	             : "memory");
}

// Arrives on the barrier once every MMA issued so far by this thread is done.
__device__ __forceinline__ void mma_commit(uint64_t *bar)
{
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(smem_addr(bar))
	             : "memory");
}

// 32 consecutive 32-bit TMEM columns of the warp's 32 lanes.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32])
{
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
	             "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
	             : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
	               "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
	               "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
	               "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
	             : "r"(taddr));
	asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}

// 4-D TMA tile load into shared memory, completing on `bar` (transaction bytes).
__device__ __forceinline__ void tma_load_4d(void *dst, const void *tmap, uint64_t *bar, int32_t c0, int32_t c1, int32_t c2,
                                            int32_t c3)
{
	asm volatile("cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];\n"
	             ::"r"(smem_addr(dst)), "l"(tmap), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_addr(bar))
	             : "memory");
}

// Byte offset of element (row, k) of a K-major BF16 tile stored with 64-byte
// swizzle (rows of 32 elements).
__host__ __device__ constexpr uint32_t swz64_offset(uint32_t row, uint32_t k)
{
	return row * 64u + ((((k >> 3) ^ (row >> 1)) & 3u) << 4) + (k & 7u) * 2u;
}

// Byte offset in the no-swizzle canonical layout with 8x8 core matrices,
// LBO between K-neighbours and SBO between row groups.
__host__ __device__ constexpr uint32_t canon_offset(uint32_t row, uint32_t k, uint32_t lbo, uint32_t sbo)
{
	return (row >> 3) * sbo + (k >> 3) * lbo + (row & 7u) * 16u + (k & 7u) * 2u;
}
} // namespace pgs_umma
