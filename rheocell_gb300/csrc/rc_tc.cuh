// Blackwell tensor-core building blocks (inline PTX): tcgen05 MMA with
// operands in shared memory and the accumulator in tensor memory (TMEM),
// mbarrier completion, TMEM loads.  Used by the network's convolutions.
//
// Operand layout: K-major, no swizzle.  A "core matrix" is 8 rows of 16
// bytes (8 bf16 along K) stored contiguously (128 B).  An operand tile of
// R rows x 16 K-elements is two core-matrix columns: SBO is the byte distance
// between row groups of 8, LBO the distance between the two 8-element K
// halves.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace rc {

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t) __cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor (tcgen05): start address, leading and
// stride byte offsets (all in 16-byte units), descriptor version 1, no
// swizzle.
__device__ __forceinline__ uint64_t tc_sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
	return (uint64_t) ((addr >> 4) & 0x3FFFu) | ((uint64_t) ((lbo >> 4) & 0x3FFFu) << 16) |
	       ((uint64_t) ((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor, kind::f16: D f32 (bits 4-5 = 1), A and B bf16
// (bits 7-9 = 1, 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
constexpr uint32_t tc_idesc_bf16(uint32_t M, uint32_t N) {
	return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

// TMEM allocation of `ncols` columns (a power of two >= 32) by one whole
// warp; the base address is written to *holder (shared memory).
__device__ __forceinline__ void tc_alloc(uint32_t *holder, uint32_t ncols) {
	asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(holder)), "r"(ncols)
	             : "memory");
	asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tc_dealloc(uint32_t taddr, uint32_t ncols) {
	asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread.
__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
	asm volatile(
	    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
	    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
	    "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
	    : "memory");
}

// Arrive on the mbarrier once all previously issued MMAs of this thread complete.
__device__ __forceinline__ void tc_commit(uint64_t *mbar) {
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
	             : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t *mbar, uint32_t count) {
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
	asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *mbar, uint32_t parity) {
	uint32_t done;
	asm volatile(
	    "{\n\t.reg .pred P1;\n\tmbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n\t"
	    "selp.b32 %0, 1, 0, P1;\n\t}\n"
	    : "=r"(done)
	    : "r"(smem_u32(mbar)), "r"(parity)
	    : "memory");
	return done != 0;
}

// Wait for the phase with the given parity to complete, at most `limit`
// polls; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t parity, long long limit) {
	for(long long i = 0; i < limit; i++) {
		if(mbar_try_wait(mbar, parity)) return true;
	}
	return false;
}

// One arrival that also announces `bytes` of asynchronous transfers the
// current phase waits for.
__device__ __forceinline__ void mbar_expect_tx(uint64_t *mbar, uint32_t bytes) {
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)), "r"(bytes) : "memory");
}

// Bulk (untiled TMA) global -> shared copy completing on an mbarrier: both
// addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *smem_dst, const void *gmem_src, uint32_t bytes, uint64_t *mbar) {
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
	                 smem_u32(smem_dst)),
	             "l"(gmem_src), "r"(bytes), "r"(smem_u32(mbar))
	             : "memory");
}

// 16-byte asynchronous global -> shared copy; src_bytes = 0 writes zeros.
__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gmem_src, uint32_t src_bytes) {
	asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(smem_dst)), "l"(gmem_src), "r"(src_bytes)
	             : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
	asm volatile("cp.async.commit_group;" ::: "memory");
	asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// Generic-proxy shared-memory writes made visible to the tensor cores.
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 16 consecutive 32-bit TMEM columns of this thread's lane (32x32b shape:
// warp w reads lanes 32*(w%4) .. +31 starting at the address's lane field).
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
	uint32_t r[16];
	asm volatile(
	    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
	    "[%16];"
	    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
	      "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
	    : "r"(taddr)
	    : "memory");
	asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
	for(int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

}  // namespace rc
