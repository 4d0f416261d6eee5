// Bulk-async (TMA 1D) copy and mbarrier primitives for sm_90+ in inline PTX, with bounded waits.
#pragma once
#include <stdint.h>

namespace fx3d {

// error codes a kernel may record in its error word (first one wins)
enum : int { KERR_NONE = 0, KERR_MBARRIER_TIMEOUT = 1 };
// iteration limit of an mbarrier wait; each try_wait suspends for at most a hardware time slice,
// so this bounds a wait to well under a second for copies that normally finish in microseconds
constexpr uint32_t MBAR_SPIN_LIMIT = 1u<<22;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, const uint32_t count) {
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(bar)), "r"(count) : "memory");
}
// make an initialised mbarrier visible to the async proxy and the other threads
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// order this thread's generic-proxy shared-memory writes before later async-proxy (bulk copy) reads
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, const uint32_t bytes) {
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, const uint32_t phase) {
	uint32_t ok;
	asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
	             : "=r"(ok) : "r"(smem_u32(bar)), "r"(phase) : "memory");
	return ok!=0u;
}
// bounded wait for phase `phase`; on timeout records KERR_MBARRIER_TIMEOUT and returns false
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, const uint32_t phase, int* err) {
	for(uint32_t it=0u; it<MBAR_SPIN_LIMIT; it++) if(mbar_try_wait(bar, phase)) return true;
	if(err) atomicCAS(err, KERR_NONE, KERR_MBARRIER_TIMEOUT);
	return false;
}

// global -> shared bulk copy completing on `bar` (addresses 16-byte aligned, bytes a multiple of 16)
__device__ __forceinline__ void bulk_load(void* dst_smem, const void* src_gmem, const uint32_t bytes, uint64_t* bar) {
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
	             :: "r"(smem_u32(dst_smem)), "l"(src_gmem), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}
// shared -> global bulk copy in the current bulk group
__device__ __forceinline__ void bulk_store(void* dst_gmem, const void* src_smem, const uint32_t bytes) {
	asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" :: "l"(dst_gmem), "r"(smem_u32(src_smem)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// wait until every committed bulk store has finished reading shared memory
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// wait until at most one committed bulk-store group is still reading shared memory
__device__ __forceinline__ void bulk_wait_read_but1() { asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory"); }
// wait until every committed bulk store is complete (writes visible)
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// per-thread asynchronous global -> shared copies of 4 or 8 bytes (both addresses aligned to the size);
// a thread waits only for its own groups, so a thread that reads back only what it copied itself
// needs no block-wide barrier
__device__ __forceinline__ void cp_async_4(const uint32_t dst_smem, const void* src_gmem) {
	asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" :: "r"(dst_smem), "l"(src_gmem) : "memory");
}
__device__ __forceinline__ void cp_async_8(const uint32_t dst_smem, const void* src_gmem) {
	asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" :: "r"(dst_smem), "l"(src_gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// wait until at most N of this thread's most recent groups are still in flight
template<int N> __device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" :: "n"(N) : "memory"); }

} // namespace fx3d
