// mbarrier and bulk asynchronous copy (TMA engine, non-tensor form) helpers
// in inline PTX, shared by the collision, table-staging and k-NN kernels.
#pragma once

#include <cstdint>

namespace mrmg {

// try_wait polls before a wait gives up (each poll after the 32nd sleeps
// ~128 ns, so a limit is reached after roughly half a second)
constexpr long long kWaitSpins = 1ll << 22;

// bytes one staged table copy may move (below the mbarrier's transaction
// count limit of 2^20 - 1 and any shared-memory allocation)
constexpr uint32_t kStageMaxBytes = 1u << 19;

// table copies that did not complete within the wait limit (the kernel then
// copied the tables with plain loads): one counter per translation unit,
// summed by mrmg_table_stage_timeouts
static __device__ unsigned int g_stage_timeouts = 0;

static __device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

static __device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(bar)), "r"(count) : "memory");
}
static __device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(bar)), "r"(bytes) : "memory");
}
static __device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(su32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait: false when the barrier did not complete within the limit
static __device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (long long i = 0; i < kWaitSpins; i++) {
    if (mbar_try_wait(bar, parity)) return true;
    if (i > 32) __nanosleep(128);
  }
  return false;
}
// bulk asynchronous copy global -> shared, completing on `bar`; both
// addresses 16-byte aligned, bytes a multiple of 16
static __device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(su32(dst)),
               "l"(src), "r"(bytes), "r"(su32(bar))
               : "memory");
}
static __device__ __forceinline__ void fence_barrier_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
static __device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// whether a staged copy of `bytes` from src to dst meets the bulk copy's
// rules (16-byte aligned addresses, a multiple of 16 bytes, within the limit)
static __device__ __forceinline__ bool bulk_ok(const void* dst, const void* src, size_t bytes) {
  return bytes > 0 && bytes <= kStageMaxBytes && (bytes & 15) == 0 && (su32(dst) & 15u) == 0 &&
         ((uintptr_t)src & 15) == 0;
}

// Copies `bytes` of a table image from global memory to this CTA's shared
// memory at `dst` with one bulk asynchronous copy per 32 KB piece, issued by
// thread 0 on one mbarrier that every thread then waits on.  Requirements
// (bulk_ok): src and dst 16-byte aligned, bytes a multiple of 16 and at
// most kStageMaxBytes; every thread of the CTA
// calls it, before anything else in the CTA touches `dst`.  Returns false
// when the copy did not complete within the wait limit: the caller then
// copies the tables itself and calls stage_bulk_drain.
static __device__ __forceinline__ bool stage_bulk(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    fence_barrier_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_expect_tx(bar, bytes);
    for (uint32_t o = 0; o < bytes; o += 32768u) {
      const uint32_t b = bytes - o < 32768u ? bytes - o : 32768u;
      bulk_g2s((unsigned char*)dst + o, (const unsigned char*)src + o, b, bar);
    }
  }
  return mbar_wait(bar, 0);
}
// after a timed-out stage_bulk: counts the timeout and waits (bounded) for
// the copy still in flight, so that none outlives the CTA
static __device__ __forceinline__ void stage_bulk_drain(uint64_t* bar) {
  if (threadIdx.x == 0) atomicAdd(&g_stage_timeouts, 1u);
  mbar_wait(bar, 0);
}

}  // namespace mrmg
