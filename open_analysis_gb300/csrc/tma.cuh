// Shared-memory staging by TMA tensor copies: staged arrays, mbarriers with bounded waits, and
// the copy instructions (cp.async.bulk.tensor, completing on an mbarrier). Used by the staged
// sweeps (staged.cu) and the fused sweep (fused.cu).
#pragma once

#include "device_common.cuh"

namespace oafdtd {

// One staged array: rows x width, dense (the layout a TMA box lands in), 128-byte aligned.
template <typename T, int R, int W>
struct alignas(128) Box {
  T v[R][W];
};

__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
// One arrival (release at CTA scope) on a barrier that counts threads, not bytes.
__device__ __forceinline__ void mbar_arrive(unsigned long long* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
  return t;
}
constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s: far above any plane's copy time
constexpr unsigned long long kDrainNs = 100000000ull;  // 0.1 s per copy still in flight at abort
constexpr unsigned kWaitPolls = 1u << 28;              // hard cap on polls whatever the timer says

// Waits for the phase of the given parity; false when the time or poll limit ran out.
static __device__ __noinline__ bool mbar_wait(unsigned long long* bar, unsigned parity, unsigned long long limit_ns) {
  const unsigned long long t0 = global_ns();
  for (unsigned n = 0; n < kWaitPolls; ++n) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((n & 63u) == 63u && global_ns() - t0 > limit_ns) return false;
  }
  return false;
}
__device__ __forceinline__ void tma_load4(void* dst, const CUtensorMap* map, unsigned long long* bar, int x, int y,
                                          int z, int w) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5}], [%6];\n" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(w), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load3(void* dst, const CUtensorMap* map, unsigned long long* bar, int x, int y,
                                          int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ void prefetch_map(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<unsigned long long>(map)) : "memory");
}
// Barrier setup of the block's leader, made visible to the TMA unit before the first copy.
template <int S>
__device__ __forceinline__ void mbar_setup(unsigned long long* bar) {
#pragma unroll
  for (int s = 0; s < S; ++s) mbar_init(&bar[s], 1);
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
// Orders the block's reads of a slot (generic proxy) before the TMA writes that refill it.
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

// Plane t of a block's march uses slot t % S in phase (t / S) & 1.
template <int S>
__device__ __forceinline__ bool wait_plane(unsigned long long* bar, int t) {
  return mbar_wait(&bar[t % S], (unsigned)((t / S) & 1), kWaitNs);
}

// A wait gave up: the leader records it and waits (bounded) for the planes [t, issued) it has
// issued and not yet seen arrive, so no copy lands after the block has exited.
template <int S>
static __device__ __noinline__ void abort_march(unsigned long long* bar, int t, int issued, int* status, bool leader) {
  if (!leader) return;
  if (status) atomicOr(status, kStatusWaitTimeout);
  for (int p = t; p < issued; ++p) mbar_wait(&bar[p % S], (unsigned)((p / S) & 1), kDrainNs);
}

__device__ __forceinline__ unsigned char* align_smem(unsigned char* raw) {
  return raw + ((128u - (smem_addr(raw) & 127u)) & 127u);
}

}  // namespace oafdtd
