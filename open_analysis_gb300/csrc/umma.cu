// BF16 GEMM on the fifth-generation tensor cores (tcgen05) for the surrogate's layers, grouped:
//   C_g (M x N) = A_g (M x K) . B_g^T   for g = 0 .. groups-1,
// A_g row-major M x K and B_g row-major N x K (both K-contiguous), the groups a fixed number of
// elements apart (the ensemble's members side by side). FP32 accumulation in tensor memory (TMEM);
// the fused epilogue of oafdtd_mlp_gemm (bias, ReLU or tanh, or their derivatives) writes FP32
// and/or BF16 results and, optionally, the BF16 result transposed (N x M), which the next layer's
// weight gradient reads K-contiguous.
//
// A persistent kernel, one CTA per SM, walking the tiles (group, 128-row block, BN-column block)
// of every group with a stride of the grid size. Ten warps with fixed roles:
//   warp 0, one lane: the producer. Each K step (64 elements, 128 bytes) of a tile's A and B
//     arrives by one TMA tensor copy each (cp.async.bulk.tensor, 3-D maps over rows, K and the
//     group, 128-byte swizzle) into a 4-stage shared-memory ring, completing on the stage's
//     "full" mbarrier; the producer refills a stage once its "empty" mbarrier says the MMAs have
//     read it. It runs ahead across tile boundaries.
//   warp 1: allocates 2 x BN columns of TMEM (two accumulators); one lane issues the MMAs
//     (tcgen05.mma.cta_group::1.kind::f16, M 128, N BN, K 16, four per stage) into the
//     accumulator of the tile's parity, commits each stage to its "empty" mbarrier and the
//     finished tile to the accumulator's "full" mbarrier, after waiting for the epilogue to
//     have drained that accumulator (its "empty" mbarrier).
//   warps 2-9: the epilogue. Warp w reads TMEM lanes 32 (w mod 4) .. +31 (a warp may only reach
//     its quarter of the lanes), one row of the tile per thread, and half of the columns, 32 at a
//     time (tcgen05.ld 32x32b.x32). It releases the accumulator after its last load, applies the
//     epilogue, stages the 32 x 32 chunk in shared memory in the TMA's swizzled layout and stores
//     it with cp.async.bulk.tensor (FP32: 128-byte swizzle; BF16: 64-byte; transposed BF16:
//     plain rows of 64 bytes), so the epilogue of one tile overlaps the MMAs of the next.
// Every mbarrier wait is bounded (about two seconds, and a poll count); a wait that gives up sets
// the caller's status word and a flag the other roles poll, every role leaves its loop, copies
// and MMAs in flight are waited for (bounded again) and TMEM is freed, so no launch hangs.

#include <cuda.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include <string>

#include "oafdtd_internal.cuh"

namespace oafdtd {

namespace {

constexpr int kUM = 128, kUK = 64, kUStages = 4, kEpiWarps = 8;
constexpr int kUThreads = 32 * (2 + kEpiWarps);
constexpr unsigned long long kUWaitNs = 2000000000ull;
constexpr unsigned kUPolls = 1u << 28;

struct UmmaArgs {
  const float* bias;          // per column and group (nullable)
  const __nv_bfloat16* mask;  // epilogues 2 and 4: layout of C (ldc, group stride sC)
  long long sBias, sC;
  int M, N, K, ldc, act, groups;
  int has32, has16, has16t;
  int* status;
};

// One stage: the A and B tiles as the 128-byte-swizzled TMA boxes leave them, 1024-byte aligned
// (the swizzle repeats every 8 rows of 128 bytes).
template <int BN>
struct __align__(1024) UStage {
  __nv_bfloat16 a[kUM * kUK];
  __nv_bfloat16 b[BN * kUK];
};

// One epilogue warp's 32 x 32 chunk in the layouts its three TMA store maps read.
struct __align__(1024) EpiStage {
  float c32[32 * 32];            // rows of 128 bytes, 128-byte swizzle
  __nv_bfloat16 c16[32 * 32];    // rows of 64 bytes, 64-byte swizzle
  __nv_bfloat16 c16t[32 * 32];   // transposed: row n holds the chunk's 32 rows m, no swizzle
};

__device__ __forceinline__ uint32_t saddr(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void ubar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(saddr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void ubar_expect(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(saddr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void ubar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(saddr(bar)) : "memory");
}
__device__ __forceinline__ bool ubar_try(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(saddr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ unsigned long long unow() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
  return t;
}
// Bounded wait for the phase of the given parity: false when the time or poll limit ran out, or
// when another role raised the CTA's failure flag (null: not polled).
__device__ __noinline__ bool ubar_wait(uint64_t* bar, unsigned parity, volatile int* failed) {
  const unsigned long long t0 = unow();
  for (unsigned n = 0; n < kUPolls; ++n) {
    if (ubar_try(bar, parity)) return true;
    if ((n & 63u) == 63u && (unow() - t0 > kUWaitNs || (failed && *failed))) return false;
  }
  return false;
}
__device__ __forceinline__ void utma_load(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];\n" ::"r"(saddr(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(saddr(bar))
      : "memory");
}
__device__ __forceinline__ void utma_store(const CUtensorMap* map, const void* src, int x, int y, int z) {
  asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%1, %2, %3}], [%4];\n" ::"l"(
                   reinterpret_cast<unsigned long long>(map)),
               "r"(x), "r"(y), "r"(z), "r"(saddr(src))
               : "memory");
}
__device__ __forceinline__ void prefetch_map(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<unsigned long long>(map)) : "memory");
}

// Shared-memory matrix descriptor of a K-major operand tile with 128-byte swizzle: start address,
// stride between 8-row groups 1024 bytes, descriptor version 1, layout SWIZZLE_128B.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;              // leading byte offset (not used by swizzled K-major layouts)
  d |= (uint64_t)(1024 >> 4) << 32;    // stride byte offset
  d |= (uint64_t)1 << 46;              // version
  d |= (uint64_t)2 << 61;              // SWIZZLE_128B
  return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, N and M.
template <int BN>
__host__ __device__ constexpr uint32_t idesc() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(kUM >> 4) << 24);
}

__device__ __forceinline__ void umma(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t id, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
      "l"(adesc), "l"(bdesc), "r"(id), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void ucommit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(saddr(bar))
               : "memory");
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}

__device__ __forceinline__ void raise_failure(volatile int* failed, int* status) {
  *failed = 1;
  if (status) atomicOr(status, 1);
}

template <int BN>
__global__ void __launch_bounds__(kUThreads, 1)
    umma_gemm_kernel(const __grid_constant__ UmmaArgs g, const __grid_constant__ CUtensorMap amap,
                     const __grid_constant__ CUtensorMap bmap, const __grid_constant__ CUtensorMap c32map,
                     const __grid_constant__ CUtensorMap c16map, const __grid_constant__ CUtensorMap c16tmap) {
  extern __shared__ unsigned char umma_raw[];
  __shared__ uint64_t full[kUStages], empty[kUStages], tfull[2], tempty[2], done;
  __shared__ uint32_t tmem_base;
  __shared__ int failed_sh, consumed_sh;
  volatile int* failed = &failed_sh;
  unsigned char* base = umma_raw + ((1024u - (saddr(umma_raw) & 1023u)) & 1023u);
  UStage<BN>* st = reinterpret_cast<UStage<BN>*>(base);
  EpiStage* ep = reinterpret_cast<EpiStage*>(base + kUStages * sizeof(UStage<BN>));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int MT = g.M / kUM, NT = g.N / BN, KT = g.K / kUK;
  const int tiles = g.groups * MT * NT;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kUStages; ++s) {
      ubar_init(&full[s], 1);
      ubar_init(&empty[s], 1);
    }
    for (int a = 0; a < 2; ++a) {
      ubar_init(&tfull[a], 1);
      ubar_init(&tempty[a], kEpiWarps);
    }
    ubar_init(&done, 1);
    failed_sh = 0;
    consumed_sh = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    prefetch_map(&amap);
    prefetch_map(&bmap);
  }
  if (warp == 1) {  // two accumulators of 128 lanes x BN FP32 columns
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(saddr(&tmem_base)),
                 "r"(2 * BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_base;
  int issued = 0;  // the producer's count of K steps whose copies it issued
  if (warp == 0) {
    if (lane == 0) {
      constexpr unsigned kStageBytes = (kUM + BN) * kUK * sizeof(__nv_bfloat16);
      for (int tile = blockIdx.x; tile < tiles && !*failed; tile += gridDim.x) {
        const int nt = tile % NT, mt = (tile / NT) % MT, gi = tile / (NT * MT);
        int kb = 0;
        for (; kb < KT; ++kb, ++issued) {
          const int s = issued % kUStages;
          const unsigned r = (unsigned)(issued / kUStages);
          if (!ubar_wait(&empty[s], (r & 1u) ^ 1u, failed)) break;
          ubar_expect(&full[s], kStageBytes);
          utma_load(st[s].a, &amap, &full[s], kb * kUK, mt * kUM, gi);
          utma_load(st[s].b, &bmap, &full[s], kb * kUK, nt * BN, gi);
        }
        if (kb < KT) {
          raise_failure(failed, g.status);
          break;
        }
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0) {
      int it = 0, t = 0;
      bool ok = true;
      for (int tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x, ++t) {
        const int acc = t & 1;
        const unsigned u = (unsigned)(t >> 1);
        ok = ubar_wait(&tempty[acc], (u & 1u) ^ 1u, failed);
        if (!ok) break;
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const uint32_t d = tmem + (uint32_t)(acc * BN);
        for (int kb = 0; kb < KT; ++kb, ++it) {
          const int s = it % kUStages;
          ok = ubar_wait(&full[s], (unsigned)((it / kUStages) & 1), failed);
          if (!ok) break;
          asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
          const uint32_t a0 = saddr(st[s].a), b0 = saddr(st[s].b);
#pragma unroll
          for (int kk = 0; kk < kUK / 16; ++kk)  // K 16 per MMA: 32 bytes further along the swizzled rows
            umma(d, sw128_desc(a0 + 32u * kk), sw128_desc(b0 + 32u * kk), idesc<BN>(), (kb | kk) != 0 ? 1u : 0u);
          ucommit(&empty[s]);  // arrives when these MMAs have read the stage
        }
        if (!ok) break;
        ucommit(&tfull[acc]);  // arrives when the tile's MMAs have completed
      }
      *(volatile int*)&consumed_sh = it;
      if (!ok) raise_failure(failed, g.status);
      ucommit(&done);  // every MMA issued so far has completed before TMEM is freed
      ubar_wait(&done, 0u, nullptr);
    }
    __syncwarp();
  } else {
    const int q = warp & 3, half = (warp - 2) >> 2;
    EpiStage& es = ep[warp - 2];
    int t = 0;
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x, ++t) {
      const int nt = tile % NT, mt = (tile / NT) % MT, gi = tile / (NT * MT);
      const int acc = t & 1;
      // warp-uniform outcome: the TMEM loads below are warp-collective
      const bool ok = __all_sync(0xffffffffu, ubar_wait(&tfull[acc], (unsigned)((t >> 1) & 1), failed));
      if (!ok) {
        if (lane == 0) raise_failure(failed, g.status);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      const int row0 = mt * kUM + 32 * q;  // the chunk's first row within the group
      const int row = row0 + lane;         // this thread's row
      for (int c = half * (BN / 2); c < (half + 1) * (BN / 2); c += 32) {
        uint32_t r[32];
        tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(acc * BN + c), r);
        if (c + 32 == (half + 1) * (BN / 2)) {  // the warp's last load from this accumulator
          asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
          __syncwarp();
          if (lane == 0) ubar_arrive(&tempty[acc]);
        }
        const int col0 = nt * BN + c;  // the chunk's first column
        const float bl = g.bias ? g.bias[gi * g.sBias + col0 + lane] : 0.f;
        float v[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]) + __shfl_sync(0xffffffffu, bl, j);
        if (g.act == 1) {
#pragma unroll
          for (int j = 0; j < 32; ++j) v[j] = v[j] > 0.f ? v[j] : 0.f;
        } else if (g.act == 3) {
#pragma unroll
          for (int j = 0; j < 32; ++j) v[j] = tanhf(v[j]);
        } else if (g.act == 2 || g.act == 4) {
          const uint4* mp = reinterpret_cast<const uint4*>(g.mask + gi * g.sC + (long long)row * g.ldc + col0);
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const uint4 w = mp[k];
            const uint32_t ww[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
            for (int h = 0; h < 4; ++h) {
              const __nv_bfloat162 p = *reinterpret_cast<const __nv_bfloat162*>(&ww[h]);
              const float m0 = __low2float(p), m1 = __high2float(p);
              const int j = 8 * k + 2 * h;
              if (g.act == 2) {
                if (!(m0 > 0.f)) v[j] = 0.f;
                if (!(m1 > 0.f)) v[j + 1] = 0.f;
              } else {
                v[j] *= 1.f - m0 * m0;
                v[j + 1] *= 1.f - m1 * m1;
              }
            }
          }
        }
        // the previous chunk's stores have read the staging buffers
        if (lane == 0) asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory");
        __syncwarp();
        if (g.has32) {
          unsigned char* rowp = reinterpret_cast<unsigned char*>(es.c32) + lane * 128;
#pragma unroll
          for (int k = 0; k < 8; ++k)
            *reinterpret_cast<float4*>(rowp + ((k ^ (lane & 7)) << 4)) =
                make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
        }
        if (g.has16) {
          unsigned char* rowp = reinterpret_cast<unsigned char*>(es.c16) + lane * 64;
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            uint4 w;
            __nv_bfloat162 p0 = __floats2bfloat162_rn(v[8 * k], v[8 * k + 1]);
            __nv_bfloat162 p1 = __floats2bfloat162_rn(v[8 * k + 2], v[8 * k + 3]);
            __nv_bfloat162 p2 = __floats2bfloat162_rn(v[8 * k + 4], v[8 * k + 5]);
            __nv_bfloat162 p3 = __floats2bfloat162_rn(v[8 * k + 6], v[8 * k + 7]);
            w.x = *reinterpret_cast<uint32_t*>(&p0);
            w.y = *reinterpret_cast<uint32_t*>(&p1);
            w.z = *reinterpret_cast<uint32_t*>(&p2);
            w.w = *reinterpret_cast<uint32_t*>(&p3);
            *reinterpret_cast<uint4*>(rowp + ((k ^ ((lane >> 1) & 3)) << 4)) = w;
          }
        }
        if (g.has16t) {
#pragma unroll
          for (int j = 0; j < 32; ++j) es.c16t[j * 32 + lane] = __float2bfloat16(v[j]);
        }
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        __syncwarp();
        if (lane == 0) {
          if (g.has32) utma_store(&c32map, es.c32, col0, row0, gi);
          if (g.has16) utma_store(&c16map, es.c16, col0, row0, gi);
          if (g.has16t) utma_store(&c16tmap, es.c16t, row0, col0, gi);
          asm volatile("cp.async.bulk.commit_group;\n" ::: "memory");
        }
      }
    }
    if (lane == 0) asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory");
    __syncwarp();
  }
  __syncthreads();
  if (warp == 0 && lane == 0) {
    // after a failure: copies issued and never consumed land before the CTA exits (bounded)
    const int consumed = *(volatile int*)&consumed_sh;
    for (int k = consumed; k < issued; ++k) ubar_wait(&full[k % kUStages], (unsigned)((k / kUStages) & 1), nullptr);
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  if (warp == 1)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(2 * BN) : "memory");
}

// 3-D tensor map of `groups` row-major matrices (rows x cols, leading dimension ld elements,
// `gstride` elements apart) with a box of box_cols x box_rows.
bool group_map(CUtensorMap* m, CUtensorMapDataType dt, int esize, const void* base, int rows, int cols, int ld,
               long long gstride, int groups, int box_cols, int box_rows, CUtensorMapSwizzle sw, const char* what,
               std::string* why) {
  const cuuint64_t dims[3] = {(cuuint64_t)cols, (cuuint64_t)rows, (cuuint64_t)groups};
  const long long gs = groups > 1 ? gstride : (long long)rows * ld;
  const cuuint64_t strides[2] = {(cuuint64_t)ld * esize, (cuuint64_t)gs * esize};
  const cuuint32_t box[3] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows, 1};
  return encode_tensor_map(m, dt, 3, base, dims, strides, box, what, why, sw);
}

template <int BN>
cudaError_t launch_bn(const UmmaProblem& p, cudaStream_t s, std::string* why) {
  constexpr auto BF = CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
  CUtensorMap amap, bmap, c32map{}, c16map{}, c16tmap{};
  if (!group_map(&amap, BF, 2, p.A, p.M, p.K, p.lda, p.sA, p.groups, kUK, kUM, CU_TENSOR_MAP_SWIZZLE_128B, "A", why) ||
      !group_map(&bmap, BF, 2, p.B, p.N, p.K, p.ldb, p.sB, p.groups, kUK, BN, CU_TENSOR_MAP_SWIZZLE_128B, "B", why))
    return cudaErrorInvalidValue;
  if (p.C32 && !group_map(&c32map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, p.C32, p.M, p.N, p.ldc, p.sC, p.groups, 32, 32,
                          CU_TENSOR_MAP_SWIZZLE_128B, "C32", why))
    return cudaErrorInvalidValue;
  if (p.C16 && !group_map(&c16map, BF, 2, p.C16, p.M, p.N, p.ldc, p.sC, p.groups, 32, 32, CU_TENSOR_MAP_SWIZZLE_64B,
                          "C16", why))
    return cudaErrorInvalidValue;
  if (p.C16T && !group_map(&c16tmap, BF, 2, p.C16T, p.N, p.M, p.ldct, p.sCT, p.groups, 32, 32,
                           CU_TENSOR_MAP_SWIZZLE_NONE, "C16T", why))
    return cudaErrorInvalidValue;
  UmmaArgs g{};
  g.bias = p.bias;
  g.mask = static_cast<const __nv_bfloat16*>(p.mask);
  g.sBias = p.sBias;
  g.sC = p.sC;
  g.M = p.M, g.N = p.N, g.K = p.K, g.ldc = p.ldc, g.act = p.act, g.groups = p.groups;
  g.has32 = p.C32 != nullptr, g.has16 = p.C16 != nullptr, g.has16t = p.C16T != nullptr;
  g.status = p.status;
  const size_t bytes = sizeof(UStage<BN>) * kUStages + sizeof(EpiStage) * kEpiWarps + 1024;
  cudaError_t err = cudaFuncSetAttribute(umma_gemm_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (err != cudaSuccess) return err;
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1)
      sms = 148;
  }
  const long long tiles = (long long)p.groups * (p.M / kUM) * (p.N / BN);
  const int grid = (int)(tiles < sms ? tiles : sms);
  umma_gemm_kernel<BN><<<grid, kUThreads, bytes, s>>>(g, amap, bmap, c32map, c16map, c16tmap);
  return cudaGetLastError();
}

bool aligned16(const void* q) { return (reinterpret_cast<uintptr_t>(q) & 15) == 0; }

}  // namespace

bool umma_shape_ok(const UmmaProblem& p) {
  const bool tiles = p.M > 0 && p.N > 0 && p.K > 0 && p.M % kUM == 0 && p.N % 64 == 0 && p.K % kUK == 0 &&
                     p.groups >= 1;
  const bool lds = p.lda % 8 == 0 && p.ldb % 8 == 0 && p.ldc % 8 == 0 && (!p.C16T || p.ldct % 8 == 0) &&
                   p.lda >= p.K && p.ldb >= p.K && p.ldc >= p.N && (!p.C16T || p.ldct >= p.M);
  const bool strides = p.groups == 1 || (p.sA % 8 == 0 && p.sB % 8 == 0 && p.sC % 8 == 0 && p.sCT % 8 == 0 &&
                                         p.sA >= (long long)p.M * p.lda && p.sB >= (long long)p.N * p.ldb &&
                                         p.sC >= (long long)p.M * p.ldc && (!p.C16T || p.sCT >= (long long)p.N * p.ldct));
  const bool ptrs = aligned16(p.A) && aligned16(p.B) && aligned16(p.C32) && aligned16(p.C16) && aligned16(p.C16T) &&
                    aligned16(p.mask);
  return tiles && lds && strides && ptrs && p.beta == 0.f;
}

cudaError_t launch_umma_gemm(const UmmaProblem& p, cudaStream_t s, std::string* why) {
  // 128-column tiles unless they would leave most SMs without a tile
  const long long tiles128 = p.N % 128 == 0 ? (long long)p.groups * (p.M / kUM) * (p.N / 128) : 0;
  if (tiles128 >= 96) return launch_bn<128>(p, s, why);
  return launch_bn<64>(p, s, why);
}

cudaError_t preload_umma() {
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, reinterpret_cast<const void*>(umma_gemm_kernel<128>));
  if (e != cudaSuccess) return e;
  return cudaFuncGetAttributes(&fa, reinterpret_cast<const void*>(umma_gemm_kernel<64>));
}

static_assert(sizeof(UStage<128>) == (kUM + 128) * kUK * 2, "stage tiles are contiguous and 1024-byte multiples");
static_assert(sizeof(UStage<64>) == (kUM + 64) * kUK * 2, "stage tiles are contiguous and 1024-byte multiples");
static_assert(sizeof(EpiStage) == 8192, "epilogue staging: three 1024-byte aligned chunks");
static_assert(kUK * sizeof(__nv_bfloat16) == 128, "one K step is one 128-byte swizzle row");
static_assert(sizeof(UStage<128>) * kUStages + sizeof(EpiStage) * kEpiWarps + 1024 <= 232448,
              "shared memory within the 227 KB a CTA may use");

}  // namespace oafdtd
