// BF16 GEMM on the fifth-generation tensor cores (tcgen05) for the surrogate's layers:
//   C (M x N) = A (M x K) . B^T, with A row-major M x K and B row-major N x K (both K-contiguous),
// FP32 accumulation in tensor memory (TMEM), and the fused epilogue of oafdtd_mlp_gemm (bias, ReLU
// or tanh, or their derivatives) writing FP32 and/or BF16 results and, optionally, the BF16 result
// transposed (N x M), which the next layer's weight gradient reads K-contiguous.
//
// One CTA of 128 threads computes a 128 x 128 tile of C. K advances 64 elements (128 bytes) at a
// time through a 4-stage shared-memory ring: each stage's A and B tiles arrive by one TMA tensor
// copy each (cp.async.bulk.tensor, 128-byte swizzle), completing on the stage's "full" mbarrier.
// One thread issues the copies and the MMAs (tcgen05.mma.cta_group::1.kind::f16, M 128, N 128,
// K 16, four per stage, the operands addressed by shared-memory descriptors); tcgen05.commit
// arrives on the stage's "empty" mbarrier when the stage's MMAs have read it, and on the "done"
// mbarrier after the last. The four warps then read the accumulator out of TMEM (each its quarter
// of the 128 lanes: one row of C per thread, 32 columns per tcgen05.ld) and apply the epilogue.
// Every mbarrier wait is bounded (about two seconds); a wait that gives up sets the caller's
// status word and the CTA skips what depended on it, so no launch hangs.

#include <cuda.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include <string>

#include "oafdtd_internal.cuh"

namespace oafdtd {

namespace {

constexpr int kUM = 128, kUN = 128, kUK = 64, kUStages = 4;
constexpr unsigned long long kUWaitNs = 2000000000ull;
constexpr unsigned kUPolls = 1u << 28;

struct UmmaArgs {
  float* C32;             // FP32 result (nullable), ldc
  __nv_bfloat16* C16;     // BF16 result (nullable), ldc
  __nv_bfloat16* C16T;    // BF16 result transposed, N x M (nullable), ldct
  const float* bias;      // per column (nullable)
  const __nv_bfloat16* mask;  // epilogues 2 and 4, layout of C (ldc)
  int M, N, K, ldc, ldct, act;
  float beta;
  int* status;
};

// One stage: the A and B tiles as the 128-byte-swizzled TMA boxes leave them, 1024-byte aligned
// (the swizzle repeats every 8 rows of 128 bytes).
struct __align__(1024) UStage {
  __nv_bfloat16 a[kUM * kUK];
  __nv_bfloat16 b[kUN * kUK];
};

__device__ __forceinline__ uint32_t saddr(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void ubar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(saddr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void ubar_expect(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(saddr(bar)), "r"(bytes) : "memory");
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
// Bounded wait for the phase of the given parity: false when the time or poll limit ran out.
__device__ __noinline__ bool ubar_wait(uint64_t* bar, unsigned parity) {
  const unsigned long long t0 = unow();
  for (unsigned n = 0; n < kUPolls; ++n) {
    if (ubar_try(bar, parity)) return true;
    if ((n & 63u) == 63u && unow() - t0 > kUWaitNs) return false;
  }
  return false;
}
__device__ __forceinline__ void utma2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::
          "r"(saddr(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(saddr(bar))
      : "memory");
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
constexpr uint32_t kUIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kUN >> 3) << 17) |
                             ((uint32_t)(kUM >> 4) << 24);

__device__ __forceinline__ void umma(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void ucommit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(saddr(bar))
               : "memory");
}

__device__ __forceinline__ float epilogue(const UmmaArgs& g, float v, int m, int n) {
  if (g.bias) v += g.bias[n];
  if (g.act == 1) v = v > 0.f ? v : 0.f;
  if (g.act == 2 && !(__bfloat162float(g.mask[(long long)m * g.ldc + n]) > 0.f)) v = 0.f;
  if (g.act == 3) v = tanhf(v);
  if (g.act == 4) {
    const float a = __bfloat162float(g.mask[(long long)m * g.ldc + n]);
    v *= 1.f - a * a;
  }
  return v;
}

__global__ void __launch_bounds__(128, 1)
    umma_gemm_kernel(const __grid_constant__ UmmaArgs g, const __grid_constant__ CUtensorMap amap,
                     const __grid_constant__ CUtensorMap bmap) {
  extern __shared__ unsigned char umma_raw[];
  __shared__ uint64_t full[kUStages], empty[kUStages], done;
  __shared__ uint32_t tmem_base;
  __shared__ int failed;
  UStage* st = reinterpret_cast<UStage*>(umma_raw + ((1024u - (saddr(umma_raw) & 1023u)) & 1023u));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * kUM, n0 = blockIdx.x * kUN;
  const int KT = g.K / kUK;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kUStages; ++s) {
      ubar_init(&full[s], 1);
      ubar_init(&empty[s], 1);
    }
    ubar_init(&done, 1);
    failed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<unsigned long long>(&amap)) : "memory");
    asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<unsigned long long>(&bmap)) : "memory");
  }
  if (warp == 0) {  // the accumulator: 128 lanes x 128 FP32 columns of tensor memory
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(saddr(&tmem_base)),
                 "r"(kUN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_base;
  if (threadIdx.x == 0) {
    constexpr unsigned kStageBytes = (kUM + kUN) * kUK * sizeof(__nv_bfloat16);
    int issued = 0, consumed = 0;
    bool ok = true;
    for (; issued < kUStages && issued < KT; ++issued) {
      UStage& s = st[issued];
      ubar_expect(&full[issued], kStageBytes);
      utma2d(s.a, &amap, &full[issued], issued * kUK, m0);
      utma2d(s.b, &bmap, &full[issued], issued * kUK, n0);
    }
    for (int kt = 0; kt < KT; ++kt) {
      const int s = kt % kUStages;
      const unsigned ph = (unsigned)((kt / kUStages) & 1);
      ok = ubar_wait(&full[s], ph);
      if (!ok) break;
      consumed = kt + 1;
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      const uint32_t a0 = saddr(st[s].a), b0 = saddr(st[s].b);
#pragma unroll
      for (int kk = 0; kk < kUK / 16; ++kk)  // K 16 per MMA: 32 bytes further along the swizzled rows
        umma(tmem, sw128_desc(a0 + 32u * kk), sw128_desc(b0 + 32u * kk), kUIdesc, (kt | kk) != 0 ? 1u : 0u);
      ucommit(&empty[s]);  // arrives when these MMAs have read the stage
      if (issued < KT) {
        ok = ubar_wait(&empty[s], ph);
        if (!ok) break;
        UStage& nx = st[s];
        ubar_expect(&full[s], kStageBytes);
        utma2d(nx.a, &amap, &full[s], issued * kUK, m0);
        utma2d(nx.b, &bmap, &full[s], issued * kUK, n0);
        ++issued;
      }
    }
    ucommit(&done);  // arrives when every MMA issued so far has completed
    if (!ok) {
      failed = 1;
      if (g.status) atomicOr(g.status, 1);
      // copies issued and not consumed land before the CTA exits (bounded)
      for (int kt = consumed; kt < issued; ++kt) ubar_wait(&full[kt % kUStages], (unsigned)((kt / kUStages) & 1));
    }
  }
  const bool ok_done = ubar_wait(&done, 0u);
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (ok_done && !failed) {
    const int m = m0 + 32 * warp + lane;  // this thread's row of the tile (its TMEM lane)
    for (int c0 = 0; c0 < kUN; c0 += 32) {
      uint32_t r[32];
      const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
          "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
            "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
            "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      if (m < g.M) {
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int n = n0 + c0 + j;
          if (n >= g.N) continue;
          const float v = epilogue(g, __uint_as_float(r[j]), m, n);
          const long long o = (long long)m * g.ldc + n;
          if (g.C32) g.C32[o] = g.beta != 0.f ? v + g.beta * g.C32[o] : v;
          if (g.C16) g.C16[o] = __float2bfloat16(v);
          if (g.C16T) g.C16T[(long long)n * g.ldct + m] = __float2bfloat16(v);
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kUN) : "memory");
}

// 2-D BF16 tensor map of a row-major rows x K matrix (leading dimension ld elements) with a
// 64 x 128 box and 128-byte swizzle.
bool bf16_map(CUtensorMap* m, const void* base, int rows, int K, int ld, std::string* why) {
  const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  const cuuint32_t box[2] = {(cuuint32_t)kUK, (cuuint32_t)kUM};
  return encode_tensor_map(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, "umma operand", why,
                           CU_TENSOR_MAP_SWIZZLE_128B);
}

}  // namespace

bool umma_shape_ok(int M, int N, int K, int lda, int ldb, const void* A, const void* B) {
  return M > 0 && N > 0 && K > 0 && M % kUM == 0 && N % kUN == 0 && K % kUK == 0 && lda % 8 == 0 && ldb % 8 == 0 &&
         (reinterpret_cast<uintptr_t>(A) & 15) == 0 && (reinterpret_cast<uintptr_t>(B) & 15) == 0;
}

cudaError_t launch_umma_gemm(const void* A, const void* B, float* C32, void* C16, void* C16T, const float* bias,
                             const void* mask, int M, int N, int K, int lda, int ldb, int ldc, int ldct, int act,
                             float beta, int* status, cudaStream_t s, std::string* why) {
  CUtensorMap amap, bmap;
  if (!bf16_map(&amap, A, M, K, lda, why) || !bf16_map(&bmap, B, N, K, ldb, why)) return cudaErrorInvalidValue;
  UmmaArgs g{C32,
             static_cast<__nv_bfloat16*>(C16),
             static_cast<__nv_bfloat16*>(C16T),
             bias,
             static_cast<const __nv_bfloat16*>(mask),
             M,
             N,
             K,
             ldc,
             ldct,
             act,
             beta,
             status};
  const size_t bytes = sizeof(UStage) * kUStages + 1024;
  cudaError_t err = cudaFuncSetAttribute(umma_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (err != cudaSuccess) return err;
  umma_gemm_kernel<<<dim3(N / kUN, M / kUM), 128, bytes, s>>>(g, amap, bmap);
  return cudaGetLastError();
}

cudaError_t preload_umma() {
  cudaFuncAttributes fa;
  return cudaFuncGetAttributes(&fa, reinterpret_cast<const void*>(umma_gemm_kernel));
}

static_assert(sizeof(UStage) == (kUM + kUN) * kUK * 2, "stage tiles are contiguous and 1024-byte multiples");
static_assert(kUK * sizeof(__nv_bfloat16) == 128, "one K step is one 128-byte swizzle row");

}  // namespace oafdtd
