// Kernels of the learned S-parameter surrogate: a BF16 tensor-core GEMM with FP32 accumulation
// and fused epilogues (bias, ReLU or tanh, and their derivatives), the loss gradient, bias gradients and
// the Adam update. The surrogate's training loop (open_analysis_gb300/surrogate.py) drives them
// on device buffers it owns; nothing here allocates.
//
// GEMM: C (M x N) = op(A) (M x K) . op(B) (K x N), op = identity or transpose per the flags:
//   A: row-major M x K (ta = 0) or row-major K x M (ta = 1), leading dimension lda;
//   B: row-major K x N (tb = 0) or row-major N x K (tb = 1), leading dimension ldb.
// Main path (gemm_pipe_kernel): a block computes a BM x 64 tile (BM = 64, or 32 when 64-row tiles
// would leave most of the SMs idle) with 4 warps (2 x 2) as 16 x 8 x 16 warp MMAs (mma.sync
// m16n8k16, BF16 in, FP32 accumulate). K advances 32 at a time through a 3-stage shared-memory
// ring filled by 16-byte cp.async copies, each operand tile stored as it lies in global memory
// (K-contiguous or M/N-contiguous); ldmatrix (.trans for the M/N-contiguous layouts) turns it into
// MMA fragments. Needs M, N, K, lda, ldb multiples of 8 and 16-byte aligned operands.
// Fallback (gemm_bf16_kernel): scalar staging, any sizes and alignments, for ragged shapes.

#include <cuda_bf16.h>
#include <stdint.h>

#include "oafdtd_internal.cuh"

namespace oafdtd {

constexpr int kBM = 64, kBN = 64, kBK = 32, kPadK = kBK + 8;  // +8 BF16: rows 80 bytes apart

struct GemmArgs {
  const __nv_bfloat16* A;
  const __nv_bfloat16* B;
  float* C32;             // FP32 result (nullable)
  __nv_bfloat16* C16;     // BF16 result (nullable)
  const float* bias;      // per column (nullable)
  const __nv_bfloat16* mask;  // activations for epilogues 2 and 4, same layout as C (nullable)
  // act: 0 none, 1 ReLU, 2 keep where mask > 0 (ReLU derivative), 3 tanh, 4 multiply by
  // 1 - mask^2 (tanh derivative, mask = the stored tanh output)
  int M, N, K, lda, ldb, ldc, ta, tb, act;
  float beta;             // C32 = acc + beta * C32 (gradient accumulation); 0 overwrites
  long long sA, sB, sC, sBias;  // elements between groups (blockIdx.z); the mask moves with C
};

// The arguments of group blockIdx.z.
__device__ __forceinline__ GemmArgs at_group(const GemmArgs& g0) {
  GemmArgs g = g0;
  const long long z = blockIdx.z;
  if (z) {
    g.A += z * g.sA;
    g.B += z * g.sB;
    if (g.C32) g.C32 += z * g.sC;
    if (g.C16) g.C16 += z * g.sC;
    if (g.mask) g.mask += z * g.sC;
    if (g.bias) g.bias += z * g.sBias;
  }
  return g;
}

__device__ __forceinline__ uint32_t pack2(const __nv_bfloat16* p) {
  return *reinterpret_cast<const uint32_t*>(p);
}

__global__ void __launch_bounds__(128) gemm_bf16_kernel(const GemmArgs g0) {
  const GemmArgs g = at_group(g0);
  __shared__ __align__(16) __nv_bfloat16 As[kBM][kPadK];
  __shared__ __align__(16) __nv_bfloat16 Bs[kBN][kPadK];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * kBN;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int grp = lane >> 2, tig = lane & 3;
  float acc[2][4][4] = {};
  const __nv_bfloat16 zero = __float2bfloat16(0.f);
  for (int k0 = 0; k0 < g.K; k0 += kBK) {
    // stage A (rows m, k contiguous) and B (columns n, k contiguous)
    for (int e = tid; e < kBM * kBK; e += blockDim.x) {
      const int r = e / kBK, kk = e % kBK;
      const int m = m0 + r, k = k0 + kk;
      __nv_bfloat16 v = zero;
      if (m < g.M && k < g.K) v = g.ta ? g.A[(long long)k * g.lda + m] : g.A[(long long)m * g.lda + k];
      As[r][kk] = v;
    }
    for (int e = tid; e < kBN * kBK; e += blockDim.x) {
      const int c = e / kBK, kk = e % kBK;
      const int n = n0 + c, k = k0 + kk;
      __nv_bfloat16 v = zero;
      if (n < g.N && k < g.K) v = g.tb ? g.B[(long long)n * g.ldb + k] : g.B[(long long)k * g.ldb + n];
      Bs[c][kk] = v;
    }
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < kBK; ks += 16) {
      uint32_t a[2][4], b[4][2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int r = wm + 16 * i + grp;
        a[i][0] = pack2(&As[r][ks + 2 * tig]);
        a[i][1] = pack2(&As[r + 8][ks + 2 * tig]);
        a[i][2] = pack2(&As[r][ks + 8 + 2 * tig]);
        a[i][3] = pack2(&As[r + 8][ks + 8 + 2 * tig]);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int c = wn + 8 * j + grp;
        b[j][0] = pack2(&Bs[c][ks + 2 * tig]);
        b[j][1] = pack2(&Bs[c][ks + 8 + 2 * tig]);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
          asm volatile(
              "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
              "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};\n"
              : "+f"(acc[i][j][0]), "+f"(acc[i][j][1]), "+f"(acc[i][j][2]), "+f"(acc[i][j][3])
              : "r"(a[i][0]), "r"(a[i][1]), "r"(a[i][2]), "r"(a[i][3]), "r"(b[j][0]), "r"(b[j][1]));
    }
    __syncthreads();
  }
  // epilogue: C fragment (row grp / grp + 8, columns 2 tig, 2 tig + 1)
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int h = 0; h < 4; ++h) {
        const int m = m0 + wm + 16 * i + grp + (h >= 2 ? 8 : 0);
        const int n = n0 + wn + 8 * j + 2 * tig + (h & 1);
        if (m >= g.M || n >= g.N) continue;
        const long long o = (long long)m * g.ldc + n;
        float v = acc[i][j][h];
        if (g.bias) v += g.bias[n];
        if (g.act == 1) v = v > 0.f ? v : 0.f;
        if (g.act == 2 && !(__bfloat162float(g.mask[o]) > 0.f)) v = 0.f;
        if (g.act == 3) v = tanhf(v);
        if (g.act == 4) {
          const float a = __bfloat162float(g.mask[o]);
          v *= 1.f - a * a;
        }
        if (g.C32) g.C32[o] = g.beta != 0.f ? v + g.beta * g.C32[o] : v;
        if (g.C16) g.C16[o] = __float2bfloat16(v);
      }
}


// ---------------------------------------------------------------------------------------------
// pipelined path
constexpr int kPipeBN = 64, kPipeBK = 32, kStages = 3;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, bool valid) {
  const int bytes = valid ? 16 : 0;  // 0: the 16 bytes are zero-filled, nothing is read
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(bytes));
}

__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t (&r)[4]) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(addr));
}

__device__ __forceinline__ void ldsm_x4_t(uint32_t addr, uint32_t (&r)[4]) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0, %1, %2, %3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(addr));
}

// Shared tile of one operand: R rows of W elements (+8 padding: rows 16 bytes out of bank step).
template <int R, int W>
struct STile {
  __nv_bfloat16 v[R][W + 8];
};

template <int TA, int TB, int BM>
struct PipeSmem {
  // A: [BM][BK] when K-contiguous (TA = 0), [BK][BM] when M-contiguous (TA = 1); B likewise.
  using ATile = STile<TA ? kPipeBK : BM, TA ? BM : kPipeBK>;
  using BTile = STile<TB ? kPipeBN : kPipeBK, TB ? kPipeBK : kPipeBN>;
  ATile a[kStages];
  BTile b[kStages];
};

template <int TA, int TB, int BM>
__device__ __forceinline__ void pipe_load(const GemmArgs& g, PipeSmem<TA, TB, BM>& sm, int slot, int k0, int m0,
                                          int n0) {
  const int tid = threadIdx.x;
  constexpr int kAChunks = BM * kPipeBK / 8, kBChunks = kPipeBN * kPipeBK / 8;
#pragma unroll
  for (int c = tid; c < kAChunks; c += 128) {
    int r, x, m, k;
    if (TA) {
      r = c / (BM / 8), x = (c % (BM / 8)) * 8, k = k0 + r, m = m0 + x;
    } else {
      r = c / (kPipeBK / 8), x = (c % (kPipeBK / 8)) * 8, m = m0 + r, k = k0 + x;
    }
    const bool ok = m < g.M && k < g.K;
    const __nv_bfloat16* src = ok ? (TA ? g.A + (long long)k * g.lda + m : g.A + (long long)m * g.lda + k) : g.A;
    cp_async16(smem_addr(&sm.a[slot].v[r][x]), src, ok);
  }
#pragma unroll
  for (int c = tid; c < kBChunks; c += 128) {
    int r, x, n, k;
    if (TB) {
      r = c / (kPipeBK / 8), x = (c % (kPipeBK / 8)) * 8, n = n0 + r, k = k0 + x;
    } else {
      r = c / (kPipeBN / 8), x = (c % (kPipeBN / 8)) * 8, k = k0 + r, n = n0 + x;
    }
    const bool ok = n < g.N && k < g.K;
    const __nv_bfloat16* src = ok ? (TB ? g.B + (long long)n * g.ldb + k : g.B + (long long)k * g.ldb + n) : g.B;
    cp_async16(smem_addr(&sm.b[slot].v[r][x]), src, ok);
  }
}

template <int TA, int TB, int BM>
__global__ void __launch_bounds__(128) gemm_pipe_kernel(const GemmArgs g0) {
  const GemmArgs g = at_group(g0);
  __shared__ __align__(128) PipeSmem<TA, TB, BM> sm;
  constexpr int MI = BM / 32;  // m16 tiles per warp (warp tile BM/2 x 32)
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * kPipeBN;
  const int wm = (warp >> 1) * (BM / 2), wn = (warp & 1) * 32;
  float acc[MI][4][4] = {};
  const int nk = (g.K + kPipeBK - 1) / kPipeBK;
#pragma unroll
  for (int s = 0; s < kStages - 1; ++s) {
    if (s < nk) pipe_load<TA, TB, BM>(g, sm, s, s * kPipeBK, m0, n0);
    asm volatile("cp.async.commit_group;\n" ::);
  }
  for (int kt = 0; kt < nk; ++kt) {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(kStages - 2));
    __syncthreads();
    const int next = kt + kStages - 1;
    if (next < nk) pipe_load<TA, TB, BM>(g, sm, next % kStages, next * kPipeBK, m0, n0);
    asm volatile("cp.async.commit_group;\n" ::);
    const int slot = kt % kStages;
#pragma unroll
    for (int ks = 0; ks < kPipeBK; ks += 16) {
      uint32_t a[MI][4], b[4][2];
#pragma unroll
      for (int i = 0; i < MI; ++i) {
        if (TA) {
          const int k = ks + (lane & 7) + (lane >> 4) * 8, m = wm + 16 * i + ((lane >> 3) & 1) * 8;
          ldsm_x4_t(smem_addr(&sm.a[slot].v[k][m]), a[i]);
        } else {
          const int m = wm + 16 * i + (lane & 15), k = ks + (lane >> 4) * 8;
          ldsm_x4(smem_addr(&sm.a[slot].v[m][k]), a[i]);
        }
      }
#pragma unroll
      for (int jp = 0; jp < 2; ++jp) {
        uint32_t r[4];
        if (TB) {
          const int n = wn + 16 * jp + (lane & 7) + (lane >> 4) * 8, k = ks + ((lane >> 3) & 1) * 8;
          ldsm_x4(smem_addr(&sm.b[slot].v[n][k]), r);
        } else {
          const int k = ks + (lane & 7) + ((lane >> 3) & 1) * 8, n = wn + 16 * jp + (lane >> 4) * 8;
          ldsm_x4_t(smem_addr(&sm.b[slot].v[k][n]), r);
        }
        b[2 * jp][0] = r[0], b[2 * jp][1] = r[1], b[2 * jp + 1][0] = r[2], b[2 * jp + 1][1] = r[3];
      }
#pragma unroll
      for (int i = 0; i < MI; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
          asm volatile(
              "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
              "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};\n"
              : "+f"(acc[i][j][0]), "+f"(acc[i][j][1]), "+f"(acc[i][j][2]), "+f"(acc[i][j][3])
              : "r"(a[i][0]), "r"(a[i][1]), "r"(a[i][2]), "r"(a[i][3]), "r"(b[j][0]), "r"(b[j][1]));
    }
  }
  asm volatile("cp.async.wait_group 0;\n" ::);
  // epilogue: each thread holds column pairs (2 tig, 2 tig + 1) of rows grp and grp + 8
  const int grp = lane >> 2, tig = lane & 3;
#pragma unroll
  for (int i = 0; i < MI; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int m = m0 + wm + 16 * i + grp + 8 * h;
        const int n = n0 + wn + 8 * j + 2 * tig;
        if (m >= g.M || n >= g.N) continue;  // N is a multiple of 8: n + 1 < N as well
        const long long o = (long long)m * g.ldc + n;
        float v0 = acc[i][j][2 * h], v1 = acc[i][j][2 * h + 1];
        if (g.bias) v0 += g.bias[n], v1 += g.bias[n + 1];
        if (g.act == 1) v0 = fmaxf(v0, 0.f), v1 = fmaxf(v1, 0.f);
        if (g.act == 2) {
          const __nv_bfloat162 mk = *reinterpret_cast<const __nv_bfloat162*>(g.mask + o);
          if (!(__low2float(mk) > 0.f)) v0 = 0.f;
          if (!(__high2float(mk) > 0.f)) v1 = 0.f;
        }
        if (g.act == 3) v0 = tanhf(v0), v1 = tanhf(v1);
        if (g.act == 4) {
          const __nv_bfloat162 mk = *reinterpret_cast<const __nv_bfloat162*>(g.mask + o);
          const float a0 = __low2float(mk), a1 = __high2float(mk);
          v0 *= 1.f - a0 * a0, v1 *= 1.f - a1 * a1;
        }
        if (g.C32) {
          float2* c = reinterpret_cast<float2*>(g.C32 + o);
          if (g.beta != 0.f) {
            const float2 old = *c;
            v0 += g.beta * old.x, v1 += g.beta * old.y;
          }
          *c = make_float2(v0, v1);
        }
        if (g.C16) *reinterpret_cast<__nv_bfloat162*>(g.C16 + o) = __floats2bfloat162_rn(v0, v1);
      }
}

template <int BM>
void launch_pipe(const GemmArgs& g, int groups, cudaStream_t s) {
  const dim3 grid((g.N + kPipeBN - 1) / kPipeBN, (g.M + BM - 1) / BM, groups);
  if (g.ta && g.tb) gemm_pipe_kernel<1, 1, BM><<<grid, 128, 0, s>>>(g);
  else if (g.ta) gemm_pipe_kernel<1, 0, BM><<<grid, 128, 0, s>>>(g);
  else if (g.tb) gemm_pipe_kernel<0, 1, BM><<<grid, 128, 0, s>>>(g);
  else gemm_pipe_kernel<0, 0, BM><<<grid, 128, 0, s>>>(g);
}

bool pipe_ok(const GemmArgs& g) {
  auto al = [](const void* p, uintptr_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; };
  return g.M % 8 == 0 && g.N % 8 == 0 && g.K % 8 == 0 && g.lda % 8 == 0 && g.ldb % 8 == 0 && g.ldc % 2 == 0 &&
         g.sA % 8 == 0 && g.sB % 8 == 0 && g.sC % 2 == 0 && al(g.A, 16) && al(g.B, 16) && al(g.C32, 8) && al(g.C16, 4) && al(g.mask, 4);
}

// Column sums of an FP32 M x N matrix (bias gradients), per group (blockIdx.y: X and out move by
// xs and os elements). A block takes 32 columns; each of its 16 row lanes sums the rows lane,
// lane + 16, ... of one column (a warp reads 32 adjacent columns of one row), then lane 0 adds the
// 16 partial sums in lane order: a fixed order, so the result is the same on every run.
constexpr int kSumCols = 32, kSumLanes = 16;

__global__ void __launch_bounds__(kSumCols * kSumLanes) colsum_kernel(const float* X, int M, int N, int ld,
                                                                      long long xs, float* out, long long os) {
  __shared__ float part[kSumLanes][kSumCols + 1];
  X += blockIdx.y * xs;
  out += blockIdx.y * os;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int n = blockIdx.x * kSumCols + tx;
  float s = 0.f;
  if (n < N)
#pragma unroll 4
    for (int m = ty; m < M; m += kSumLanes) s += X[(long long)m * ld + n];
  part[ty][tx] = s;
  __syncthreads();
  if (ty == 0 && n < N) {
    float t = 0.f;
    for (int q = 0; q < kSumLanes; ++q) t += part[q][tx];
    out[n] = t;
  }
}

// Mean-squared-error gradient of each group's mean over its M_g rows: G = (2 / (M_g N)) (Y - T),
// in FP32 and BF16; loss partials per row.
__global__ void mse_grad_kernel(const float* Y, const float* T, int Mg, int N, float* G32, __nv_bfloat16* G16,
                                float* row_loss) {
  const int m = blockIdx.x;
  float s = 0.f;
  const float scale = 2.f / ((float)Mg * (float)N);
  for (int n = threadIdx.x; n < N; n += blockDim.x) {
    const long long o = (long long)m * N + n;
    const float d = Y[o] - T[o];
    s += d * d;
    const float gr = scale * d;
    G32[o] = gr;
    G16[o] = __float2bfloat16(gr);
  }
  __shared__ float part[256];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int q = 0; q < (int)blockDim.x; ++q) t += part[q];
    row_loss[m] = t;
  }
}

// Adam on FP32 master weights, with the BF16 copy the GEMMs read. The learning rate and the step
// number (for the bias corrections) are read from device memory, so that a captured training step
// replays unchanged while both move on.
__global__ void adam_kernel(float* w, __nv_bfloat16* w16, const float* grad, float* m1, float* m2, long long n,
                            const float* lr_dev, float b1, float b2, float eps, const int* step) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float t = (float)*step, lr = *lr_dev;
  const float c1 = 1.f - powf(b1, t), c2 = 1.f - powf(b2, t);
  const float g = grad[i];
  const float a = b1 * m1[i] + (1.f - b1) * g;
  const float b = b2 * m2[i] + (1.f - b2) * g * g;
  m1[i] = a;
  m2[i] = b;
  const float v = w[i] - lr * (a / c1) / (sqrtf(b / c2) + eps);
  w[i] = v;
  if (w16) w16[i] = __float2bfloat16(v);
}

__global__ void count_kernel(int* counter) { *counter += 1; }

// Rows idx[0..rows) of an FP32 matrix with `cols` columns, into FP32 and/or BF16 copies.
__global__ void gather_kernel(const float* src, int cols, const int* idx, int rows, float* d32,
                              __nv_bfloat16* d16) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)rows * cols) return;
  const int r = (int)(e / cols), c = (int)(e % cols);
  const float v = src[(long long)idx[r] * cols + c];
  if (d32) d32[e] = v;
  if (d16) d16[e] = __float2bfloat16(v);
}

// dst (cols x rows, leading dimension ldd) = src^T (rows x cols, leading dimension lds), BF16,
// through 32 x 32 shared tiles (both sides coalesced); group blockIdx.z at ss / sd elements.
__global__ void transpose16_kernel(const __nv_bfloat16* src, int rows, int cols, int lds, long long ss,
                                   __nv_bfloat16* dst, int ldd, long long sd) {
  __shared__ __nv_bfloat16 t[32][33];
  src += blockIdx.z * ss;
  dst += blockIdx.z * sd;
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int r = r0 + y, c = c0 + threadIdx.x;
    if (r < rows && c < cols) t[y][threadIdx.x] = src[(long long)r * lds + c];
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int c = c0 + y, r = r0 + threadIdx.x;
    if (r < rows && c < cols) dst[(long long)c * ldd + r] = t[threadIdx.x][y];
  }
}

// One GEMM launch of `groups` problems (blockIdx.z): the pipelined kernel where the shape and
// alignment allow, the scalar-staging kernel elsewhere. Returns 0 or -3 (launch error).
int gemm_grouped(const GemmArgs& g, int groups, cudaStream_t s, const char* who) {
  if (pipe_ok(g)) {
    // 64-row tiles unless that leaves fewer than two blocks per SM on a 152-SM part
    const long long tiles64 = (long long)((g.N + 63) / 64) * ((g.M + 63) / 64) * groups;
    if (tiles64 < 304) launch_pipe<32>(g, groups, s);
    else launch_pipe<64>(g, groups, s);
  } else {
    const dim3 grid((g.N + kBN - 1) / kBN, (g.M + kBM - 1) / kBM, groups);
    gemm_bf16_kernel<<<grid, 128, 0, s>>>(g);
  }
  const cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) {
    set_last_error(std::string(who) + ": " + cudaGetErrorString(err));
    return -3;
  }
  return 0;
}

}  // namespace oafdtd

// --------------------------------------------------------------------------------------- C ABI
extern "C" {

int oafdtd_mlp_transpose(const void* src, int32_t rows, int32_t cols, int32_t lds, void* dst, int32_t ldd,
                         int32_t groups, int64_t src_stride, int64_t dst_stride, void* stream) {
  if (!src || !dst || rows < 1 || cols < 1 || lds < cols || ldd < rows || groups < 1 || groups > 65535 ||
      (groups > 1 && (src_stride < (int64_t)rows * lds || dst_stride < (int64_t)cols * ldd))) {
    oafdtd::set_last_error("oafdtd_mlp_transpose: bad arguments");
    return -1;
  }
  const dim3 grid((cols + 31) / 32, (rows + 31) / 32, groups), block(32, 8);
  oafdtd::transpose16_kernel<<<grid, block, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const __nv_bfloat16*>(src), rows, cols, lds, src_stride, static_cast<__nv_bfloat16*>(dst), ldd,
      dst_stride);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

int oafdtd_mlp_gemm_tn(const void* A, const void* B, float* C32, void* C16, void* C16T, const float* bias,
                       const void* mask, int32_t M, int32_t N, int32_t K, int32_t lda, int32_t ldb, int32_t ldc,
                       int32_t ldct, int32_t act, float beta, int32_t groups, int64_t strideA, int64_t strideB,
                       int64_t strideC, int64_t strideCT, int64_t strideBias, int32_t* status, void* stream) {
  const bool bad_strides = groups > 1 && (strideA < (int64_t)M * lda || strideB < (int64_t)N * ldb ||
                                          ((C32 || C16 || mask) && strideC < (int64_t)M * ldc) ||
                                          (C16T && strideCT < (int64_t)N * ldct) || (bias && strideBias < N));
  if (!A || !B || (!C32 && !C16 && !C16T) || M < 1 || N < 1 || K < 1 || act < 0 || act > 4 ||
      ((act == 2 || act == 4) && !mask) || (C16T && ldct < M) || lda < K || ldb < K ||
      ((C32 || C16 || mask) && ldc < N) || groups < 1 || groups > 65535 || bad_strides) {
    oafdtd::set_last_error("oafdtd_mlp_gemm_tn: bad arguments");
    return -1;
  }
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  oafdtd::UmmaProblem p{A, B, C32, C16, C16T, bias, mask, M, N, K, lda, ldb, ldc, ldct, act, groups,
                        strideA, strideB, strideC, strideCT, strideBias, beta, status};
  if (oafdtd::umma_shape_ok(p)) {
    std::string why;
    const cudaError_t err = oafdtd::launch_umma_gemm(p, s, &why);
    if (err != cudaSuccess) {
      oafdtd::set_last_error(std::string("oafdtd_mlp_gemm_tn: ") + (why.empty() ? cudaGetErrorString(err) : why));
      return err == cudaErrorInvalidValue ? -1 : -3;
    }
    return 0;
  }
  // other shapes: the mma.sync kernels (B transposed), then the transposed copy of the BF16 result
  if (C16T && !C16) {
    oafdtd::set_last_error("oafdtd_mlp_gemm_tn: a transposed result off the tcgen05 shapes needs C16 as well");
    return -1;
  }
  oafdtd::GemmArgs g;
  g.A = static_cast<const __nv_bfloat16*>(A);
  g.B = static_cast<const __nv_bfloat16*>(B);
  g.C32 = C32;
  g.C16 = static_cast<__nv_bfloat16*>(C16);
  g.bias = bias;
  g.mask = static_cast<const __nv_bfloat16*>(mask);
  g.M = M, g.N = N, g.K = K, g.lda = lda, g.ldb = ldb, g.ldc = ldc, g.ta = 0, g.tb = 1, g.act = act;
  g.beta = beta;
  g.sA = strideA, g.sB = strideB, g.sC = strideC, g.sBias = strideBias;
  int rc = oafdtd::gemm_grouped(g, groups, s, "oafdtd_mlp_gemm_tn");
  if (rc == 0 && C16T) rc = oafdtd_mlp_transpose(C16, M, N, ldc, C16T, ldct, groups, strideC, strideCT, stream);
  return rc;
}

int oafdtd_mlp_gemm(const void* A, const void* B, float* C32, void* C16, const float* bias, const void* mask,
                    int32_t M, int32_t N, int32_t K, int32_t lda, int32_t ldb, int32_t ldc, int32_t ta, int32_t tb,
                    int32_t act, float beta, void* stream) {
  if (!A || !B || (!C32 && !C16) || M < 1 || N < 1 || K < 1 || act < 0 || act > 4 || ((act == 2 || act == 4) && !mask)) {
    oafdtd::set_last_error("oafdtd_mlp_gemm: bad arguments");
    return -1;
  }
  oafdtd::GemmArgs g;
  g.A = static_cast<const __nv_bfloat16*>(A);
  g.B = static_cast<const __nv_bfloat16*>(B);
  g.C32 = C32;
  g.C16 = static_cast<__nv_bfloat16*>(C16);
  g.bias = bias;
  g.mask = static_cast<const __nv_bfloat16*>(mask);
  g.M = M, g.N = N, g.K = K, g.lda = lda, g.ldb = ldb, g.ldc = ldc, g.ta = ta, g.tb = tb, g.act = act;
  g.beta = beta;
  g.sA = g.sB = g.sC = g.sBias = 0;
  return oafdtd::gemm_grouped(g, 1, static_cast<cudaStream_t>(stream), "oafdtd_mlp_gemm");
}

int oafdtd_mlp_colsum(const float* X, int32_t M, int32_t N, int32_t ld, float* out, int32_t groups,
                      int64_t x_stride, int64_t out_stride, void* stream) {
  if (!X || !out || M < 1 || N < 1 || ld < N || groups < 1 || groups > 65535 ||
      (groups > 1 && (x_stride < (int64_t)M * ld || out_stride < N)))
    return -1;
  const dim3 block(oafdtd::kSumCols, oafdtd::kSumLanes), grid((N + oafdtd::kSumCols - 1) / oafdtd::kSumCols, groups);
  oafdtd::colsum_kernel<<<grid, block, 0, static_cast<cudaStream_t>(stream)>>>(X, M, N, ld, x_stride, out,
                                                                                out_stride);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

int oafdtd_mlp_mse_grad(const float* Y, const float* T, int32_t M, int32_t N, float* G32, void* G16,
                        float* row_loss, int32_t groups, void* stream) {
  if (!Y || !T || !G32 || !G16 || !row_loss || M < 1 || N < 1 || groups < 1 || M % groups != 0) return -1;
  oafdtd::mse_grad_kernel<<<M, 256, 0, static_cast<cudaStream_t>(stream)>>>(Y, T, M / groups, N, G32,
                                                                              static_cast<__nv_bfloat16*>(G16), row_loss);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

int oafdtd_mlp_adam(float* w, void* w16, const float* grad, float* m1, float* m2, int64_t n, const float* lr,
                    float b1, float b2, float eps, const int32_t* step, void* stream) {
  if (!w || !grad || !m1 || !m2 || !lr || !step || n < 1) return -1;
  oafdtd::adam_kernel<<<(unsigned)((n + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      w, static_cast<__nv_bfloat16*>(w16), grad, m1, m2, n, lr, b1, b2, eps, step);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

int oafdtd_mlp_count(int32_t* counter, void* stream) {
  if (!counter) return -1;
  oafdtd::count_kernel<<<1, 1, 0, static_cast<cudaStream_t>(stream)>>>(counter);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

int oafdtd_mlp_gather(const float* src, int32_t cols, const int32_t* idx, int32_t rows, float* dst32, void* dst16,
                      void* stream) {
  if (!src || !idx || cols < 1 || rows < 1 || (!dst32 && !dst16)) return -1;
  const long long n = (long long)rows * cols;
  oafdtd::gather_kernel<<<(unsigned)((n + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      src, cols, idx, rows, dst32, static_cast<__nv_bfloat16*>(dst16));
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

}  // extern "C"
