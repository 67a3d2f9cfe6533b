// Sweeps with the planes staged through shared memory (variants 1 and 2; the default is 2).
//
// A block owns a 2-D tile of 32 quads (128 x cells) by 8 rows and marches up a chunk of z
// planes. Each plane's inputs (the tile plus the one-cell halo the curl needs) are copied into a
// ring of three shared-memory slots, two planes ahead of the plane being computed, so every SM
// keeps ~130 KB of loads in flight without holding them in registers; the Debye currents of the
// next plane are prefetched into registers. Neighbours in x and y are read from the staged tile;
// results go straight to global memory.
//
// Variant 2 moves each array of a plane with one TMA tensor copy (cp.async.bulk.tensor) issued
// by one thread and completing on the slot's mbarrier; parts of a box past the grid are
// zero-filled. Variant 1 spreads 16-byte cp.async copies over the block and leaves those parts
// unwritten. Either way the cells they feed are never updated.
//
// Every mbarrier wait is bounded (about two seconds): a block whose copies do not arrive sets
// bit 0 of the status word, waits (bounded again) for the copies it issued and returns; the host
// reports OAFDTD_E_TIMEOUT.
//
// These kernels cover the interior box of each sweep, which holds no CPML correction cell: every
// cell gets its bulk update (and, in the E sweep, its Debye update). The slab kernel (slab.cu)
// covers the rest. The arithmetic is the reference's, operation by operation
// (packages/oa-fdtd/src/oa_fdtd/reference.py:152-180, :119-127).

#include <mutex>
#include <type_traits>

#include "tma.cuh"

namespace oafdtd {

constexpr int kTQ = 32;       // quads per tile row (128 cells)
constexpr int kTY = 8;        // rows per tile
constexpr int kTW = 4 * kTQ;  // tile width in cells
constexpr int kHW = kTW + 4;  // staged width with a one-quad halo

// ------------------------------------------------------------------------------------- blocks
// Stages per kernel: three planes in flight, two for the E sweep with z corrections (its slot is
// larger; two blocks per SM must fit).
template <bool kE, bool kZ>
__host__ __device__ constexpr int stages() {
  return kE && kZ ? 2 : 3;
}

// The z-term psi tiles of the two components that have one (E: Ex, Ey; H: Hx, Hy).
template <typename real>
struct ZPart {
  Box<real, kTY, kTW> p[2];
};
struct NoPart {};

// The box a block works on and its plane range. Plain sweeps cover the interior box in chunks of
// tile_z planes; z sweeps cover one whole z-slab box (low or high) per block.
struct BlockSpan {
  int x0, y0, b, zr, k0, k1;
  Span3 box;
  bool empty;
};

template <typename real, bool kZ>
__device__ __forceinline__ BlockSpan block_span(const SweepArgs<real>& a, int kind, const uint3 bid) {
  BlockSpan s;
  if (kZ) {
    s.zr = (int)bid.z & 1;
    s.b = (int)bid.z >> 1;
    s.box = a.zin[kind][s.zr];
    s.k0 = s.box.k0;
    s.k1 = s.box.k1;
  } else {
    s.zr = 0;
    s.box = a.inner[kind];
    const int nkc = (s.box.k1 - s.box.k0 + a.tile_z - 1) / a.tile_z;
    s.b = (int)bid.z / nkc;
    const int kc = (int)bid.z % nkc;
    s.k0 = s.box.k0 + kc * a.tile_z;
    s.k1 = min(s.k0 + a.tile_z, s.box.k1);
  }
  s.x0 = 4 * (s.box.q0 + (int)bid.x * kTQ);
  s.y0 = s.box.j0 + (int)bid.y * kTY;
  s.empty = s.k1 <= s.k0 || s.x0 >= 4 * s.box.q1 || s.y0 >= s.box.j1;
  return s;
}

// psi tile copies of one plane of a z sweep (cp.async variant): [component][row][quad]
template <typename real>
__device__ __forceinline__ void z_stage(const SweepArgs<real>& a, ZPart<real>& zp, int kind, int zr, int b, int k,
                                        int x0, int y0) {
  constexpr int CQ = (int)(4 * sizeof(real) / 16);
  constexpr int EL = 16 / sizeof(real);
  constexpr int count = 2 * kTY * (kTW / 4) * CQ;
  for (int t = threadIdx.x + threadIdx.y * blockDim.x; t < count; t += blockDim.x * blockDim.y) {
    const int part = t % CQ, q = (t / CQ) % (kTW / 4), r = (t / CQ / (kTW / 4)) % kTY;
    const int cc = t / CQ / (kTW / 4) / kTY;
    const int sd = a.zsd[kind][zr][cc];
    if (sd < 0) continue;
    const CpmlTerm<real>& T = kind == 0 ? a.ecorr[cc][1] : a.hcorr[cc][1];
    const CpmlSide<real>& s = sd == 0 ? T.side[0] : T.side[1];
    const int x = x0 + 4 * q, y = y0 + r;
    if (x >= a.X || y >= a.Y || k < s.lo[2] || k >= s.hi[2]) continue;
    const int w = s.hi[2] - s.lo[2];
    cp_async16(&zp.p[cc].v[r][4 * q] + part * EL,
               s.psi + (((long long)b * w + (k - s.lo[2])) * a.Y + y) * a.X + x + part * EL);
  }
}

// psi tile copies of one plane of a z sweep (TMA variant); returns the bytes they bring.
template <typename real>
__device__ __forceinline__ unsigned z_bytes(const SweepArgs<real>& a, int kind, int zr) {
  unsigned n = 0;
#pragma unroll
  for (int cc = 0; cc < 2; ++cc)
    if (a.zsd[kind][zr][cc] >= 0) n += kTY * kTW * sizeof(real);
  return n;
}
template <typename real>
__device__ __forceinline__ void z_issue(const SweepArgs<real>& a, const SweepMaps& tm, ZPart<real>& zp,
                                        unsigned long long* bar, int kind, int zr, int b, int k, int x0, int y0) {
#pragma unroll
  for (int cc = 0; cc < 2; ++cc) {
    const int sd = a.zsd[kind][zr][cc];
    if (sd < 0) continue;
    const CpmlTerm<real>& T = kind == 0 ? a.ecorr[cc][1] : a.hcorr[cc][1];
    const CpmlSide<real>& s = sd == 0 ? T.side[0] : T.side[1];
    // a plane outside the slab (H's high box reaches one plane past it) reads zero fill
    tma_load4(&zp.p[cc], &tm.psi_z[kind][cc][zr], bar, x0, y0, k - s.lo[2], b);
  }
}

// ------------------------------------------------------------------------------------- H sweep
// Slot: E[3] rows y0..y0+8, x0..x0+131; H[3] rows y0..y0+7, x0..x0+127; z sweeps also the psi
// of Hx and Hy.
template <typename real, bool kZ>
struct HSlot {
  Box<real, kTY + 1, kHW> e[3];
  Box<real, kTY, kTW> h[3];
  typename std::conditional<kZ, ZPart<real>, NoPart>::type z;
};

// Planes k0..k1 are staged: E for all of them (plane k1 only feeds the z derivative of plane
// k1 - 1), H for k < k1.
template <typename real, bool kZ>
__device__ __forceinline__ void h_stage(const SweepArgs<real>& a, HSlot<real, kZ>& s, int b, int zr, int k, int k1,
                                        int x0, int y0) {
  const int X = a.X, Y = a.Y, Z = a.nz + 2;
  if (k >= Z || k > k1) return;
  const long long base = (long long)b * a.bs + (long long)k * X * Y;
  constexpr int CQ = (int)(4 * sizeof(real) / 16);
  constexpr int EL = 16 / sizeof(real);
  constexpr int ecount = 3 * (kTY + 1) * (kHW / 4) * CQ;
  constexpr int hcount = 3 * kTY * (kTW / 4) * CQ;
  const int total = k < k1 ? ecount + hcount : ecount;
  for (int t = threadIdx.x + threadIdx.y * blockDim.x; t < total; t += blockDim.x * blockDim.y) {
    if (t < ecount) {
      const int part = t % CQ, q = (t / CQ) % (kHW / 4), r = (t / CQ / (kHW / 4)) % (kTY + 1);
      const int c = t / CQ / (kHW / 4) / (kTY + 1);
      const int x = x0 + 4 * q, y = y0 + r;
      if (x >= X || y >= Y) continue;
      cp_async16(&s.e[c].v[r][4 * q] + part * EL, a.E[c] + base + (long long)y * X + x + part * EL);
    } else {
      const int u = t - ecount;
      const int part = u % CQ, q = (u / CQ) % (kTW / 4), r = (u / CQ / (kTW / 4)) % kTY;
      const int c = u / CQ / (kTW / 4) / kTY;
      const int x = x0 + 4 * q, y = y0 + r;
      if (x >= X || y >= Y) continue;
      cp_async16(&s.h[c].v[r][4 * q] + part * EL, a.H[c] + base + (long long)y * X + x + part * EL);
    }
  }
  if constexpr (kZ) {
    if (k < k1) z_stage(a, s.z, 1, zr, b, k, x0, y0);
  }
}

template <typename real, bool kZ>
__device__ __forceinline__ void h_issue(const SweepArgs<real>& a, const SweepMaps& tm, HSlot<real, kZ>& s,
                                        unsigned long long* bar, int b, int zr, int k, int k1, int x0, int y0) {
  constexpr unsigned eb = 3u * (kTY + 1) * kHW * sizeof(real);
  constexpr unsigned hb = 3u * kTY * kTW * sizeof(real);
  const bool with_h = k < k1;
  unsigned bytes = with_h ? eb + hb : eb;
  if constexpr (kZ) {
    if (with_h) bytes += z_bytes(a, 1, zr);
  }
  mbar_expect_tx(bar, bytes);
#pragma unroll
  for (int c = 0; c < 3; ++c) tma_load4(&s.e[c], &tm.e_wide[c], bar, x0, y0, k, b);
  if (with_h) {
#pragma unroll
    for (int c = 0; c < 3; ++c) tma_load4(&s.h[c], &tm.h_tile[c], bar, x0, y0, k, b);
    if constexpr (kZ) z_issue(a, tm, s.z, bar, 1, zr, b, k, x0, y0);
  }
}

template <typename real, bool kTma, bool kZ>
__device__ __forceinline__ void h_staged_body(const SweepArgs<real>& a, const SweepMaps& tm, const uint3 bid) {
  constexpr int S = stages<false, kZ>();
  extern __shared__ unsigned char smem_raw[];
  __shared__ unsigned long long bar[S];
  HSlot<real, kZ>* slot = reinterpret_cast<HSlot<real, kZ>*>(align_smem(smem_raw));
  const int tx = threadIdx.x, ty = threadIdx.y;
  const bool leader = tx == 0 && ty == 0;
  const int nx = a.nx, ny = a.ny, nz = a.nz, X = a.X, Y = a.Y, Z = nz + 2;
  const BlockSpan sp = block_span<real, kZ>(a, 1, bid);
  if (sp.empty) return;
  const int x0 = sp.x0, y0 = sp.y0, b = sp.b, zr = sp.zr, k0 = sp.k0, k1 = sp.k1;
  const int n_stage = k1 < Z ? k1 - k0 + 1 : k1 - k0;
  const int i0 = x0 + 4 * tx, j = y0 + ty;
  const bool live = i0 < 4 * sp.box.q1 && j < sp.box.j1 && i0 <= nx + 1;
  const long long base = (long long)b * a.bs;
  const real dtmu = a.dtmu;
  const Quad<real> ipx = i0 < X ? ld4(a.ip[0] + i0) : Quad<real>{};
  const real ipy = a.ip[1][min(j, Y - 1)];
  if (kTma) {
    if (leader) {
      mbar_setup<S>(bar);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        prefetch_map(&tm.e_wide[c]);
        prefetch_map(&tm.h_tile[c]);
      }
    }
    __syncthreads();
    if (leader)
      for (int s = 0; s < S && s < n_stage; ++s) h_issue(a, tm, slot[s], &bar[s], b, zr, k0 + s, k1, x0, y0);
  } else {
#pragma unroll
    for (int s = 0; s < S; ++s) {
      h_stage(a, slot[s], b, zr, k0 + s, k1, x0, y0);
      cp_commit();
    }
  }
  for (int k = k0; k < k1; ++k) {
    const int t = k - k0;
    if (kTma) {
      bool ok = wait_plane<S>(bar, t);
      if (ok && t + 1 < n_stage) ok = wait_plane<S>(bar, t + 1);
      if (__syncthreads_or(!ok)) {
        abort_march<S>(bar, t, min(n_stage, t + S), a.status, leader);
        return;
      }
    } else {
      cp_wait<S - 2>();
      __syncthreads();
    }
    const HSlot<real, kZ>& cur = slot[t % S];
    const HSlot<real, kZ>& nxt = slot[(t + 1) % S];
    if (live) {
      const long long p = base + (long long)k * X * Y + (long long)j * X + i0;
      const bool kin = k <= nz;
      const real ipz = a.ip[2][k];
      const Quad<real> ex = ld4(&cur.e[0].v[ty][4 * tx]), ey = ld4(&cur.e[1].v[ty][4 * tx]);
      const Quad<real> ez = ld4(&cur.e[2].v[ty][4 * tx]);
      const real ez_r = cur.e[2].v[ty][4 * tx + 4], ey_r = cur.e[1].v[ty][4 * tx + 4];
      const real kf[4] = {dtmu, dtmu, dtmu, dtmu};
      if (j <= ny && kin) {  // Hx: node along x (1..nx+1), cell along y and z
        const Quad<real> ezy = ld4(&cur.e[2].v[ty + 1][4 * tx]);
        const Quad<real> ey1 = ld4(&nxt.e[1].v[ty][4 * tx]);
        Quad<real> h = ld4(&cur.h[0].v[ty][4 * tx]);
        real d0[4], d1[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int i = i0 + e;
          d0[e] = (ezy.v[e] - ez.v[e]) * ipy;  // axis y
          d1[e] = (ey1.v[e] - ey.v[e]) * ipz;  // axis z
          if (i >= 1 && i <= nx + 1) h.v[e] = h.v[e] + dtmu * ((-d0[e]) + d1[e]);
        }
        if constexpr (kZ)
          z_apply(z_term(a, a.hcorr[0][1], a.zsd[1][zr][0], &cur.z.p[0].v[ty][4 * tx], b, k, j, i0, 1), h, d1, kf,
                  i0);
        st4(a.Ho[0] + p, h);
      }
      if (kin) {  // Hy: cell along x (1..nx), node along y (1..ny+1), cell along z
        const Quad<real> ex1 = ld4(&nxt.e[0].v[ty][4 * tx]);
        Quad<real> h = ld4(&cur.h[1].v[ty][4 * tx]);
        real d0[4], d1[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int i = i0 + e;
          const real ezr = e < 3 ? ez.v[e + 1] : ez_r;
          d0[e] = (ezr - ez.v[e]) * ipx.v[e];  // axis x
          d1[e] = (ex1.v[e] - ex.v[e]) * ipz;  // axis z
          if (i >= 1 && i <= nx) h.v[e] = h.v[e] + dtmu * ((-d1[e]) + d0[e]);
        }
        if constexpr (kZ)
          z_apply(z_term(a, a.hcorr[1][1], a.zsd[1][zr][1], &cur.z.p[1].v[ty][4 * tx], b, k, j, i0, 1), h, d1, kf,
                  i0);
        st4(a.Ho[1] + p, h);
      }
      if (j <= ny) {  // Hz: cell along x and y, node along z (1..nz+1)
        const Quad<real> exy = ld4(&cur.e[0].v[ty + 1][4 * tx]);
        Quad<real> h = ld4(&cur.h[2].v[ty][4 * tx]);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int i = i0 + e;
          const real eyr = e < 3 ? ey.v[e + 1] : ey_r;
          const real d0 = (eyr - ey.v[e]) * ipx.v[e];  // axis x
          const real d1 = (exy.v[e] - ex.v[e]) * ipy;  // axis y
          if (i >= 1 && i <= nx) h.v[e] = h.v[e] + dtmu * ((-d0) + d1);
        }
        st4(a.Ho[2] + p, h);
      }
    }
    __syncthreads();  // every thread is done with the slot of plane k
    if (kTma) {
      if (leader && t + S < n_stage) {
        fence_proxy_async();
        h_issue(a, tm, slot[t % S], &bar[t % S], b, zr, k + S, k1, x0, y0);
      }
    } else {
      h_stage(a, slot[t % S], b, zr, k + S, k1, x0, y0);
      cp_commit();
    }
  }
  if (!kTma) cp_wait<0>();
}

template <typename real, bool kTma, bool kZ>
__global__ void __launch_bounds__(256, 2)
    h_staged_kernel(const __grid_constant__ SweepArgs<real> a, const __grid_constant__ SweepMaps tm) {
  h_staged_body<real, kTma, kZ>(a, tm, blockIdx);
}

// Several engines' H sweeps in one launch: engine e's arguments at A[e] and M[e].
template <typename real, bool kTma, bool kZ>
__global__ void __launch_bounds__(256, 2)
    h_staged_batch_kernel(const SweepArgs<real>* __restrict__ A, const SweepMaps* __restrict__ M, const BatchGrid G) {
  __shared__ __align__(16) unsigned char args[sizeof(SweepArgs<real>)];
  int e;
  const uint3 bid = G.block(&e);
  h_staged_body<real, kTma, kZ>(stage_args(A + e, args), M[e], bid);
}

// ------------------------------------------------------------------------------------- E sweep
// Slot: H[3] rows y0-1..y0+7, x0-4..x0+127; E[3] and mat[3] rows y0..y0+7, x0..x0+127; z sweeps
// also the psi of Ex and Ey.
template <typename real, bool kZ>
struct ESlot {
  Box<real, kTY + 1, kHW> h[3];
  Box<real, kTY, kTW> e[3];
  Box<uint16_t, kTY, kTW> m[3];
  typename std::conditional<kZ, ZPart<real>, NoPart>::type z;
};

template <typename real, bool kZ>
__device__ __forceinline__ void e_stage(const SweepArgs<real>& a, ESlot<real, kZ>& s, int b, int zr, int k, int kend,
                                        int x0, int y0) {
  const int X = a.X, Y = a.Y;
  if (k >= kend) return;
  const long long plane = (long long)k * X * Y;
  const long long base = (long long)b * a.bs + plane;
  constexpr int CQ = (int)(4 * sizeof(real) / 16);
  constexpr int EL = 16 / sizeof(real);
  constexpr int hcount = 3 * (kTY + 1) * (kHW / 4) * CQ;
  constexpr int ecount = 3 * kTY * (kTW / 4) * CQ;
  constexpr int mcount = 3 * kTY * (kTW / 8);  // 16-byte copies of eight indices
  for (int t = threadIdx.x + threadIdx.y * blockDim.x; t < hcount + ecount + mcount;
       t += blockDim.x * blockDim.y) {
    if (t < hcount) {
      const int part = t % CQ, q = (t / CQ) % (kHW / 4), r = (t / CQ / (kHW / 4)) % (kTY + 1);
      const int c = t / CQ / (kHW / 4) / (kTY + 1);
      const int x = x0 - 4 + 4 * q, y = y0 - 1 + r;
      if (x < 0 || x >= X || y >= Y) continue;
      cp_async16(&s.h[c].v[r][4 * q] + part * EL, a.Ho[c] + base + (long long)y * X + x + part * EL);
    } else if (t < hcount + ecount) {
      const int u = t - hcount;
      const int part = u % CQ, q = (u / CQ) % (kTW / 4), r = (u / CQ / (kTW / 4)) % kTY;
      const int c = u / CQ / (kTW / 4) / kTY;
      const int x = x0 + 4 * q, y = y0 + r;
      if (x >= X || y >= Y) continue;
      cp_async16(&s.e[c].v[r][4 * q] + part * EL, a.E[c] + base + (long long)y * X + x + part * EL);
    } else {
      const int u = t - hcount - ecount;
      const int q = u % (kTW / 8), r = (u / (kTW / 8)) % kTY, c = u / (kTW / 8) / kTY;
      const int x = x0 + 8 * q, y = y0 + r;
      if (x >= X || y >= Y) continue;
      cp_async16(&s.m[c].v[r][8 * q], a.mat[c] + plane + (long long)y * X + x);
    }
  }
  if constexpr (kZ) z_stage(a, s.z, 0, zr, b, k, x0, y0);
}

template <typename real, bool kZ>
__device__ __forceinline__ void e_issue(const SweepArgs<real>& a, const SweepMaps& tm, ESlot<real, kZ>& s,
                                        unsigned long long* bar, int b, int zr, int k, int x0, int y0) {
  unsigned bytes = 3u * ((kTY + 1) * kHW * sizeof(real) + kTY * kTW * sizeof(real) + kTY * kTW * sizeof(uint16_t));
  if constexpr (kZ) bytes += z_bytes(a, 0, zr);
  mbar_expect_tx(bar, bytes);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    tma_load4(&s.h[c], &tm.h_wide[c], bar, x0 - 4, y0 - 1, k, b);
    tma_load4(&s.e[c], &tm.e_tile[c], bar, x0, y0, k, b);
    tma_load3(&s.m[c], &tm.mat[c], bar, x0, y0, k);
  }
  if constexpr (kZ) z_issue(a, tm, s.z, bar, 0, zr, b, k, x0, y0);
}

// Debye currents of plane k for the three components (single-pole runs only; zero elsewhere).
template <typename real>
__device__ __forceinline__ void j_prefetch(const SweepArgs<real>& a, Quad<real> (&jv)[3], int k, int j, int i0, int b,
                                           bool live) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    jv[c] = Quad<real>{};
    if (live && a.ade_P == 1 && k >= a.jk0[c] && k < a.jk0[c] + a.jnk[c]) {
      const long long jq = (((long long)b * a.jnk[c] + (k - a.jk0[c])) * a.Y + j) * a.X + i0;
      jv[c] = ld4(a.J[c] + jq);
    }
  }
}

template <typename real, bool kTma, bool kZ, bool kMulti>
__device__ __forceinline__ void e_staged_body(const SweepArgs<real>& a, const SweepMaps& tm, const uint3 bid) {
  constexpr int S = stages<true, kZ>();
  extern __shared__ unsigned char smem_raw[];
  __shared__ unsigned long long bar[S];
  ESlot<real, kZ>* slot = reinterpret_cast<ESlot<real, kZ>*>(align_smem(smem_raw));
  const int tx = threadIdx.x, ty = threadIdx.y;
  const bool leader = tx == 0 && ty == 0;
  const int nx = a.nx, X = a.X, Y = a.Y;
  const BlockSpan sp = block_span<real, kZ>(a, 0, bid);
  if (sp.empty) return;
  const int x0 = sp.x0, y0 = sp.y0, b = sp.b, zr = sp.zr, k0 = sp.k0, k1 = sp.k1;
  const int n_stage = k1 - k0;
  const int i0 = x0 + 4 * tx, j = y0 + ty;
  const bool live = i0 < 4 * sp.box.q1 && j < sp.box.j1 && i0 <= nx + 1;
  const long long base = (long long)b * a.bs;
  const Quad<real> idx4 = i0 < X ? ld4(a.idd[0] + i0) : Quad<real>{};
  const real idy = a.idd[1][min(j, Y - 1)];
  Quad<real> hx_m{}, hy_m{};  // H at plane k - 1, carried
  if (live) {
    const long long p = base + (long long)(k0 - 1) * X * Y + (long long)j * X + i0;
    hx_m = ld4(a.Ho[0] + p);
    hy_m = ld4(a.Ho[1] + p);
  }
  Quad<real> jcur[3];
  j_prefetch(a, jcur, k0, j, i0, b, live);
  if (kTma) {
    if (leader) {
      mbar_setup<S>(bar);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        prefetch_map(&tm.h_wide[c]);
        prefetch_map(&tm.e_tile[c]);
        prefetch_map(&tm.mat[c]);
      }
    }
    __syncthreads();
    if (leader)
      for (int s = 0; s < S && s < n_stage; ++s) e_issue(a, tm, slot[s], &bar[s], b, zr, k0 + s, x0, y0);
  } else {
#pragma unroll
    for (int s = 0; s < S; ++s) {
      e_stage(a, slot[s], b, zr, k0 + s, k1, x0, y0);
      cp_commit();
    }
  }
  for (int k = k0; k < k1; ++k) {
    const int t = k - k0;
    Quad<real> jnext[3];
    j_prefetch(a, jnext, k + 1 < k1 ? k + 1 : -1, j, i0, b, live);
    if (kTma) {
      const bool ok = wait_plane<S>(bar, t);
      if (__syncthreads_or(!ok)) {
        abort_march<S>(bar, t, min(n_stage, t + S), a.status, leader);
        return;
      }
    } else {
      cp_wait<S - 1>();
      __syncthreads();
    }
    const ESlot<real, kZ>& cur = slot[t % S];
    if (live) {
      const long long q = (long long)k * X * Y + (long long)j * X + i0;
      const real idz = a.idd[2][k];
      const Quad<real> hx = ld4(&cur.h[0].v[ty + 1][4 * tx + 4]), hy = ld4(&cur.h[1].v[ty + 1][4 * tx + 4]);
      const Quad<real> hz = ld4(&cur.h[2].v[ty + 1][4 * tx + 4]);
      const Quad<real> hzy = ld4(&cur.h[2].v[ty][4 * tx + 4]), hxy = ld4(&cur.h[0].v[ty][4 * tx + 4]);
      const real hz_l = cur.h[2].v[ty + 1][4 * tx + 3], hy_l = cur.h[1].v[ty + 1][4 * tx + 3];
      ZTerm<real> zt[2];
      zt[0].on = zt[1].on = false;
      if constexpr (kZ) {
        zt[0] = z_term(a, a.ecorr[0][1], a.zsd[0][zr][0], &cur.z.p[0].v[ty][4 * tx], b, k, j, i0, 0);
        zt[1] = z_term(a, a.ecorr[1][1], a.zsd[0][zr][1], &cur.z.p[1].v[ty][4 * tx], b, k, j, i0, 0);
      }
      real d0[4], d1[4];
      // Ex: terms (a = y, +Hz) then (a = z, -Hy)
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        d0[e] = (hz.v[e] - hzy.v[e]) * idy;
        d1[e] = (hy.v[e] - hy_m.v[e]) * idz;
      }
      e_apply<real, kZ, kMulti>(a, 0, a.Eo[0] + base, q, ld4(&cur.e[0].v[ty][4 * tx]), &cur.m[0].v[ty][4 * tx], d0, d1,
                        true, jcur[0], zt[0], i0, j, k, b);
      // Ey: terms (a = z, +Hx) then (a = x, -Hz); d0 is the x term, d1 the z term
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const real hzl = e > 0 ? hz.v[e - 1] : hz_l;
        d0[e] = (hz.v[e] - hzl) * idx4.v[e];
        d1[e] = (hx.v[e] - hx_m.v[e]) * idz;
      }
      e_apply<real, kZ, kMulti>(a, 1, a.Eo[1] + base, q, ld4(&cur.e[1].v[ty][4 * tx]), &cur.m[1].v[ty][4 * tx], d0, d1,
                        false, jcur[1], zt[1], i0, j, k, b);
      // Ez: terms (a = x, +Hy) then (a = y, -Hx); no z term
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const real hyl = e > 0 ? hy.v[e - 1] : hy_l;
        d0[e] = (hy.v[e] - hyl) * idx4.v[e];
        d1[e] = (hx.v[e] - hxy.v[e]) * idy;
      }
      ZTerm<real> none;
      none.on = false;
      e_apply<real, false, kMulti>(a, 2, a.Eo[2] + base, q, ld4(&cur.e[2].v[ty][4 * tx]), &cur.m[2].v[ty][4 * tx], d0, d1,
                           true, jcur[2], none, i0, j, k, b);
      hx_m = hx;
      hy_m = hy;
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) jcur[c] = jnext[c];
    __syncthreads();
    if (kTma) {
      if (leader && t + S < n_stage) {
        fence_proxy_async();
        e_issue(a, tm, slot[t % S], &bar[t % S], b, zr, k + S, x0, y0);
      }
    } else {
      e_stage(a, slot[t % S], b, zr, k + S, k1, x0, y0);
      cp_commit();
    }
  }
  if (!kTma) cp_wait<0>();
}

template <typename real, bool kTma, bool kZ, bool kMulti>
__global__ void __launch_bounds__(256, 2)
    e_staged_kernel(const __grid_constant__ SweepArgs<real> a, const __grid_constant__ SweepMaps tm) {
  e_staged_body<real, kTma, kZ, kMulti>(a, tm, blockIdx);
}

// Several engines' E sweeps in one launch: engine e's arguments at A[e] and M[e].
template <typename real, bool kTma, bool kZ, bool kMulti>
__global__ void __launch_bounds__(256, 2)
    e_staged_batch_kernel(const SweepArgs<real>* __restrict__ A, const SweepMaps* __restrict__ M, const BatchGrid G) {
  __shared__ __align__(16) unsigned char args[sizeof(SweepArgs<real>)];
  int e;
  const uint3 bid = G.block(&e);
  e_staged_body<real, kTma, kZ, kMulti>(stage_args(A + e, args), M[e], bid);
}

// ------------------------------------------------------------------------------------- launch
template <typename real, bool kTma, bool kZ>
cudaError_t launch_one(const SweepArgs<real>& a, const SweepMaps& m, cudaStream_t s, bool h, dim3 grid) {
  dim3 block(kTQ, kTY);
  if (h) {
    const size_t bytes = sizeof(HSlot<real, kZ>) * stages<false, kZ>() + 128;
    auto kern = h_staged_kernel<real, kTma, kZ>;
    const cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (err != cudaSuccess) return err;
    kern<<<grid, block, bytes, s>>>(a, m);
  } else {
    const size_t bytes = sizeof(ESlot<real, kZ>) * stages<true, kZ>() + 128;
    // more than one Debye pole: the general update (a call); single-pole runs compile without it
    auto kern = a.ade_P > 1 ? e_staged_kernel<real, kTma, kZ, true> : e_staged_kernel<real, kTma, kZ, false>;
    const cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (err != cudaSuccess) return err;
    kern<<<grid, block, bytes, s>>>(a, m);
  }
  return cudaGetLastError();
}

template <typename real>
cudaError_t staged_grids(const SweepArgs<real>& a, int kind, dim3* inner, dim3* z) {
  // Every TMA box starts at x = 4 (q0 + 32 n) (the E sweep's halo box 4 cells earlier, which may
  // be -4: a load may start before the grid): a multiple of 8 cells keeps the start 16-byte
  // aligned for the 2-byte index boxes too.
  *inner = dim3(0, 0, 0);
  *z = dim3(0, 0, 0);
  const Span3 in = a.inner[kind];
  if (in.q1 > in.q0 && in.j1 > in.j0 && in.k1 > in.k0) {
    if (in.q0 % 2 != 0) return cudaErrorInvalidValue;
    const int nkc = (in.k1 - in.k0 + a.tile_z - 1) / a.tile_z;
    *inner = dim3((in.q1 - in.q0 + kTQ - 1) / kTQ, (in.j1 - in.j0 + kTY - 1) / kTY, nkc * a.B);
  }
  // the z-slab planes over the same x-y extent: one block per tile, member and side
  int nq = 0, nj = 0;
  for (int zr = 0; zr < 2; ++zr) {
    const Span3& zb = a.zin[kind][zr];
    if (zb.k1 <= zb.k0 || zb.q1 <= zb.q0 || zb.j1 <= zb.j0) continue;
    if (zb.q0 % 2 != 0) return cudaErrorInvalidValue;
    nq = max(nq, zb.q1 - zb.q0);
    nj = max(nj, zb.j1 - zb.j0);
  }
  if (nq > 0 && nj > 0) *z = dim3((nq + kTQ - 1) / kTQ, (nj + kTY - 1) / kTY, 2 * a.B);
  return cudaSuccess;
}

template <typename real>
cudaError_t launch_staged_sweep(const SweepArgs<real>& a, const SweepMaps& m, cudaStream_t s, bool h) {
  const bool tma = a.staged == 2;
  dim3 inner, z;
  if (const cudaError_t e = staged_grids(a, h ? 1 : 0, &inner, &z)) return e;
  if (inner.x > 0) {
    const cudaError_t err = tma ? launch_one<real, true, false>(a, m, s, h, inner)
                                : launch_one<real, false, false>(a, m, s, h, inner);
    if (err != cudaSuccess) return err;
  }
  if (z.x > 0) {
    const cudaError_t err = tma ? launch_one<real, true, true>(a, m, s, h, z) : launch_one<real, false, true>(a, m, s, h, z);
    if (err != cudaSuccess) return err;
  }
  return cudaSuccess;
}

template <typename real, bool kTma, bool kZ>
cudaError_t launch_batch_one(const SweepArgs<real>* A, const SweepMaps* M, const BatchGrid& G, int blocks, bool h,
                             bool multi_pole, cudaStream_t s) {
  const dim3 block(kTQ, kTY);
  if (h) {
    const size_t bytes = sizeof(HSlot<real, kZ>) * stages<false, kZ>() + 128;
    auto kern = h_staged_batch_kernel<real, kTma, kZ>;
    const cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (err != cudaSuccess) return err;
    kern<<<blocks, block, bytes, s>>>(A, M, G);
  } else {
    const size_t bytes = sizeof(ESlot<real, kZ>) * stages<true, kZ>() + 128;
    auto kern = multi_pole ? e_staged_batch_kernel<real, kTma, kZ, true> : e_staged_batch_kernel<real, kTma, kZ, false>;
    const cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (err != cudaSuccess) return err;
    kern<<<blocks, block, bytes, s>>>(A, M, G);
  }
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_staged_batch(const SweepArgs<real>* A, const SweepMaps* M, const BatchGrid& G, int blocks, bool h,
                                bool tma, bool z, bool multi_pole, cudaStream_t s) {
  if (blocks <= 0) return cudaSuccess;
  if (tma) return z ? launch_batch_one<real, true, true>(A, M, G, blocks, h, multi_pole, s)
                    : launch_batch_one<real, true, false>(A, M, G, blocks, h, multi_pole, s);
  return z ? launch_batch_one<real, false, true>(A, M, G, blocks, h, multi_pole, s)
           : launch_batch_one<real, false, false>(A, M, G, blocks, h, multi_pole, s);
}

// ------------------------------------------------------------------------------- descriptors
using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiled encoder() {
  static EncodeTiled fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiled>(p);
  });
  return fn;
}

// dims/box innermost first; strides in bytes for dims 1..rank-1.
bool encode_tensor_map(CUtensorMap* m, CUtensorMapDataType dt, int rank, const void* base, const cuuint64_t* dims,
                       const cuuint64_t* strides, const cuuint32_t* box, const char* what, std::string* why,
                       CUtensorMapSwizzle swizzle) {
  const EncodeTiled f = encoder();
  if (f == nullptr) {
    *why = "the driver does not provide cuTensorMapEncodeTiled";
    return false;
  }
  const cuuint32_t ones[4] = {1, 1, 1, 1};
  const CUresult r = f(m, dt, (cuuint32_t)rank, const_cast<void*>(base), dims, strides, box, ones,
                       CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                       CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    *why = std::string("cuTensorMapEncodeTiled(") + what + ") returned " + std::to_string((int)r);
    return false;
  }
  return true;
}


template <typename real>
bool encode_sweep_maps(const SweepArgs<real>& a, SweepMaps* m, std::string* why) {
  const CUtensorMapDataType dt = sizeof(real) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
  const cuuint64_t X = (cuuint64_t)a.X, Y = (cuuint64_t)a.Y, Z = (cuuint64_t)a.nz + 2, B = (cuuint64_t)a.B;
  const cuuint64_t dims[4] = {X, Y, Z, B};
  const cuuint64_t rs = sizeof(real);
  const cuuint64_t strides[3] = {X * rs, X * Y * rs, X * Y * Z * rs};
  const cuuint32_t wide[4] = {kHW, kTY + 1, 1, 1};
  const cuuint32_t tile[4] = {kTW, kTY, 1, 1};
  const cuuint64_t mdims[3] = {X, Y, Z};
  const cuuint64_t mstrides[2] = {X * 2, X * Y * 2};
  for (int c = 0; c < 3; ++c) {
    if (!encode_tensor_map(&m->e_wide[c], dt, 4, a.E[c], dims, strides, wide, "E wide", why) ||
        !encode_tensor_map(&m->e_tile[c], dt, 4, a.E[c], dims, strides, tile, "E tile", why) ||
        !encode_tensor_map(&m->h_wide[c], dt, 4, a.Ho[c], dims, strides, wide, "H wide", why) ||
        !encode_tensor_map(&m->h_tile[c], dt, 4, a.H[c], dims, strides, tile, "H tile", why) ||
        !encode_tensor_map(&m->mat[c], CU_TENSOR_MAP_DATA_TYPE_UINT16, 3, a.mat[c], mdims, mstrides, tile, "mat", why))
      return false;
  }
  for (int kind = 0; kind < 2; ++kind)
    for (int cc = 0; cc < 2; ++cc)
      for (int zr = 0; zr < 2; ++zr) {
        const int sd = a.zsd[kind][zr][cc];
        if (sd < 0) continue;
        const CpmlSide<real>& s = (kind == 0 ? a.ecorr[cc][1] : a.hcorr[cc][1]).side[sd];
        const cuuint64_t w = (cuuint64_t)(s.hi[2] - s.lo[2]);
        const cuuint64_t pdims[4] = {X, Y, w, B};
        const cuuint64_t pstrides[3] = {X * rs, X * Y * rs, X * Y * w * rs};
        if (!encode_tensor_map(&m->psi_z[kind][cc][zr], dt, 4, s.psi, pdims, pstrides, tile, "psi", why)) return false;
      }
  return true;
}

static_assert(sizeof(Box<float, kTY + 1, kHW>) % 128 == 0 && sizeof(Box<uint16_t, kTY, kTW>) % 128 == 0,
              "staged arrays keep the 128-byte alignment TMA destinations need");
static_assert((kHW * sizeof(float)) % 16 == 0 && (kTW * sizeof(uint16_t)) % 16 == 0,
              "TMA box rows are whole 16-byte units");
static_assert(sizeof(ESlot<float, false>) * stages<true, false>() + 128 <= 113 * 1024 &&
                  sizeof(ESlot<float, true>) * stages<true, true>() + 128 <= 113 * 1024 &&
                  sizeof(HSlot<float, true>) * stages<false, true>() + 128 <= 113 * 1024,
              "two blocks per SM for every float sweep");

template <typename real>
cudaError_t preload_staged() {
  cudaFuncAttributes fa;
  const void* fns[] = {
      reinterpret_cast<const void*>(h_staged_kernel<real, true, false>),
      reinterpret_cast<const void*>(h_staged_kernel<real, true, true>),
      reinterpret_cast<const void*>(h_staged_kernel<real, false, false>),
      reinterpret_cast<const void*>(h_staged_kernel<real, false, true>),
      reinterpret_cast<const void*>(e_staged_kernel<real, true, false, false>),
      reinterpret_cast<const void*>(e_staged_kernel<real, true, true, false>),
      reinterpret_cast<const void*>(e_staged_kernel<real, false, false, false>),
      reinterpret_cast<const void*>(e_staged_kernel<real, false, true, false>),
      reinterpret_cast<const void*>(e_staged_kernel<real, true, false, true>),
      reinterpret_cast<const void*>(e_staged_kernel<real, true, true, true>),
      reinterpret_cast<const void*>(e_staged_kernel<real, false, false, true>),
      reinterpret_cast<const void*>(e_staged_kernel<real, false, true, true>),
      reinterpret_cast<const void*>(h_staged_batch_kernel<real, true, false>),
      reinterpret_cast<const void*>(h_staged_batch_kernel<real, true, true>),
      reinterpret_cast<const void*>(h_staged_batch_kernel<real, false, false>),
      reinterpret_cast<const void*>(h_staged_batch_kernel<real, false, true>),
      reinterpret_cast<const void*>(e_staged_batch_kernel<real, true, false, false>),
      reinterpret_cast<const void*>(e_staged_batch_kernel<real, true, true, false>),
      reinterpret_cast<const void*>(e_staged_batch_kernel<real, false, false, false>),
      reinterpret_cast<const void*>(e_staged_batch_kernel<real, false, true, false>),
      reinterpret_cast<const void*>(e_staged_batch_kernel<real, true, false, true>),
      reinterpret_cast<const void*>(e_staged_batch_kernel<real, true, true, true>),
      reinterpret_cast<const void*>(e_staged_batch_kernel<real, false, false, true>),
      reinterpret_cast<const void*>(e_staged_batch_kernel<real, false, true, true>),
  };
  for (const void* f : fns) {
    const cudaError_t err = cudaFuncGetAttributes(&fa, f);
    if (err != cudaSuccess) return err;
  }
  return cudaSuccess;
}

template cudaError_t preload_staged<float>();
template cudaError_t preload_staged<double>();
template cudaError_t staged_grids<float>(const SweepArgs<float>&, int, dim3*, dim3*);
template cudaError_t staged_grids<double>(const SweepArgs<double>&, int, dim3*, dim3*);
template cudaError_t launch_staged_batch<float>(const SweepArgs<float>*, const SweepMaps*, const BatchGrid&, int, bool,
                                                bool, bool, bool, cudaStream_t);
template cudaError_t launch_staged_batch<double>(const SweepArgs<double>*, const SweepMaps*, const BatchGrid&, int,
                                                 bool, bool, bool, bool, cudaStream_t);
template cudaError_t launch_staged_sweep<float>(const SweepArgs<float>&, const SweepMaps&, cudaStream_t, bool);
template cudaError_t launch_staged_sweep<double>(const SweepArgs<double>&, const SweepMaps&, cudaStream_t, bool);
template bool encode_sweep_maps<float>(const SweepArgs<float>&, SweepMaps*, std::string*);
template bool encode_sweep_maps<double>(const SweepArgs<double>&, SweepMaps*, std::string*);

}  // namespace oafdtd
