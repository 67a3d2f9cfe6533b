// Sweeps with the planes staged through shared memory by a cp.async pipeline (the default
// variant).
//
// A block owns a 2-D tile of 32 quads (128 x cells) by 8 rows and marches up a chunk of z
// planes. Each plane's inputs (the tile plus the one-cell halo the curl needs) are copied into a
// ring of three shared-memory slots with 16-byte cp.async copies, two planes ahead of the plane
// being computed, so every SM keeps ~100 KB of loads in flight without holding them in
// registers; the Debye currents of the next plane are prefetched into registers. Neighbours in
// x and y are read from the staged tile; results go straight to global memory.
//
// One launch per sweep gives every cell its bulk update (and, in the E sweep, its Debye update);
// the CPML corrections follow in the correction passes (cpml.cu). The arithmetic is the
// reference's, operation by operation (packages/oa-fdtd/src/oa_fdtd/reference.py:152-180,
// :119-127).

#include "device_common.cuh"

namespace oafdtd {

constexpr int kTQ = 32;       // quads per tile row (128 cells)
constexpr int kTY = 8;        // rows per tile
constexpr int kTW = 4 * kTQ;  // tile width in cells
constexpr int kHW = kTW + 4;  // staged width with a one-quad halo
constexpr int kStages = 3;

// ------------------------------------------------------------------------------------- H sweep
// Slot: E[3][kTY + 1][kHW] (rows y0..y0+8, x0..x0+131), H[3][kTY][kTW].
template <typename real>
struct HSlot {
  real e[3][kTY + 1][kHW];
  real h[3][kTY][kTW];
};

// Stage plane k: E for k <= k1 (plane k1 only feeds the z derivative of plane k1 - 1), H for
// k < k1.
template <typename real>
__device__ __forceinline__ void h_stage(const SweepArgs<real>& a, HSlot<real>& s, int b, int k, int k1, int x0,
                                        int y0) {
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
      cp_async16(&s.e[c][r][4 * q] + part * EL, a.E[c] + base + (long long)y * X + x + part * EL);
    } else {
      const int u = t - ecount;
      const int part = u % CQ, q = (u / CQ) % (kTW / 4), r = (u / CQ / (kTW / 4)) % kTY;
      const int c = u / CQ / (kTW / 4) / kTY;
      const int x = x0 + 4 * q, y = y0 + r;
      if (x >= X || y >= Y) continue;
      cp_async16(&s.h[c][r][4 * q] + part * EL, a.H[c] + base + (long long)y * X + x + part * EL);
    }
  }
}

template <typename real>
__global__ void __launch_bounds__(256, 2) h_staged_kernel(const __grid_constant__ SweepArgs<real> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  HSlot<real>* slot = reinterpret_cast<HSlot<real>*>(smem_raw);
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int nx = a.nx, ny = a.ny, nz = a.nz, X = a.X, Y = a.Y;
  const int x0 = blockIdx.x * kTW, y0 = 1 + blockIdx.y * kTY;
  const int nkc = (nz + 1 + a.tile_z - 1) / a.tile_z;
  const int b = blockIdx.z / nkc, kc = blockIdx.z % nkc;
  const int k0 = 1 + kc * a.tile_z, k1 = min(k0 + a.tile_z, nz + 2);
  const int i0 = x0 + 4 * tx, j = y0 + ty;
  const bool live = i0 < X && j <= ny + 1 && i0 <= nx + 1;
  const long long base = (long long)b * a.bs;
  const real dtmu = a.dtmu;
  const Quad<real> ipx = i0 < X ? ld4(a.ip[0] + i0) : Quad<real>{};
  const real ipy = a.ip[1][min(j, Y - 1)];
#pragma unroll
  for (int s = 0; s < kStages; ++s) {
    h_stage(a, slot[s], b, k0 + s, k1, x0, y0);
    cp_commit();
  }
  for (int k = k0; k < k1; ++k) {
    cp_wait<kStages - 2>();
    __syncthreads();
    const HSlot<real>& cur = slot[(k - k0) % kStages];
    const HSlot<real>& nxt = slot[(k - k0 + 1) % kStages];
    if (live) {
      const long long p = base + (long long)k * X * Y + (long long)j * X + i0;
      const bool kin = k <= nz;
      const real ipz = a.ip[2][k];
      const Quad<real> ex = ld4(&cur.e[0][ty][4 * tx]), ey = ld4(&cur.e[1][ty][4 * tx]);
      const Quad<real> ez = ld4(&cur.e[2][ty][4 * tx]);
      const real ez_r = cur.e[2][ty][4 * tx + 4], ey_r = cur.e[1][ty][4 * tx + 4];
      if (j <= ny && kin) {  // Hx: node along x (1..nx+1), cell along y and z
        const Quad<real> ezy = ld4(&cur.e[2][ty + 1][4 * tx]);
        const Quad<real> ey1 = ld4(&nxt.e[1][ty][4 * tx]);
        Quad<real> h = ld4(&cur.h[0][ty][4 * tx]);
        real d0[4], d1[4];
        bool valid[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int i = i0 + e;
          valid[e] = i >= 1 && i <= nx + 1;
          d0[e] = (ezy.v[e] - ez.v[e]) * ipy;  // axis y
          d1[e] = (ey1.v[e] - ey.v[e]) * ipz;  // axis z
          if (valid[e]) h.v[e] = h.v[e] + dtmu * ((-d0[e]) + d1[e]);
        }
        st4(a.H[0] + p, h);
      }
      if (kin) {  // Hy: cell along x (1..nx), node along y (1..ny+1), cell along z
        const Quad<real> ex1 = ld4(&nxt.e[0][ty][4 * tx]);
        Quad<real> h = ld4(&cur.h[1][ty][4 * tx]);
        real d0[4], d1[4];
        bool valid[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int i = i0 + e;
          valid[e] = i >= 1 && i <= nx;
          const real ezr = e < 3 ? ez.v[e + 1] : ez_r;
          d0[e] = (ezr - ez.v[e]) * ipx.v[e];  // axis x
          d1[e] = (ex1.v[e] - ex.v[e]) * ipz;  // axis z
          if (valid[e]) h.v[e] = h.v[e] + dtmu * ((-d1[e]) + d0[e]);
        }
        st4(a.H[1] + p, h);
      }
      if (j <= ny) {  // Hz: cell along x and y, node along z (1..nz+1)
        const Quad<real> exy = ld4(&cur.e[0][ty + 1][4 * tx]);
        Quad<real> h = ld4(&cur.h[2][ty][4 * tx]);
        real d0[4], d1[4];
        bool valid[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int i = i0 + e;
          valid[e] = i >= 1 && i <= nx;
          const real eyr = e < 3 ? ey.v[e + 1] : ey_r;
          d0[e] = (eyr - ey.v[e]) * ipx.v[e];  // axis x
          d1[e] = (exy.v[e] - ex.v[e]) * ipy;  // axis y
          if (valid[e]) h.v[e] = h.v[e] + dtmu * ((-d0[e]) + d1[e]);
        }
        st4(a.H[2] + p, h);
      }
    }
    __syncthreads();  // every thread is done with the slot of plane k
    h_stage(a, slot[(k - k0) % kStages], b, k + kStages, k1, x0, y0);
    cp_commit();
  }
  cp_wait<0>();
}

// ------------------------------------------------------------------------------------- E sweep
// Slot: H[3][kTY + 1][kHW] (rows y0-1..y0+7, x0-4..x0+127), E[3][kTY][kTW], mat[3][kTY][kTW].
template <typename real>
struct ESlot {
  real h[3][kTY + 1][kHW];
  real e[3][kTY][kTW];
  uint16_t m[3][kTY][kTW];
};

template <typename real>
__device__ __forceinline__ void e_stage(const SweepArgs<real>& a, ESlot<real>& s, int b, int k, int kend, int x0,
                                        int y0) {
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
      cp_async16(&s.h[c][r][4 * q] + part * EL, a.H[c] + base + (long long)y * X + x + part * EL);
    } else if (t < hcount + ecount) {
      const int u = t - hcount;
      const int part = u % CQ, q = (u / CQ) % (kTW / 4), r = (u / CQ / (kTW / 4)) % kTY;
      const int c = u / CQ / (kTW / 4) / kTY;
      const int x = x0 + 4 * q, y = y0 + r;
      if (x >= X || y >= Y) continue;
      cp_async16(&s.e[c][r][4 * q] + part * EL, a.E[c] + base + (long long)y * X + x + part * EL);
    } else {
      const int u = t - hcount - ecount;
      const int q = u % (kTW / 8), r = (u / (kTW / 8)) % kTY, c = u / (kTW / 8) / kTY;
      const int x = x0 + 8 * q, y = y0 + r;
      if (x >= X || y >= Y) continue;
      cp_async16(&s.m[c][r][8 * q], a.mat[c] + plane + (long long)y * X + x);
    }
  }
}

// Bulk update, CPML and the Debye update of one E component on one quad. d0/d1 are the
// derivatives along the component's two axes in ascending order; the reference's term order is
// (d0, -d1) when first_plus, else (d1, -d0). j4 holds the prefetched Debye current (P = 1).
template <typename real>
__device__ __forceinline__ void e_apply(const SweepArgs<real>& a, int c, real* __restrict__ E, long long p,
                                        const Quad<real>& e_old, const uint16_t* m, const real (&d0)[4],
                                        const real (&d1)[4], bool first_plus, const Quad<real>& j4in,
                                        int i0, int j, int k, int b) {
  const int X = a.X, Y = a.Y, nx = a.nx;
  Quad<real> e4 = e_old;
  Coef<real> cf[4];
  real kf[4];
  bool valid[4];
  bool disp = false;
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int i = i0 + e;
    cf[e] = a.coef[m[e]];
    kf[e] = cf[e].cb;
    valid[e] = i >= 1 && i <= nx + 1;
    const real acc = first_plus ? d0[e] + (-d1[e]) : d1[e] + (-d0[e]);
    if (valid[e]) e4.v[e] = cf[e].ca * e4.v[e] + cf[e].cb * acc;
    disp |= valid[e] && m[e] >= a.ade_lo && m[e] < a.ade_hi;
  }
  if (disp) {
    const long long jstride = (long long)a.B * a.jnk[c] * Y * X;
    const long long jq = (((long long)b * a.jnk[c] + (k - a.jk0[c])) * Y + j) * X + i0;
    real* J = a.J[c];
    if (a.ade_P == 1) {
      Quad<real> j4 = j4in;
      const real onekp = a.ade_onekp[0], kp = a.ade_kp[0];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        if (!(valid[e] && m[e] >= a.ade_lo && m[e] < a.ade_hi)) continue;
        const real jt = (real)0.5 * (onekp * j4.v[e]);
        const real en = e4.v[e] - cf[e].cbe * jt;
        const real de = en - e_old.v[e];
        j4.v[e] = kp * j4.v[e] + cf[e].beta0 * de;
        e4.v[e] = en;
      }
      st4(J + jq, j4);
    } else {
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        if (!(valid[e] && m[e] >= a.ade_lo && m[e] < a.ade_hi)) continue;
        e4.v[e] = ade_cell(e4.v[e], e_old.v[e], cf[e].cbe, cf[e].beta0, m[e], J, jq + e, jstride, a.ade_kp,
                           a.ade_onekp, a.ade_beta, a.ade_P);
      }
    }
  }
  st4(E + p, e4);
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

template <typename real>
__global__ void __launch_bounds__(256, 2) e_staged_kernel(const __grid_constant__ SweepArgs<real> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ESlot<real>* slot = reinterpret_cast<ESlot<real>*>(smem_raw);
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int nx = a.nx, ny = a.ny, nz = a.nz, X = a.X, Y = a.Y;
  const int x0 = blockIdx.x * kTW, y0 = 1 + blockIdx.y * kTY;
  const int nkc = (nz + 1 + a.tile_z - 1) / a.tile_z;
  const int b = blockIdx.z / nkc, kc = blockIdx.z % nkc;
  const int k0 = 1 + kc * a.tile_z, k1 = min(k0 + a.tile_z, nz + 2);
  const int i0 = x0 + 4 * tx, j = y0 + ty;
  const bool live = i0 < X && j <= ny + 1 && i0 <= nx + 1;
  const long long base = (long long)b * a.bs;
  const Quad<real> idx4 = i0 < X ? ld4(a.idd[0] + i0) : Quad<real>{};
  const real idy = a.idd[1][min(j, Y - 1)];
  Quad<real> hx_m{}, hy_m{};  // H at plane k - 1, carried
  if (live) {
    const long long p = base + (long long)(k0 - 1) * X * Y + (long long)j * X + i0;
    hx_m = ld4(a.H[0] + p);
    hy_m = ld4(a.H[1] + p);
  }
  Quad<real> jcur[3];
  j_prefetch(a, jcur, k0, j, i0, b, live);
#pragma unroll
  for (int s = 0; s < kStages; ++s) {
    e_stage(a, slot[s], b, k0 + s, k1, x0, y0);
    cp_commit();
  }
  for (int k = k0; k < k1; ++k) {
    Quad<real> jnext[3];
    j_prefetch(a, jnext, k + 1 < k1 ? k + 1 : -1, j, i0, b, live);
    cp_wait<kStages - 1>();
    __syncthreads();
    const ESlot<real>& cur = slot[(k - k0) % kStages];
    if (live) {
      const long long q = (long long)k * X * Y + (long long)j * X + i0;
      const real idz = a.idd[2][k];
      const Quad<real> hx = ld4(&cur.h[0][ty + 1][4 * tx + 4]), hy = ld4(&cur.h[1][ty + 1][4 * tx + 4]);
      const Quad<real> hz = ld4(&cur.h[2][ty + 1][4 * tx + 4]);
      const Quad<real> hzy = ld4(&cur.h[2][ty][4 * tx + 4]), hxy = ld4(&cur.h[0][ty][4 * tx + 4]);
      const real hz_l = cur.h[2][ty + 1][4 * tx + 3], hy_l = cur.h[1][ty + 1][4 * tx + 3];
      real d0[4], d1[4];
      // Ex: terms (a = y, +Hz) then (a = z, -Hy)
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        d0[e] = (hz.v[e] - hzy.v[e]) * idy;
        d1[e] = (hy.v[e] - hy_m.v[e]) * idz;
      }
      e_apply<real>(a, 0, a.E[0] + base, q, ld4(&cur.e[0][ty][4 * tx]), &cur.m[0][ty][4 * tx], d0, d1, true, jcur[0], i0, j, k, b);
      // Ey: terms (a = z, +Hx) then (a = x, -Hz); d0 is the x term, d1 the z term
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const real hzl = e > 0 ? hz.v[e - 1] : hz_l;
        d0[e] = (hz.v[e] - hzl) * idx4.v[e];
        d1[e] = (hx.v[e] - hx_m.v[e]) * idz;
      }
      e_apply<real>(a, 1, a.E[1] + base, q, ld4(&cur.e[1][ty][4 * tx]), &cur.m[1][ty][4 * tx], d0, d1, false, jcur[1], i0, j, k, b);
      // Ez: terms (a = x, +Hy) then (a = y, -Hx)
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const real hyl = e > 0 ? hy.v[e - 1] : hy_l;
        d0[e] = (hy.v[e] - hyl) * idx4.v[e];
        d1[e] = (hx.v[e] - hxy.v[e]) * idy;
      }
      e_apply<real>(a, 2, a.E[2] + base, q, ld4(&cur.e[2][ty][4 * tx]), &cur.m[2][ty][4 * tx], d0, d1, true, jcur[2], i0, j, k, b);
      hx_m = hx;
      hy_m = hy;
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) jcur[c] = jnext[c];
    __syncthreads();
    e_stage(a, slot[(k - k0) % kStages], b, k + kStages, k1, x0, y0);
    cp_commit();
  }
  cp_wait<0>();
}

// ------------------------------------------------------------------------------------- launch
template <typename real>
cudaError_t launch_staged_sweep(const SweepArgs<real>& a, cudaStream_t s, bool h) {
  const int nkc = (a.nz + 1 + a.tile_z - 1) / a.tile_z;
  dim3 block(kTQ, kTY);
  dim3 grid((a.X + kTW - 1) / kTW, (a.ny + 1 + kTY - 1) / kTY, nkc * a.B);
  cudaError_t err;
  if (h) {
    const size_t bytes = sizeof(HSlot<real>) * kStages;
    err = cudaFuncSetAttribute(h_staged_kernel<real>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (err != cudaSuccess) return err;
    h_staged_kernel<real><<<grid, block, bytes, s>>>(a);
  } else {
    const size_t bytes = sizeof(ESlot<real>) * kStages;
    err = cudaFuncSetAttribute(e_staged_kernel<real>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (err != cudaSuccess) return err;
    e_staged_kernel<real><<<grid, block, bytes, s>>>(a);
  }
  return cudaGetLastError();
}

template cudaError_t launch_staged_sweep<float>(const SweepArgs<float>&, cudaStream_t, bool);
template cudaError_t launch_staged_sweep<double>(const SweepArgs<double>&, cudaStream_t, bool);

}  // namespace oafdtd
