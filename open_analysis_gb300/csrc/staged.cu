// Bulk sweeps with the planes staged through shared memory by a cp.async pipeline.
//
// A block owns a 2-D tile of 32 quads (128 x cells) by 8 rows and marches up a chunk of z
// planes. Each plane's inputs (the tile plus the one-cell halo the curl needs) are copied into a
// ring of three shared-memory slots with 16-byte cp.async copies, two planes ahead of the plane
// being computed, so every SM keeps ~100 KB of loads in flight without holding them in
// registers. Neighbours in x and y are read from the staged tile; results go straight to global
// memory. Only cells outside every CPML slab are updated here (the slab launches in sweeps.cu do
// the rest, concurrently); the arithmetic is the same as theirs, operation by operation.

#include "oafdtd_internal.cuh"

namespace oafdtd {

constexpr int kTQ = 32;                  // quads per tile row (128 cells)
constexpr int kTY = 8;                   // rows per tile
constexpr int kTW = 4 * kTQ;             // tile width in cells
constexpr int kHW = kTW + 4;             // staged width with a one-quad halo
constexpr int kStages = 3;

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

template <typename real>
struct Q4 {
  real v[4];
};
__device__ __forceinline__ Q4<float> lds4(const float* p) {
  const float4 t = *reinterpret_cast<const float4*>(p);
  return Q4<float>{{t.x, t.y, t.z, t.w}};
}
__device__ __forceinline__ Q4<double> lds4(const double* p) {
  const double2 a = reinterpret_cast<const double2*>(p)[0], b = reinterpret_cast<const double2*>(p)[1];
  return Q4<double>{{a.x, a.y, b.x, b.y}};
}
__device__ __forceinline__ void stg4(float* p, const Q4<float>& q) {
  *reinterpret_cast<float4*>(p) = make_float4(q.v[0], q.v[1], q.v[2], q.v[3]);
}
__device__ __forceinline__ void stg4(double* p, const Q4<double>& q) {
  reinterpret_cast<double2*>(p)[0] = make_double2(q.v[0], q.v[1]);
  reinterpret_cast<double2*>(p)[1] = make_double2(q.v[2], q.v[3]);
}

template <typename real>
__device__ __forceinline__ bool bulk_quad(const SweepArgs<real>& a, int i0, int j) {
  if (j < 1 || j > a.ny + 1 || i0 > a.nx + 1) return false;
  if (!a.has_cpml) return true;
  bool col = a.slab_y[j] != 0;
#pragma unroll
  for (int e = 0; e < 4; ++e) col |= a.slab_x[i0 + e] != 0;
  return !col;
}

// ------------------------------------------------------------------------------------- H sweep
// Slot layout: E[3][kTY + 1][kHW] (rows y0..y0+8, x0..x0+131), H[3][kTY][kTW].
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
  constexpr int ecount = 3 * (kTY + 1) * (kHW / 4) * CQ;
  constexpr int hcount = 3 * kTY * (kTW / 4) * CQ;
  const int total = k < k1 ? ecount + hcount : ecount;
  for (int t = threadIdx.x + threadIdx.y * blockDim.x; t < total; t += blockDim.x * blockDim.y) {
    if (t < ecount) {
      const int part = t % CQ, q = (t / CQ) % (kHW / 4), r = (t / CQ / (kHW / 4)) % (kTY + 1);
      const int c = t / CQ / (kHW / 4) / (kTY + 1);
      const int x = x0 + 4 * q, y = y0 + r;
      if (x >= X || y >= Y) continue;
      cp_async16(&s.e[c][r][4 * q] + part * (16 / sizeof(real)), a.E[c] + base + (long long)y * X + x + part * (16 / sizeof(real)));
    } else {
      const int u = t - ecount;
      const int part = u % CQ, q = (u / CQ) % (kTW / 4), r = (u / CQ / (kTW / 4)) % kTY;
      const int c = u / CQ / (kTW / 4) / kTY;
      const int x = x0 + 4 * q, y = y0 + r;
      if (x >= X || y >= Y) continue;
      cp_async16(&s.h[c][r][4 * q] + part * (16 / sizeof(real)), a.H[c] + base + (long long)y * X + x + part * (16 / sizeof(real)));
    }
  }
}

template <typename real>
__global__ void __launch_bounds__(256, 2) h_staged_kernel(const __grid_constant__ SweepArgs<real> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  HSlot<real>* slot = reinterpret_cast<HSlot<real>*>(smem_raw);
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int x0 = blockIdx.x * kTW, y0 = 1 + blockIdx.y * kTY;
  const int nkc = (a.zi1 - a.zi0 + a.tile_z - 1) / a.tile_z;
  const int b = blockIdx.z / nkc, kc = blockIdx.z % nkc;
  const int k0 = a.zi0 + kc * a.tile_z, k1 = min(k0 + a.tile_z, a.zi1);
  const int i0 = x0 + 4 * tx, j = y0 + ty;
  const bool live = i0 < a.X && bulk_quad(a, i0, j);
  const int nx = a.nx, ny = a.ny, nz = a.nz, X = a.X, Y = a.Y;
  const long long base = (long long)b * a.bs;
  const real dtmu = a.dtmu;
  const Q4<real> ipx = i0 < X ? lds4(a.ip[0] + i0) : Q4<real>{};
  const real ipy = a.ip[1][min(j, Y - 1)];
  // prologue: stages k0, k0 + 1, k0 + 2
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
      const Q4<real> ex = lds4(&cur.e[0][ty][4 * tx]), ey = lds4(&cur.e[1][ty][4 * tx]);
      const Q4<real> ez = lds4(&cur.e[2][ty][4 * tx]);
      const real ez_r = cur.e[2][ty][4 * tx + 4], ey_r = cur.e[1][ty][4 * tx + 4];
      if (j <= ny && kin) {  // Hx
        const Q4<real> ezy = lds4(&cur.e[2][ty + 1][4 * tx]);
        const Q4<real> ey1 = lds4(&nxt.e[1][ty][4 * tx]);
        Q4<real> h = lds4(&cur.h[0][ty][4 * tx]);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int i = i0 + e;
          if (i < 1 || i > nx + 1) continue;
          const real dy = (ezy.v[e] - ez.v[e]) * ipy;
          const real dz = (ey1.v[e] - ey.v[e]) * ipz;
          h.v[e] = h.v[e] + dtmu * ((-dy) + dz);
        }
        stg4(a.H[0] + p, h);
      }
      if (kin) {  // Hy
        const Q4<real> ex1 = lds4(&nxt.e[0][ty][4 * tx]);
        Q4<real> h = lds4(&cur.h[1][ty][4 * tx]);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int i = i0 + e;
          if (i < 1 || i > nx) continue;
          const real ezr = e < 3 ? ez.v[e + 1] : ez_r;
          const real dz = (ex1.v[e] - ex.v[e]) * ipz;
          const real dx = (ezr - ez.v[e]) * ipx.v[e];
          h.v[e] = h.v[e] + dtmu * ((-dz) + dx);
        }
        stg4(a.H[1] + p, h);
      }
      if (j <= ny) {  // Hz
        const Q4<real> exy = lds4(&cur.e[0][ty + 1][4 * tx]);
        Q4<real> h = lds4(&cur.h[2][ty][4 * tx]);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int i = i0 + e;
          if (i < 1 || i > nx) continue;
          const real eyr = e < 3 ? ey.v[e + 1] : ey_r;
          const real dx = (eyr - ey.v[e]) * ipx.v[e];
          const real dy = (exy.v[e] - ex.v[e]) * ipy;
          h.v[e] = h.v[e] + dtmu * ((-dx) + dy);
        }
        stg4(a.H[2] + p, h);
      }
    }
    __syncthreads();  // every thread is done with the slot of plane k
    h_stage(a, slot[(k - k0) % kStages], b, k + kStages, k1, x0, y0);
    cp_commit();
  }
  cp_wait<0>();
}

// ------------------------------------------------------------------------------------- E sweep
// Slot layout: H[3][kTY + 1][kHW] (rows y0-1..y0+7, x0-4..x0+127), E[3][kTY][kTW],
// mat[3][kTY][kTW].
template <typename real>
struct ESlot {
  real h[3][kTY + 1][kHW];
  real e[3][kTY][kTW];
  uint16_t m[3][kTY][kTW];
};

template <typename real>
__device__ __forceinline__ void e_stage(const SweepArgs<real>& a, ESlot<real>& s, int b, int k, int kend, int x0, int y0) {
  const int X = a.X, Y = a.Y;
  if (k >= kend) return;
  const long long plane = (long long)k * X * Y;
  const long long base = (long long)b * a.bs + plane;
  constexpr int CQ = (int)(4 * sizeof(real) / 16);
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
      cp_async16(&s.h[c][r][4 * q] + part * (16 / sizeof(real)), a.H[c] + base + (long long)y * X + x + part * (16 / sizeof(real)));
    } else if (t < hcount + ecount) {
      const int u = t - hcount;
      const int part = u % CQ, q = (u / CQ) % (kTW / 4), r = (u / CQ / (kTW / 4)) % kTY;
      const int c = u / CQ / (kTW / 4) / kTY;
      const int x = x0 + 4 * q, y = y0 + r;
      if (x >= X || y >= Y) continue;
      cp_async16(&s.e[c][r][4 * q] + part * (16 / sizeof(real)), a.E[c] + base + (long long)y * X + x + part * (16 / sizeof(real)));
    } else {
      const int u = t - hcount - ecount;
      const int q = u % (kTW / 8), r = (u / (kTW / 8)) % kTY, c = u / (kTW / 8) / kTY;
      const int x = x0 + 8 * q, y = y0 + r;
      if (x >= X || y >= Y) continue;
      cp_async16(&s.m[c][r][8 * q], a.mat[c] + plane + (long long)y * X + x);
    }
  }
}

template <typename real>
__device__ __forceinline__ void e_apply(const SweepArgs<real>& a, int c, real* __restrict__ E, long long p,
                                        const Q4<real>& e_old, const uint16_t* m, const real (&d0)[4],
                                        const real (&d1)[4], bool first_plus, int i0, int j, int k, int b) {
  const int X = a.X, Y = a.Y, nx = a.nx;
  Q4<real> e4 = e_old;
  Coef<real> cf[4];
  bool disp = false;
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int i = i0 + e;
    cf[e] = a.coef[m[e]];
    if (i < 1 || i > nx + 1) continue;
    const real acc = first_plus ? d0[e] + (-d1[e]) : d1[e] + (-d0[e]);
    e4.v[e] = cf[e].ca * e4.v[e] + cf[e].cb * acc;
    disp |= m[e] >= a.ade_lo && m[e] < a.ade_hi;
  }
  if (disp) {
    const long long jstride = (long long)a.B * a.jnk[c] * Y * X;
    const long long jq = (((long long)b * a.jnk[c] + (k - a.jk0[c])) * Y + j) * X + i0;
    real* J = a.J[c];
    if (a.ade_P == 1) {
      Q4<real> j4 = lds4(J + jq);
      const real onekp = a.ade_onekp[0], kp = a.ade_kp[0];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int i = i0 + e;
        if (i < 1 || i > nx + 1 || !(m[e] >= a.ade_lo && m[e] < a.ade_hi)) continue;
        const real jt = (real)0.5 * (onekp * j4.v[e]);
        const real en = e4.v[e] - cf[e].cbe * jt;
        const real de = en - e_old.v[e];
        j4.v[e] = kp * j4.v[e] + cf[e].beta0 * de;
        e4.v[e] = en;
      }
      stg4(J + jq, j4);
    } else {
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int i = i0 + e;
        if (i < 1 || i > nx + 1 || !(m[e] >= a.ade_lo && m[e] < a.ade_hi)) continue;
        real jt = (real)0;
        for (int q = 0; q < a.ade_P; ++q) jt = jt + a.ade_onekp[q] * J[jq + e + q * jstride];
        jt = (real)0.5 * jt;
        const real en = e4.v[e] - cf[e].cbe * jt;
        const real de = en - e_old.v[e];
        for (int q = 0; q < a.ade_P; ++q) {
          const long long jj = jq + e + q * jstride;
          const real bp = q == 0 ? cf[e].beta0 : a.ade_beta[(long long)m[e] * a.ade_P + q];
          J[jj] = a.ade_kp[q] * J[jj] + bp * de;
        }
        e4.v[e] = en;
      }
    }
  }
  stg4(E + p, e4);
}

template <typename real>
__global__ void __launch_bounds__(256, 2) e_staged_kernel(const __grid_constant__ SweepArgs<real> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ESlot<real>* slot = reinterpret_cast<ESlot<real>*>(smem_raw);
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int x0 = blockIdx.x * kTW, y0 = 1 + blockIdx.y * kTY;
  const int nkc = (a.zi1 - a.zi0 + a.tile_z - 1) / a.tile_z;
  const int b = blockIdx.z / nkc, kc = blockIdx.z % nkc;
  const int k0 = a.zi0 + kc * a.tile_z, k1 = min(k0 + a.tile_z, a.zi1);
  const int i0 = x0 + 4 * tx, j = y0 + ty;
  const bool live = i0 < a.X && bulk_quad(a, i0, j);
  const int X = a.X, Y = a.Y;
  const long long base = (long long)b * a.bs;
  const Q4<real> idx4 = i0 < X ? lds4(a.idd[0] + i0) : Q4<real>{};
  const real idy = a.idd[1][min(j, Y - 1)];
  // H at plane k0 - 1 (the carried x and y components)
  Q4<real> hx_m{}, hy_m{};
  if (live) {
    const long long p = base + (long long)(k0 - 1) * X * Y + (long long)j * X + i0;
    hx_m = lds4(a.H[0] + p);
    hy_m = lds4(a.H[1] + p);
  }
#pragma unroll
  for (int s = 0; s < kStages; ++s) {
    e_stage(a, slot[s], b, k0 + s, k1, x0, y0);
    cp_commit();
  }
  for (int k = k0; k < k1; ++k) {
    cp_wait<kStages - 1>();
    __syncthreads();
    const ESlot<real>& cur = slot[(k - k0) % kStages];
    if (live) {
      const long long q = (long long)k * X * Y + (long long)j * X + i0;
      const real idz = a.idd[2][k];
      const Q4<real> hx = lds4(&cur.h[0][ty + 1][4 * tx + 4]), hy = lds4(&cur.h[1][ty + 1][4 * tx + 4]);
      const Q4<real> hz = lds4(&cur.h[2][ty + 1][4 * tx + 4]);
      const Q4<real> hzy = lds4(&cur.h[2][ty][4 * tx + 4]), hxy = lds4(&cur.h[0][ty][4 * tx + 4]);
      const real hz_l = cur.h[2][ty + 1][4 * tx + 3], hy_l = cur.h[1][ty + 1][4 * tx + 3];
      real d0[4], d1[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        d0[e] = (hz.v[e] - hzy.v[e]) * idy;
        d1[e] = (hy.v[e] - hy_m.v[e]) * idz;
      }
      e_apply(a, 0, a.E[0] + base, q, lds4(&cur.e[0][ty][4 * tx]), &cur.m[0][ty][4 * tx], d0, d1, true, i0, j, k, b);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const real hzl = e > 0 ? hz.v[e - 1] : hz_l;
        d0[e] = (hz.v[e] - hzl) * idx4.v[e];
        d1[e] = (hx.v[e] - hx_m.v[e]) * idz;
      }
      e_apply(a, 1, a.E[1] + base, q, lds4(&cur.e[1][ty][4 * tx]), &cur.m[1][ty][4 * tx], d0, d1, false, i0, j, k, b);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const real hyl = e > 0 ? hy.v[e - 1] : hy_l;
        d0[e] = (hy.v[e] - hyl) * idx4.v[e];
        d1[e] = (hx.v[e] - hxy.v[e]) * idy;
      }
      e_apply(a, 2, a.E[2] + base, q, lds4(&cur.e[2][ty][4 * tx]), &cur.m[2][ty][4 * tx], d0, d1, true, i0, j, k, b);
      hx_m = hx;
      hy_m = hy;
    }
    __syncthreads();
    e_stage(a, slot[(k - k0) % kStages], b, k + kStages, k1, x0, y0);
    cp_commit();
  }
  cp_wait<0>();
}

template <typename real>
size_t h_staged_smem() {
  return sizeof(HSlot<real>) * kStages;
}
template <typename real>
size_t e_staged_smem() {
  return sizeof(ESlot<real>) * kStages;
}

template <typename real>
cudaError_t launch_staged_bulk(const SweepArgs<real>& a, cudaStream_t s, bool h) {
  const int inner = a.zi1 - a.zi0;
  if (inner <= 0) return cudaSuccess;
  const int nkc = (inner + a.tile_z - 1) / a.tile_z;
  dim3 block(kTQ, kTY);
  dim3 grid((a.X + kTW - 1) / kTW, (a.ny + 1 + kTY - 1) / kTY, nkc * a.B);
  if (h) {
    const size_t bytes = h_staged_smem<real>();
    cudaError_t err = cudaFuncSetAttribute(h_staged_kernel<real>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (err != cudaSuccess) return err;
    h_staged_kernel<real><<<grid, block, bytes, s>>>(a);
  } else {
    const size_t bytes = e_staged_smem<real>();
    cudaError_t err = cudaFuncSetAttribute(e_staged_kernel<real>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (err != cudaSuccess) return err;
    e_staged_kernel<real><<<grid, block, bytes, s>>>(a);
  }
  return cudaGetLastError();
}

template cudaError_t launch_staged_bulk<float>(const SweepArgs<float>&, cudaStream_t, bool);
template cudaError_t launch_staged_bulk<double>(const SweepArgs<double>&, cudaStream_t, bool);

}  // namespace oafdtd
