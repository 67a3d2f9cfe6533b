// Register-marching sweeps (the fallback variant; the staged variant in staged.cu is the
// default).
//
// Thread mapping: each thread owns a "quad", four consecutive x cells of one storage row (a
// 16-byte float4 for float32), and marches up a chunk of z planes, carrying the neighbouring
// plane in registers. Quads are numbered over the flattened (y, x/4) plane. The x neighbour in
// the next (H sweep) or previous (E sweep) quad comes from a warp shuffle; a lane at a warp edge
// reads it itself. Every cell gets its bulk update here; the CPML corrections follow in the
// correction passes (cpml.cu). Material coefficients come from a packed table (ca, cb, cbe,
// beta_0) indexed by the 16-bit combined index; entries [ade_lo, ade_hi) are dispersive.
//
// The library is compiled with -fmad=false: every product and sum is rounded separately, as in
// the NumPy reference (packages/oa-fdtd/src/oa_fdtd/reference.py:152-180, :119-127).

#include "device_common.cuh"

namespace oafdtd {

// Where a thread works: its quad and its plane range.
struct Work {
  int t;        // quad index in the flattened (y, x/4) plane
  int j, i0;
  bool live;    // the quad holds real edges
  bool row_end;
  int k0, k1;
};

template <typename real>
__device__ __forceinline__ Work work_of(const SweepArgs<real>& a) {
  const int X = a.X, Y = a.Y, X4 = X >> 2, nx = a.nx, ny = a.ny, nz = a.nz;
  Work w;
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  w.t = min(g, Y * X4 - 1);
  w.j = w.t / X4;
  w.i0 = (w.t - w.j * X4) * 4;
  w.row_end = w.i0 + 4 >= X;
  w.live = g < Y * X4 && w.j >= 1 && w.j <= ny + 1 && w.i0 <= nx + 1;
  w.k0 = 1 + blockIdx.y * a.tile_z;
  w.k1 = min(w.k0 + a.tile_z, nz + 2);
  return w;
}

// ------------------------------------------------------------------------------------- H sweep
template <typename real>
__global__ void __launch_bounds__(256, 4) h_sweep_kernel(const __grid_constant__ SweepArgs<real> a) {
  const Work w = work_of<real>(a);
  const int X = a.X, Y = a.Y, nx = a.nx, ny = a.ny, nz = a.nz;
  const int j = w.j, i0 = w.i0;
  const int b = blockIdx.z;
  const int lane = threadIdx.x & 31;
  const long long bs = a.bs;
  const real* __restrict__ Ex = a.E[0] + b * bs;
  const real* __restrict__ Ey = a.E[1] + b * bs;
  const real* __restrict__ Ez = a.E[2] + b * bs;
  real* __restrict__ Hx = a.H[0] + b * bs;
  real* __restrict__ Hy = a.H[1] + b * bs;
  real* __restrict__ Hz = a.H[2] + b * bs;
  const long long sy1 = j <= ny ? X : 0;  // y + 1 row offset (only used where j <= ny)
  const Quad<real> ipx = ld4(a.ip[0] + i0);
  const real ipy = a.ip[1][j];
  const real dtmu = a.dtmu;
  const long long sz = (long long)X * Y;
  const bool nb_quad = __shfl_down_sync(0xffffffffu, w.t, 1) == w.t + 1 && lane < 31;
  const unsigned who = __ballot_sync(0xffffffffu, w.live);
  const bool nb = nb_quad && ((who >> (lane + 1)) & 1u);
  long long p = (long long)w.k0 * sz + (long long)j * X + i0;
  Quad<real> ex = zero4<real>(), ey = zero4<real>();
  if (w.live && w.k0 < w.k1) {
    ex = ld4(Ex + p);
    ey = ld4(Ey + p);
  }
  for (int k = w.k0; k < w.k1; ++k, p += sz) {
    const bool kin = k <= nz;
    Quad<real> ex1 = zero4<real>(), ey1 = zero4<real>(), ez = zero4<real>();
    if (w.live) {
      if (kin) {
        ex1 = ld4(Ex + p + sz);
        ey1 = ld4(Ey + p + sz);
      }
      ez = ld4(Ez + p);
    }
    // x + 1 neighbours of element 3 (every lane takes part in the shuffles)
    real ez_r = __shfl_down_sync(0xffffffffu, ez.v[0], 1);
    real ey_r = __shfl_down_sync(0xffffffffu, ey.v[0], 1);
    if (!w.live) continue;
    if (!nb && !w.row_end) {
      ez_r = Ez[p + 4];
      ey_r = Ey[p + 4];
    }
    const real ipz = a.ip[2][k];
    if (j <= ny && kin) {  // Hx: node along x (1..nx+1), cell along y and z
      const Quad<real> ezy = ld4(Ez + p + sy1);
      Quad<real> h = ld4(Hx + p);
      real d0[4], d1[4];
      bool valid[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int i = i0 + e;
        valid[e] = i >= 1 && i <= nx + 1;
        d0[e] = (ezy.v[e] - ez.v[e]) * ipy;   // axis y
        d1[e] = (ey1.v[e] - ey.v[e]) * ipz;   // axis z
        const real acc = (-d0[e]) + d1[e];
        if (valid[e]) h.v[e] = h.v[e] + dtmu * acc;
      }
      st4(Hx + p, h);
    }
    if (kin) {  // Hy: cell along x (1..nx), node along y (1..ny+1), cell along z
      Quad<real> h = ld4(Hy + p);
      real d0[4], d1[4];
      bool valid[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int i = i0 + e;
        valid[e] = i >= 1 && i <= nx;
        const real ezr = e < 3 ? ez.v[e + 1] : ez_r;
        d0[e] = (ezr - ez.v[e]) * ipx.v[e];   // axis x
        d1[e] = (ex1.v[e] - ex.v[e]) * ipz;   // axis z
        const real acc = (-d1[e]) + d0[e];
        if (valid[e]) h.v[e] = h.v[e] + dtmu * acc;
      }
      st4(Hy + p, h);
    }
    if (j <= ny) {  // Hz: cell along x and y, node along z (1..nz+1)
      const Quad<real> exy = ld4(Ex + p + sy1);
      Quad<real> h = ld4(Hz + p);
      real d0[4], d1[4];
      bool valid[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int i = i0 + e;
        valid[e] = i >= 1 && i <= nx;
        const real eyr = e < 3 ? ey.v[e + 1] : ey_r;
        d0[e] = (eyr - ey.v[e]) * ipx.v[e];   // axis x
        d1[e] = (exy.v[e] - ex.v[e]) * ipy;   // axis y
        const real acc = (-d0[e]) + d1[e];
        if (valid[e]) h.v[e] = h.v[e] + dtmu * acc;
      }
      st4(Hz + p, h);
    }
    ex = ex1;
    ey = ey1;
  }
}

// ------------------------------------------------------------------------------------- E sweep
// Bulk update and the Debye update of one E component on one quad.
// d0/d1 are the derivatives along the component's two axes in ascending order; the bulk term
// order of the reference is (d0, -d1) when first_plus, else (d1, -d0).
template <typename real>
__device__ __forceinline__ void e_quad(const SweepArgs<real>& a, int c, real* __restrict__ E, long long p,
                                       const Quad<uint16_t>& m, const real (&d0)[4], const real (&d1)[4],
                                       bool first_plus, int i0, int j, int k, int b) {
  const int X = a.X, Y = a.Y, nx = a.nx;
  const Coef<real>* __restrict__ tab = a.coef;
  Quad<real> e4 = ld4(E + p);
  const Quad<real> e0 = e4;
  Coef<real> cf[4];
  real kf[4];
  bool valid[4];
  bool disp = false;
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int i = i0 + e;
    cf[e] = tab[m.v[e]];
    kf[e] = cf[e].cb;
    valid[e] = i >= 1 && i <= nx + 1;
    const real acc = first_plus ? d0[e] + (-d1[e]) : d1[e] + (-d0[e]);
    if (valid[e]) e4.v[e] = cf[e].ca * e4.v[e] + cf[e].cb * acc;
    disp |= valid[e] && m.v[e] >= a.ade_lo && m.v[e] < a.ade_hi;
  }
  if (disp) {
    const long long jstride = (long long)a.B * a.jnk[c] * Y * X;
    const long long jq = (((long long)b * a.jnk[c] + (k - a.jk0[c])) * Y + j) * X + i0;
    real* J = a.J[c];
    if (a.ade_P == 1) {
      Quad<real> j4 = ld4(J + jq);
      const real onekp = a.ade_onekp[0], kp = a.ade_kp[0];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        if (!(valid[e] && m.v[e] >= a.ade_lo && m.v[e] < a.ade_hi)) continue;
        const real jt = (real)0.5 * (onekp * j4.v[e]);
        const real en = e4.v[e] - cf[e].cbe * jt;
        const real de = en - e0.v[e];
        j4.v[e] = kp * j4.v[e] + cf[e].beta0 * de;
        e4.v[e] = en;
      }
      st4(J + jq, j4);
    } else {
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        if (!(valid[e] && m.v[e] >= a.ade_lo && m.v[e] < a.ade_hi)) continue;
        e4.v[e] = ade_cell(e4.v[e], e0.v[e], cf[e].cbe, cf[e].beta0, m.v[e], J, jq + e, jstride, a.ade_kp,
                           a.ade_onekp, a.ade_beta, a.ade_P);
      }
    }
  }
  st4(E + p, e4);
}

template <typename real>
__global__ void __launch_bounds__(256, 3) e_sweep_kernel(const __grid_constant__ SweepArgs<real> a) {
  const Work w = work_of<real>(a);
  const int X = a.X, Y = a.Y;
  const int j = w.j, i0 = w.i0;
  const int b = blockIdx.z;
  const int lane = threadIdx.x & 31;
  const long long bs = a.bs;
  const real* __restrict__ Hx = a.H[0] + b * bs;
  const real* __restrict__ Hy = a.H[1] + b * bs;
  const real* __restrict__ Hz = a.H[2] + b * bs;
  const Quad<real> idx4 = ld4(a.idd[0] + i0);
  const real idy = a.idd[1][j];
  const long long sz = (long long)X * Y;
  const bool nb_quad = __shfl_up_sync(0xffffffffu, w.t, 1) == w.t - 1 && lane > 0;
  const unsigned who = __ballot_sync(0xffffffffu, w.live);
  const bool nb = nb_quad && ((who >> (lane - 1)) & 1u);
  long long p = (long long)w.k0 * sz + (long long)j * X + i0;  // batch-free index of the quad
  Quad<real> hx_m = zero4<real>(), hy_m = zero4<real>();
  if (w.live && w.k0 < w.k1) {
    hx_m = ld4(Hx + p - sz);
    hy_m = ld4(Hy + p - sz);
  }
  for (int k = w.k0; k < w.k1; ++k, p += sz) {
    Quad<real> hx = zero4<real>(), hy = zero4<real>(), hz = zero4<real>();
    if (w.live) {
      hx = ld4(Hx + p);
      hy = ld4(Hy + p);
      hz = ld4(Hz + p);
    }
    // x - 1 neighbours of element 0
    real hz_l = __shfl_up_sync(0xffffffffu, hz.v[3], 1);
    real hy_l = __shfl_up_sync(0xffffffffu, hy.v[3], 1);
    if (!w.live) continue;
    if (!nb && i0 > 0) {
      hz_l = Hz[p - 1];
      hy_l = Hy[p - 1];
    }
    const real idz = a.idd[2][k];
    const Quad<real> hzy = ld4(Hz + p - X), hxy = ld4(Hx + p - X);
    real d0[4], d1[4];
    // Ex: terms (a = y, +Hz) then (a = z, -Hy)
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      d0[e] = (hz.v[e] - hzy.v[e]) * idy;
      d1[e] = (hy.v[e] - hy_m.v[e]) * idz;
    }
    e_quad<real>(a, 0, a.E[0] + b * bs, p, ld4(a.mat[0] + p), d0, d1, true, i0, j, k, b);
    // Ey: terms (a = z, +Hx) then (a = x, -Hz); d0 is the x term, d1 the z term
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const real hzl = e > 0 ? hz.v[e - 1] : hz_l;
      d0[e] = (hz.v[e] - hzl) * idx4.v[e];
      d1[e] = (hx.v[e] - hx_m.v[e]) * idz;
    }
    e_quad<real>(a, 1, a.E[1] + b * bs, p, ld4(a.mat[1] + p), d0, d1, false, i0, j, k, b);
    // Ez: terms (a = x, +Hy) then (a = y, -Hx)
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const real hyl = e > 0 ? hy.v[e - 1] : hy_l;
      d0[e] = (hy.v[e] - hyl) * idx4.v[e];
      d1[e] = (hx.v[e] - hxy.v[e]) * idy;
    }
    e_quad<real>(a, 2, a.E[2] + b * bs, p, ld4(a.mat[2] + p), d0, d1, true, i0, j, k, b);
    hx_m = hx;
    hy_m = hy;
  }
}

// ------------------------------------------------------------------------------------- launchers
template <typename real>
cudaError_t launch_h_sweep(const SweepArgs<real>& a, const SweepMaps& m, cudaStream_t s) {
  if (a.staged) return launch_staged_sweep<real>(a, m, s, true);
  const long long quads = (long long)a.Y * (a.X / 4);
  dim3 grid((unsigned)((quads + 255) / 256), (a.nz + 1 + a.tile_z - 1) / a.tile_z, a.B);
  h_sweep_kernel<real><<<grid, 256, 0, s>>>(a);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_e_sweep(const SweepArgs<real>& a, const SweepMaps& m, cudaStream_t s) {
  if (a.staged) return launch_staged_sweep<real>(a, m, s, false);
  const long long quads = (long long)a.Y * (a.X / 4);
  dim3 grid((unsigned)((quads + 255) / 256), (a.nz + 1 + a.tile_z - 1) / a.tile_z, a.B);
  e_sweep_kernel<real><<<grid, 256, 0, s>>>(a);
  return cudaGetLastError();
}

template cudaError_t launch_h_sweep<float>(const SweepArgs<float>&, const SweepMaps&, cudaStream_t);
template cudaError_t launch_e_sweep<float>(const SweepArgs<float>&, const SweepMaps&, cudaStream_t);
template cudaError_t launch_h_sweep<double>(const SweepArgs<double>&, const SweepMaps&, cudaStream_t);
template cudaError_t launch_e_sweep<double>(const SweepArgs<double>&, const SweepMaps&, cudaStream_t);

}  // namespace oafdtd
