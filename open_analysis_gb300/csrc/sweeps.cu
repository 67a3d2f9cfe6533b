// The two Yee sweeps of a time step, fused with every per-cell correction.
//
// Thread mapping: each thread owns four consecutive x cells of one storage row (a 16-byte
// float4 for float32); the threads of a block cover a contiguous stretch of the flattened
// (y, x/4) plane, and every thread marches up a chunk of z planes, carrying the neighbouring
// plane in registers. The x neighbour in the next (H sweep) or previous (E sweep) thread's quad
// comes from a warp shuffle; a lane whose neighbour lane did not load that plane reads it itself.
//
// Every sweep is two launches over the same grid that split the cells between them:
//  * the bulk launch (SLAB = false) updates the cells outside every CPML slab; it carries no CPML
//    code, so it runs with few registers and high occupancy;
//  * the slab launch (SLAB = true) updates the cells whose quad column or plane meets a slab and
//    applies the corrections cell by cell, in the reference's order (bulk update, then the
//    corrections by ascending derivative axis, each rounded to the field precision).
// Cells are independent within a sweep (H reads only E, E reads only H), so the split changes no
// value. Material coefficients come from a packed table (ca, cb, cbe, beta_0) indexed by the
// 16-bit combined index; entries [ade_lo, ade_hi) are dispersive, so no flag lookup is needed.
//
// The library is compiled with -fmad=false: every product and sum is rounded separately, as in
// the NumPy reference (packages/oa-fdtd/src/oa_fdtd/reference.py:152-207, :119-127).

#include "oafdtd_internal.cuh"

namespace oafdtd {

template <typename real>
struct Quad {
  real v[4];
};

__device__ __forceinline__ Quad<float> ld4(const float* p) {
  const float4 t = *reinterpret_cast<const float4*>(p);
  return Quad<float>{{t.x, t.y, t.z, t.w}};
}
__device__ __forceinline__ Quad<double> ld4(const double* p) {
  const double2 a = reinterpret_cast<const double2*>(p)[0];
  const double2 b = reinterpret_cast<const double2*>(p)[1];
  return Quad<double>{{a.x, a.y, b.x, b.y}};
}
__device__ __forceinline__ void st4(float* p, const Quad<float>& q) {
  *reinterpret_cast<float4*>(p) = make_float4(q.v[0], q.v[1], q.v[2], q.v[3]);
}
__device__ __forceinline__ void st4(double* p, const Quad<double>& q) {
  reinterpret_cast<double2*>(p)[0] = make_double2(q.v[0], q.v[1]);
  reinterpret_cast<double2*>(p)[1] = make_double2(q.v[2], q.v[3]);
}
__device__ __forceinline__ Quad<uint16_t> ld4(const uint16_t* p) {
  const ushort4 t = *reinterpret_cast<const ushort4*>(p);
  return Quad<uint16_t>{{t.x, t.y, t.z, t.w}};
}

template <typename real>
__device__ __forceinline__ Quad<real> zero4() {
  return Quad<real>{{(real)0, (real)0, (real)0, (real)0}};
}

// One CPML correction on one cell: psi <- b psi + c d; f += (sign k) (ek d + psi).
template <typename real>
__device__ __noinline__ void cpml_cell(real& f, const CpmlTerm<real>& t, int i, int j, int k, int b,
                                       real d, real kfac, const real* cb_, const real* cc_,
                                       const real* ck_, int X, int Y, int Z) {
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const CpmlSide<real>& sd = t.side[s];
    if (sd.psi == nullptr) continue;
    if (i < sd.lo[0] || i >= sd.hi[0] || j < sd.lo[1] || j >= sd.hi[1] || k < sd.lo[2] || k >= sd.hi[2])
      continue;
    // psi covers the slab along the derivative axis and the full storage extent on the others
    long long q;
    if (t.axis == 0) {
      const int w = sd.hi[0] - sd.lo[0];
      q = (((long long)b * Z + k) * Y + j) * w + (i - sd.lo[0]);
    } else if (t.axis == 1) {
      const int w = sd.hi[1] - sd.lo[1];
      q = (((long long)b * Z + k) * w + (j - sd.lo[1])) * X + i;
    } else {
      const int w = sd.hi[2] - sd.lo[2];
      q = (((long long)b * w + (k - sd.lo[2])) * Y + j) * X + i;
    }
    const int ia = t.axis == 0 ? i : (t.axis == 1 ? j : k);
    real ps = sd.psi[q];
    ps = ps * cb_[ia];
    ps = ps + cc_[ia] * d;
    sd.psi[q] = ps;
    const real upd = ck_[ia] * d + ps;
    f = f + (t.sign * kfac) * upd;
  }
}

// Debye update of one dispersive edge with any pole count: jt = 1/2 sum_p (1 + k_p) J_p;
// E^{n+1} = e - cbe jt; J_p = k_p J_p + beta_p (E^{n+1} - E^n).
template <typename real>
__device__ __noinline__ real ade_cell(real e, real e0, real cbe, real beta0, int m, real* J, long long jq,
                                      long long jstride, const real* kp, const real* onekp,
                                      const real* beta, int P) {
  real jt = (real)0;
  for (int p = 0; p < P; ++p) jt = jt + onekp[p] * J[jq + p * jstride];
  jt = (real)0.5 * jt;
  const real en = e - cbe * jt;
  const real de = en - e0;
  for (int p = 0; p < P; ++p) {
    const long long q = jq + p * jstride;
    const real bp = p == 0 ? beta0 : beta[(long long)m * P + p];
    J[q] = kp[p] * J[q] + bp * de;
  }
  return en;
}

struct QuadPos {
  int j, i0;
  bool live, row_end;
};

__device__ __forceinline__ QuadPos quad_pos(int X, int Y, int nx, int ny) {
  const int X4 = X >> 2;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int tt = min(t, Y * X4 - 1);
  QuadPos q;
  q.j = tt / X4;
  q.i0 = (tt - q.j * X4) * 4;
  q.live = t < Y * X4 && q.j >= 1 && q.j <= ny + 1 && q.i0 <= nx + 1;
  q.row_end = q.i0 + 4 >= X;
  return q;
}

template <typename real>
__device__ __forceinline__ bool column_in_slab(const SweepArgs<real>& a, const QuadPos& q) {
  if (!a.has_cpml) return false;
  bool s = a.slab_y[q.j] != 0;
#pragma unroll
  for (int e = 0; e < 4; ++e) s |= a.slab_x[q.i0 + e] != 0;
  return s;
}

// ------------------------------------------------------------------------------------- H sweep
// Minimum resident blocks per SM of the bulk launches: caps their registers so that enough warps
// are resident to keep HBM busy; the slab launches are left unconstrained.
template <typename real, bool SLAB>
struct Occupancy {
  static constexpr int h = SLAB ? 1 : 4;
  static constexpr int e = SLAB ? 1 : 3;
};

template <typename real, bool SLAB>
__global__ void __launch_bounds__(256, Occupancy<real, SLAB>::h) h_sweep_kernel(const __grid_constant__ SweepArgs<real> a) {
  const int X = a.X, Y = a.Y, Z = a.nz + 2;
  const int nx = a.nx, ny = a.ny, nz = a.nz;
  const QuadPos qp = quad_pos(X, Y, nx, ny);
  const int j = qp.j, i0 = qp.i0;
  const int b = blockIdx.z;
  const int lane = threadIdx.x & 31;
  const int k0 = 1 + blockIdx.y * a.tile_z;
  const int k1 = min(k0 + a.tile_z, nz + 2);
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
  const bool col = column_in_slab(a, qp);
  const long long sz = (long long)X * Y;
  long long p = (long long)k0 * sz + (long long)j * X + i0;
  Quad<real> ex = zero4<real>(), ey = zero4<real>();
  bool carried = false;
  for (int k = k0; k < k1; ++k, p += sz) {
    const bool in_slab = col || (a.has_cpml && a.slab_z[k] != 0);
    const bool proc = qp.live && (in_slab == SLAB);
    const unsigned who = __ballot_sync(0xffffffffu, proc);
    const bool kin = k <= nz;
    Quad<real> ex1 = zero4<real>(), ey1 = zero4<real>(), ez = zero4<real>();
    if (proc) {
      if (!carried) {
        ex = ld4(Ex + p);
        ey = ld4(Ey + p);
      }
      if (kin) {
        ex1 = ld4(Ex + p + sz);
        ey1 = ld4(Ey + p + sz);
      }
      ez = ld4(Ez + p);
    }
    // x + 1 neighbours of element 3 (every lane takes part in the shuffles)
    real ez_r = __shfl_down_sync(0xffffffffu, ez.v[0], 1);
    real ey_r = __shfl_down_sync(0xffffffffu, ey.v[0], 1);
    if (!proc) {
      carried = false;
      continue;
    }
    const bool nb = lane < 31 && ((who >> (lane + 1)) & 1u);
    if (!nb && !qp.row_end) {
      ez_r = Ez[p + 4];
      ey_r = Ey[p + 4];
    }
    const real ipz = a.ip[2][k];
    if (j <= ny && kin) {  // Hx: node along x (1..nx+1), cell along y and z
      const Quad<real> ezy = ld4(Ez + p + sy1);
      Quad<real> h = ld4(Hx + p);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int i = i0 + e;
        if (i < 1 || i > nx + 1) continue;
        const real dy = (ezy.v[e] - ez.v[e]) * ipy;
        const real dz = (ey1.v[e] - ey.v[e]) * ipz;
        const real acc = (-dy) + dz;
        real hv = h.v[e] + dtmu * acc;
        if (SLAB) {
          cpml_cell(hv, a.hcorr[0][0], i, j, k, b, dy, dtmu, a.ph[1][0], a.ph[1][1], a.ph[1][2], X, Y, Z);
          cpml_cell(hv, a.hcorr[0][1], i, j, k, b, dz, dtmu, a.ph[2][0], a.ph[2][1], a.ph[2][2], X, Y, Z);
        }
        h.v[e] = hv;
      }
      st4(Hx + p, h);
    }
    if (kin) {  // Hy: cell along x (1..nx), node along y (1..ny+1), cell along z
      Quad<real> h = ld4(Hy + p);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int i = i0 + e;
        if (i < 1 || i > nx) continue;
        const real ezr = e < 3 ? ez.v[e + 1] : ez_r;
        const real dz = (ex1.v[e] - ex.v[e]) * ipz;
        const real dx = (ezr - ez.v[e]) * ipx.v[e];
        const real acc = (-dz) + dx;
        real hv = h.v[e] + dtmu * acc;
        if (SLAB) {
          cpml_cell(hv, a.hcorr[1][0], i, j, k, b, dx, dtmu, a.ph[0][0], a.ph[0][1], a.ph[0][2], X, Y, Z);
          cpml_cell(hv, a.hcorr[1][1], i, j, k, b, dz, dtmu, a.ph[2][0], a.ph[2][1], a.ph[2][2], X, Y, Z);
        }
        h.v[e] = hv;
      }
      st4(Hy + p, h);
    }
    if (j <= ny) {  // Hz: cell along x and y, node along z (1..nz+1)
      const Quad<real> exy = ld4(Ex + p + sy1);
      Quad<real> h = ld4(Hz + p);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int i = i0 + e;
        if (i < 1 || i > nx) continue;
        const real eyr = e < 3 ? ey.v[e + 1] : ey_r;
        const real dx = (eyr - ey.v[e]) * ipx.v[e];
        const real dy = (exy.v[e] - ex.v[e]) * ipy;
        const real acc = (-dx) + dy;
        real hv = h.v[e] + dtmu * acc;
        if (SLAB) {
          cpml_cell(hv, a.hcorr[2][0], i, j, k, b, dx, dtmu, a.ph[0][0], a.ph[0][1], a.ph[0][2], X, Y, Z);
          cpml_cell(hv, a.hcorr[2][1], i, j, k, b, dy, dtmu, a.ph[1][0], a.ph[1][1], a.ph[1][2], X, Y, Z);
        }
        h.v[e] = hv;
      }
      st4(Hz + p, h);
    }
    ex = ex1;
    ey = ey1;
    carried = kin;
  }
}

// ------------------------------------------------------------------------------------- E sweep
// Bulk update, CPML (slab launch) and the Debye update of one E component on one quad.
template <typename real, bool SLAB>
__device__ __forceinline__ void e_quad(const SweepArgs<real>& a, int c, real* __restrict__ E, long long p,
                                       const Quad<uint16_t>& m, const real (&d0)[4], const real (&d1)[4],
                                       bool first_plus, int i0, int j, int k, int b) {
  const int X = a.X, Y = a.Y, Z = a.nz + 2, nx = a.nx;
  const Coef<real>* __restrict__ tab = a.coef;
  Quad<real> e4 = ld4(E + p);
  const Quad<real> e0 = e4;
  Coef<real> cf[4];
  bool disp = false;
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int i = i0 + e;
    cf[e] = tab[m.v[e]];
    if (i < 1 || i > nx + 1) continue;
    // acc = d0 + (-d1) with the terms in the reference's table order for this component
    const real acc = first_plus ? d0[e] + (-d1[e]) : d1[e] + (-d0[e]);
    real ev = cf[e].ca * e4.v[e] + cf[e].cb * acc;
    if (SLAB) {
      const CpmlTerm<real>& t0 = a.ecorr[c][0];
      const CpmlTerm<real>& t1 = a.ecorr[c][1];
      cpml_cell(ev, t0, i, j, k, b, d0[e], cf[e].cb, a.pe[t0.axis][0], a.pe[t0.axis][1], a.pe[t0.axis][2], X,
                Y, Z);
      cpml_cell(ev, t1, i, j, k, b, d1[e], cf[e].cb, a.pe[t1.axis][0], a.pe[t1.axis][1], a.pe[t1.axis][2], X,
                Y, Z);
    }
    e4.v[e] = ev;
    disp |= m.v[e] >= a.ade_lo && m.v[e] < a.ade_hi;
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
        if (!(m.v[e] >= a.ade_lo && m.v[e] < a.ade_hi)) continue;
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
        if (!(m.v[e] >= a.ade_lo && m.v[e] < a.ade_hi)) continue;
        e4.v[e] = ade_cell(e4.v[e], e0.v[e], cf[e].cbe, cf[e].beta0, m.v[e], J, jq + e, jstride, a.ade_kp,
                           a.ade_onekp, a.ade_beta, a.ade_P);
      }
    }
  }
  st4(E + p, e4);
}

template <typename real, bool SLAB>
__global__ void __launch_bounds__(256, Occupancy<real, SLAB>::e) e_sweep_kernel(const __grid_constant__ SweepArgs<real> a) {
  const int X = a.X, Y = a.Y;
  const int nx = a.nx, ny = a.ny, nz = a.nz;
  const QuadPos qp = quad_pos(X, Y, nx, ny);
  const int j = qp.j, i0 = qp.i0;
  const int b = blockIdx.z;
  const int lane = threadIdx.x & 31;
  const int k0 = 1 + blockIdx.y * a.tile_z;
  const int k1 = min(k0 + a.tile_z, nz + 2);
  const long long bs = a.bs;
  const real* __restrict__ Hx = a.H[0] + b * bs;
  const real* __restrict__ Hy = a.H[1] + b * bs;
  const real* __restrict__ Hz = a.H[2] + b * bs;
  const Quad<real> idx4 = ld4(a.idd[0] + i0);
  const real idy = a.idd[1][j];
  const bool col = column_in_slab(a, qp);
  const long long sz = (long long)X * Y;
  long long p = (long long)k0 * sz + (long long)j * X + i0;  // batch-free index of the quad
  Quad<real> hx_m = zero4<real>(), hy_m = zero4<real>();
  bool carried = false;
  for (int k = k0; k < k1; ++k, p += sz) {
    const bool in_slab = col || (a.has_cpml && a.slab_z[k] != 0);
    const bool proc = qp.live && (in_slab == SLAB);
    const unsigned who = __ballot_sync(0xffffffffu, proc);
    Quad<real> hx = zero4<real>(), hy = zero4<real>(), hz = zero4<real>();
    if (proc) {
      if (!carried) {
        hx_m = ld4(Hx + p - sz);
        hy_m = ld4(Hy + p - sz);
      }
      hx = ld4(Hx + p);
      hy = ld4(Hy + p);
      hz = ld4(Hz + p);
    }
    // x - 1 neighbours of element 0
    real hz_l = __shfl_up_sync(0xffffffffu, hz.v[3], 1);
    real hy_l = __shfl_up_sync(0xffffffffu, hy.v[3], 1);
    if (!proc) {
      carried = false;
      continue;
    }
    const bool nb = lane > 0 && ((who >> (lane - 1)) & 1u);
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
    e_quad<real, SLAB>(a, 0, a.E[0] + b * bs, p, ld4(a.mat[0] + p), d0, d1, true, i0, j, k, b);
    // Ey: terms (a = z, +Hx) then (a = x, -Hz); ascending axes: d0 = x term, d1 = z term
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const real hzl = e > 0 ? hz.v[e - 1] : hz_l;
      d0[e] = (hz.v[e] - hzl) * idx4.v[e];
      d1[e] = (hx.v[e] - hx_m.v[e]) * idz;
    }
    e_quad<real, SLAB>(a, 1, a.E[1] + b * bs, p, ld4(a.mat[1] + p), d0, d1, false, i0, j, k, b);
    // Ez: terms (a = x, +Hy) then (a = y, -Hx)
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const real hyl = e > 0 ? hy.v[e - 1] : hy_l;
      d0[e] = (hy.v[e] - hyl) * idx4.v[e];
      d1[e] = (hx.v[e] - hxy.v[e]) * idy;
    }
    e_quad<real, SLAB>(a, 2, a.E[2] + b * bs, p, ld4(a.mat[2] + p), d0, d1, true, i0, j, k, b);
    hx_m = hx;
    hy_m = hy;
    carried = true;
  }
}

// ------------------------------------------------------------------------------------- launchers
template <typename real>
cudaError_t launch_h_sweep(const SweepArgs<real>& a, int tile_y, cudaStream_t s) {
  (void)tile_y;
  const int nkc = (a.nz + 1 + a.tile_z - 1) / a.tile_z;
  const long long quads = (long long)a.Y * (a.X / 4);
  dim3 grid((unsigned)((quads + 255) / 256), nkc, a.B);
  h_sweep_kernel<real, false><<<grid, 256, 0, s>>>(a);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess || !a.has_cpml) return err;
  h_sweep_kernel<real, true><<<grid, 256, 0, s>>>(a);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_e_sweep(const SweepArgs<real>& a, int tile_y, cudaStream_t s) {
  (void)tile_y;
  const int nkc = (a.nz + 1 + a.tile_z - 1) / a.tile_z;
  const long long quads = (long long)a.Y * (a.X / 4);
  dim3 grid((unsigned)((quads + 255) / 256), nkc, a.B);
  e_sweep_kernel<real, false><<<grid, 256, 0, s>>>(a);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess || !a.has_cpml) return err;
  e_sweep_kernel<real, true><<<grid, 256, 0, s>>>(a);
  return cudaGetLastError();
}

template cudaError_t launch_h_sweep<float>(const SweepArgs<float>&, int, cudaStream_t);
template cudaError_t launch_e_sweep<float>(const SweepArgs<float>&, int, cudaStream_t);
template cudaError_t launch_h_sweep<double>(const SweepArgs<double>&, int, cudaStream_t);
template cudaError_t launch_e_sweep<double>(const SweepArgs<double>&, int, cudaStream_t);

}  // namespace oafdtd
