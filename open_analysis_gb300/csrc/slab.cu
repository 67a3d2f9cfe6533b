// The slab kernel: everything outside the interior box of a sweep.
//
// The update domain of each sweep is split into an interior box, which holds no CPML correction
// cell and is swept by the staged kernels (staged.cu), and up to six disjoint boxes around it:
// the z slabs (whole planes), then the y slabs and the x slabs of the remaining planes. This
// kernel marches those boxes. With the staged sweeps off (variant 0) its one box is the whole
// domain.
//
// Each thread owns a "quad" (four consecutive x cells of one storage row) and marches a chunk of
// z planes, carrying the neighbouring plane in registers. For every cell it does, in the
// reference's order (packages/oa-fdtd/src/oa_fdtd/reference.py:152-207, :115-127):
//   1. the bulk update (E: ca E + cb curl H; H: H + dt/mu0 curl E);
//   2. the CPML corrections of the component in ascending derivative axis, each
//      psi <- b psi + c d; F <- F + (sign k)(ek d + psi), with d the derivative the bulk update
//      used and k = cb of the edge (E) or dt/mu0 (H);
//   3. (E) the Debye update of dispersive edges: jt = 1/2 sum_p (1 + k_p) J_p;
//      E^{n+1} = E - cbe jt; J_p = k_p J_p + beta_p (E^{n+1} - E^n). Dispersive edges that take an
//      injection keep it for the edge pass, after the surface impedance and the injection.
// The library is compiled without FMA contraction, so each product and sum rounds as in NumPy.
//
// psi layout, one array per (kind, component, axis, side): (B, Z', Y', X') with the slab width
// on the derivative axis and the full storage extent on the other two.

#include "device_common.cuh"

namespace oafdtd {

constexpr int kSlabThreads = 256;

// Launch geometry: the boxes of one kind with their first block.
struct SlabLaunch {
  Span3 box[6];
  int n;
  int first[7];  // first block of each box; first[n] = total blocks
  int cblk[6];   // column blocks per (box, chunk, member)
  int nch[6];    // z chunks per box
};

template <typename real>
__device__ __forceinline__ long long psi_index(const CpmlSide<real>& s, int ax, int b, int k, int j, int i, int X,
                                               int Y, int Z) {
  if (ax == 0) {
    const int w = s.hi[0] - s.lo[0];
    return (((long long)b * Z + k) * Y + j) * w + (i - s.lo[0]);
  }
  if (ax == 1) {
    const int w = s.hi[1] - s.lo[1];
    return (((long long)b * Z + k) * w + (j - s.lo[1])) * X + i;
  }
  const int w = s.hi[2] - s.lo[2];
  return (((long long)b * w + (k - s.lo[2])) * Y + j) * X + i;
}

// The CPML corrections of one component on one quad, both derivative axes in ascending order.
// d[t] holds the derivative along term t's axis; kf the coefficient k per cell.
template <typename real>
__device__ __forceinline__ void correct(const CpmlTerm<real> (&T)[2], const real* const (&co)[3][3], Quad<real>& f,
                                        const real (&d0)[4], const real (&d1)[4], const real (&kf)[4], int b,
                                        int k, int j, int i0, int X, int Y, int Z) {
#pragma unroll
  for (int t = 0; t < 2; ++t) {
    const CpmlTerm<real>& term = T[t];
#pragma unroll
    for (int sd = 0; sd < 2; ++sd) {
      const CpmlSide<real>& s = term.side[sd];
      if (s.psi == nullptr) continue;
      if (j < s.lo[1] || j >= s.hi[1] || k < s.lo[2] || k >= s.hi[2] || i0 + 3 < s.lo[0] || i0 >= s.hi[0]) continue;
      const int ax = term.axis;
      const real* __restrict__ cb_ = co[ax][0];
      const real* __restrict__ cc_ = co[ax][1];
      const real* __restrict__ ck_ = co[ax][2];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int i = i0 + e;
        if (i < s.lo[0] || i >= s.hi[0]) continue;
        const int ia = ax == 0 ? i : (ax == 1 ? j : k);
        const long long pq = psi_index(s, ax, b, k, j, i, X, Y, Z);
        const real d = t == 0 ? d0[e] : d1[e];
        real ps = s.psi[pq];
        ps = ps * cb_[ia];
        ps = ps + cc_[ia] * d;
        s.psi[pq] = ps;
        const real upd = ck_[ia] * d + ps;
        f.v[e] = f.v[e] + (term.sign * kf[e]) * upd;
      }
    }
  }
}

// Where a thread works: member, box, quad column and plane range.
struct SlabWork {
  int b, j, i0, k0, k1;
  bool live;
};

__device__ __forceinline__ SlabWork slab_work(const SlabLaunch& L, int tile_z, int nx) {
  int s = 0;
  while (s + 1 < L.n && (int)blockIdx.x >= L.first[s + 1]) ++s;
  const Span3 bx = L.box[s];
  int r = (int)blockIdx.x - L.first[s];
  const int cb = r % L.cblk[s];
  r /= L.cblk[s];
  const int ch = r % L.nch[s];
  SlabWork w;
  w.b = r / L.nch[s];
  const int nq = bx.q1 - bx.q0;
  const int col = cb * kSlabThreads + (int)threadIdx.x;
  const int ncol = nq * (bx.j1 - bx.j0);
  const int c = min(col, ncol - 1);
  w.j = bx.j0 + c / nq;
  w.i0 = 4 * (bx.q0 + c % nq);
  w.k0 = bx.k0 + ch * tile_z;
  w.k1 = min(w.k0 + tile_z, bx.k1);
  w.live = col < ncol && w.i0 <= nx + 1;
  return w;
}

// ------------------------------------------------------------------------------------- E
template <typename real>
__device__ __forceinline__ void e_cell_quad(const SweepArgs<real>& a, int c, long long p, const Quad<uint16_t>& m, const real (&d0)[4], const real (&d1)[4],
                                            bool first_plus, int i0, int j, int k, int b) {
  const int X = a.X, Y = a.Y, Z = a.nz + 2, nx = a.nx;
  real* __restrict__ E = a.E[c];
  Quad<real> e4 = ld4(E + p);
  const Quad<real> e0 = e4;
  Coef<real> cf[4];
  real kf[4];
  bool valid[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int i = i0 + e;
    cf[e] = a.coef[m.v[e]];
    kf[e] = cf[e].cb;
    valid[e] = i >= 1 && i <= nx + 1;
    const real acc = first_plus ? d0[e] + (-d1[e]) : d1[e] + (-d0[e]);
    if (valid[e]) e4.v[e] = cf[e].ca * e4.v[e] + cf[e].cb * acc;
  }
  if (a.has_cpml) correct<real>(a.ecorr[c], a.pe, e4, d0, d1, kf, b, k, j, i0, X, Y, Z);
  bool disp = false;
#pragma unroll
  for (int e = 0; e < 4; ++e) disp |= valid[e] && m.v[e] >= a.ade_lo && m.v[e] < a.ade_hi;
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
__global__ void __launch_bounds__(kSlabThreads, 2)
    slab_e_kernel(const __grid_constant__ SweepArgs<real> a, const __grid_constant__ SlabLaunch L) {
  const SlabWork w = slab_work(L, a.tile_z, a.nx);
  if (!w.live || w.k0 >= w.k1) return;
  const int X = a.X, Y = a.Y, b = w.b, j = w.j, i0 = w.i0;
  const long long sz = (long long)X * Y;
  const long long base = (long long)b * a.bs;
  const real* __restrict__ Hx = a.H[0] + base;
  const real* __restrict__ Hy = a.H[1] + base;
  const real* __restrict__ Hz = a.H[2] + base;
  const Quad<real> idx4 = ld4(a.idd[0] + i0);
  const real idy = a.idd[1][j];
  long long q = (long long)w.k0 * sz + (long long)j * X + i0;  // offset within one member
  Quad<real> hx_m = ld4(Hx + q - sz), hy_m = ld4(Hy + q - sz);
  for (int k = w.k0; k < w.k1; ++k, q += sz) {
    const real idz = a.idd[2][k];
    const Quad<real> hx = ld4(Hx + q), hy = ld4(Hy + q), hz = ld4(Hz + q);
    const Quad<real> hzy = ld4(Hz + q - X), hxy = ld4(Hx + q - X);
    const real hz_l = Hz[q - 1], hy_l = Hy[q - 1];
    const Quad<uint16_t> m0 = ld4(a.mat[0] + q), m1 = ld4(a.mat[1] + q), m2 = ld4(a.mat[2] + q);
    real d0[4], d1[4];
    // Ex: terms (a = y, +Hz) then (a = z, -Hy)
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      d0[e] = (hz.v[e] - hzy.v[e]) * idy;
      d1[e] = (hy.v[e] - hy_m.v[e]) * idz;
    }
    e_cell_quad<real>(a, 0, base + q, m0, d0, d1, true, i0, j, k, b);
    // Ey: terms (a = z, +Hx) then (a = x, -Hz); d0 is the x term, d1 the z term
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const real hzl = e > 0 ? hz.v[e - 1] : hz_l;
      d0[e] = (hz.v[e] - hzl) * idx4.v[e];
      d1[e] = (hx.v[e] - hx_m.v[e]) * idz;
    }
    e_cell_quad<real>(a, 1, base + q, m1, d0, d1, false, i0, j, k, b);
    // Ez: terms (a = x, +Hy) then (a = y, -Hx)
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const real hyl = e > 0 ? hy.v[e - 1] : hy_l;
      d0[e] = (hy.v[e] - hyl) * idx4.v[e];
      d1[e] = (hx.v[e] - hxy.v[e]) * idy;
    }
    e_cell_quad<real>(a, 2, base + q, m2, d0, d1, true, i0, j, k, b);
    hx_m = hx;
    hy_m = hy;
  }
}

// ------------------------------------------------------------------------------------- H
template <typename real>
__device__ __forceinline__ void h_cell_quad(const SweepArgs<real>& a, int c, long long p, const real (&d0)[4],
                                            const real (&d1)[4], const real (&acc)[4], int ilast, int i0, int j,
                                            int k, int b) {
  real* __restrict__ H = a.H[c];
  Quad<real> h = ld4(H + p);
  const real dtmu = a.dtmu;
  real kf[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int i = i0 + e;
    kf[e] = dtmu;
    if (i >= 1 && i <= ilast) h.v[e] = h.v[e] + dtmu * acc[e];
  }
  if (a.has_cpml) correct<real>(a.hcorr[c], a.ph, h, d0, d1, kf, b, k, j, i0, a.X, a.Y, a.nz + 2);
  st4(H + p, h);
}

template <typename real>
__global__ void __launch_bounds__(kSlabThreads, 2)
    slab_h_kernel(const __grid_constant__ SweepArgs<real> a, const __grid_constant__ SlabLaunch L) {
  const SlabWork w = slab_work(L, a.tile_z, a.nx);
  if (!w.live || w.k0 >= w.k1) return;
  const int X = a.X, Y = a.Y, nx = a.nx, ny = a.ny, nz = a.nz, b = w.b, j = w.j, i0 = w.i0;
  const long long sz = (long long)X * Y;
  const long long base = (long long)b * a.bs;
  const real* __restrict__ Ex = a.E[0] + base;
  const real* __restrict__ Ey = a.E[1] + base;
  const real* __restrict__ Ez = a.E[2] + base;
  const Quad<real> ipx = ld4(a.ip[0] + i0);
  const real ipy = a.ip[1][j];
  const bool right = i0 + 4 < X;  // the x + 1 neighbour of element 3 is in the row
  long long q = (long long)w.k0 * sz + (long long)j * X + i0;
  Quad<real> ex = ld4(Ex + q), ey = ld4(Ey + q);
  for (int k = w.k0; k < w.k1; ++k, q += sz) {
    const bool kin = k <= nz;
    const real ipz = a.ip[2][k];
    Quad<real> ex1 = zero4<real>(), ey1 = zero4<real>();
    if (kin) {
      ex1 = ld4(Ex + q + sz);
      ey1 = ld4(Ey + q + sz);
    }
    const Quad<real> ez = ld4(Ez + q);
    const real ez_r = right ? Ez[q + 4] : (real)0, ey_r = right ? Ey[q + 4] : (real)0;
    real d0[4], d1[4], acc[4];
    if (j <= ny && kin) {  // Hx: node along x (1..nx+1), cell along y and z
      const Quad<real> ezy = ld4(Ez + q + X);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        d0[e] = (ezy.v[e] - ez.v[e]) * ipy;  // axis y
        d1[e] = (ey1.v[e] - ey.v[e]) * ipz;  // axis z
        acc[e] = (-d0[e]) + d1[e];
      }
      h_cell_quad<real>(a, 0, base + q, d0, d1, acc, nx + 1, i0, j, k, b);
    }
    if (kin) {  // Hy: cell along x (1..nx), node along y (1..ny+1), cell along z
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const real ezr = e < 3 ? ez.v[e + 1] : ez_r;
        d0[e] = (ezr - ez.v[e]) * ipx.v[e];  // axis x
        d1[e] = (ex1.v[e] - ex.v[e]) * ipz;  // axis z
        acc[e] = (-d1[e]) + d0[e];
      }
      h_cell_quad<real>(a, 1, base + q, d0, d1, acc, nx, i0, j, k, b);
    }
    if (j <= ny) {  // Hz: cell along x and y, node along z (1..nz+1)
      const Quad<real> exy = ld4(Ex + q + X);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const real eyr = e < 3 ? ey.v[e + 1] : ey_r;
        d0[e] = (eyr - ey.v[e]) * ipx.v[e];  // axis x
        d1[e] = (exy.v[e] - ex.v[e]) * ipy;  // axis y
        acc[e] = (-d0[e]) + d1[e];
      }
      h_cell_quad<real>(a, 2, base + q, d0, d1, acc, nx, i0, j, k, b);
    }
    ex = ex1;
    ey = ey1;
  }
}

// ------------------------------------------------------------------------------------- launch
template <typename real>
cudaError_t launch_slab(const SweepArgs<real>& a, int kind, cudaStream_t s) {
  SlabLaunch L{};
  L.n = 0;
  long long total = 0;
  for (int n = 0; n < a.n_slab[kind]; ++n) {
    const Span3& bx = a.slab[kind][n];
    const long long cols = (long long)(bx.q1 - bx.q0) * (bx.j1 - bx.j0);
    if (cols <= 0 || bx.k1 <= bx.k0) continue;
    L.box[L.n] = bx;
    L.first[L.n] = (int)total;
    L.cblk[L.n] = (int)((cols + kSlabThreads - 1) / kSlabThreads);
    L.nch[L.n] = (bx.k1 - bx.k0 + a.tile_z - 1) / a.tile_z;
    total += (long long)L.cblk[L.n] * L.nch[L.n] * a.B;
    ++L.n;
  }
  if (L.n == 0) return cudaSuccess;
  if (total > 2147483647LL) return cudaErrorInvalidConfiguration;
  L.first[L.n] = (int)total;
  if (kind == 0)
    slab_e_kernel<real><<<(unsigned)total, kSlabThreads, 0, s>>>(a, L);
  else
    slab_h_kernel<real><<<(unsigned)total, kSlabThreads, 0, s>>>(a, L);
  return cudaGetLastError();
}

template cudaError_t launch_slab<float>(const SweepArgs<float>&, int, cudaStream_t);
template cudaError_t launch_slab<double>(const SweepArgs<double>&, int, cudaStream_t);

}  // namespace oafdtd
