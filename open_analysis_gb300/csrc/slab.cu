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
// Planes marched per thread. The slab boxes are thin (CPML slabs of ~10 cells): short marches
// give the kernel enough independent threads to hide its load latency.
constexpr int kSlabPlanes = 4;

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

// psi of one correction term on one quad: the side whose box holds the quad's row (-1: none) and
// the values. y and z slabs keep psi rows at the field pitch, so their quads are whole 16-byte
// vectors (elements outside the box are written back unchanged); x slabs are read per element.
template <typename real>
struct PsiQuad {
  Quad<real> v;
  int sd;
};

template <typename real>
__device__ __forceinline__ const CpmlSide<real>& side_of(const CpmlTerm<real>& T, int sd) {
  return sd == 0 ? T.side[0] : T.side[1];
}

template <typename real>
__device__ __forceinline__ void psi_load(const CpmlTerm<real>& T, PsiQuad<real>& P, int b, int k, int j, int i0,
                                         int X, int Y, int Z) {
  P.sd = -1;
#pragma unroll
  for (int sd = 0; sd < 2; ++sd) {
    const CpmlSide<real>& s = T.side[sd];
    if (P.sd >= 0 || s.psi == nullptr) continue;
    if (j < s.lo[1] || j >= s.hi[1] || k < s.lo[2] || k >= s.hi[2] || i0 + 3 < s.lo[0] || i0 >= s.hi[0]) continue;
    P.sd = sd;
    if (T.axis == 0) {
      const long long pq = psi_index(s, 0, b, k, j, i0, X, Y, Z);
#pragma unroll
      for (int e = 0; e < 4; ++e)
        P.v.v[e] = (i0 + e >= s.lo[0] && i0 + e < s.hi[0]) ? s.psi[pq + e] : (real)0;
    } else {
      P.v = ld4(s.psi + psi_index(s, T.axis, b, k, j, i0, X, Y, Z));
    }
  }
}

template <typename real>
__device__ __forceinline__ void psi_store(const CpmlTerm<real>& T, const PsiQuad<real>& P, int b, int k, int j,
                                          int i0, int X, int Y, int Z) {
  if (P.sd < 0) return;
  const CpmlSide<real>& s = side_of(T, P.sd);
  const long long pq = psi_index(s, T.axis, b, k, j, i0, X, Y, Z);
  if (T.axis == 0) {
#pragma unroll
    for (int e = 0; e < 4; ++e)
      if (i0 + e >= s.lo[0] && i0 + e < s.hi[0]) s.psi[pq + e] = P.v.v[e];
  } else {
    st4(s.psi + pq, P.v);
  }
}

// One correction on a quad: psi <- b psi + c d; F <- F + (sign k)(ek d + psi) for the cells of
// the box. The coefficient arrays are read-only for the whole run.
template <typename real>
__device__ __forceinline__ void psi_apply(const CpmlTerm<real>& T, PsiQuad<real>& P, const real* const (&co)[3][3],
                                          Quad<real>& f, const real (&d)[4], const real (&kf)[4], int k, int j,
                                          int i0) {
  if (P.sd < 0) return;
  const CpmlSide<real>& s = side_of(T, P.sd);
  const int ax = T.axis;
  const real* cb_ = co[ax][0];
  const real* cc_ = co[ax][1];
  const real* ck_ = co[ax][2];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int i = i0 + e;
    if (i < s.lo[0] || i >= s.hi[0]) continue;
    const int ia = ax == 0 ? i : (ax == 1 ? j : k);
    real ps = P.v.v[e] * __ldg(cb_ + ia);
    ps = ps + __ldg(cc_ + ia) * d[e];
    P.v.v[e] = ps;
    const real upd = __ldg(ck_ + ia) * d[e] + ps;
    f.v[e] = f.v[e] + (T.sign * kf[e]) * upd;
  }
}

// Where a thread works: member, box, quad column and plane range.
struct SlabWork {
  int b, j, i0, k0, k1;
  bool live;
};

__device__ __forceinline__ SlabWork slab_work(const SlabLaunch& L, int nx) {
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
  w.k0 = bx.k0 + ch * kSlabPlanes;
  w.k1 = min(w.k0 + kSlabPlanes, bx.k1);
  w.live = col < ncol && w.i0 <= nx + 1;
  return w;
}

// ------------------------------------------------------------------------------------- E
// Index of the Debye current of pole 0 at (b, k, j, i) in the dense (P, B, nzA, Y, X) array.
template <typename real>
__device__ __forceinline__ long long jindex(const SweepArgs<real>& a, int c, int b, int k, int j, int i) {
  return (((long long)b * a.jnk[c] + (k - a.jk0[c])) * a.Y + j) * a.X + i;
}

// Per plane: every load first (H, E, indices, Debye currents, psi), then the arithmetic, then every
// store, so no load waits behind a store it cannot be proven not to alias.
template <typename real>
__device__ __forceinline__ void e_update(const SweepArgs<real>& a, int c, Quad<real>& e4, const Quad<uint16_t>& m,
                                         const real (&d0)[4], const real (&d1)[4], bool first_plus,
                                         PsiQuad<real> (&ps)[2], Quad<real>& j4, bool& disp, int i0, int j,
                                         int k, int b) {
  const int nx = a.nx;
  const Quad<real> e0 = e4;
  Coef<real> cf[4];
  real kf[4];
  bool valid[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int i = i0 + e;
    cf[e] = ldg_coef(a.coef + m.v[e]);
    kf[e] = cf[e].cb;
    valid[e] = i >= 1 && i <= nx + 1;
    const real acc = first_plus ? d0[e] + (-d1[e]) : d1[e] + (-d0[e]);
    if (valid[e]) e4.v[e] = cf[e].ca * e4.v[e] + cf[e].cb * acc;
  }
  psi_apply<real>(a.ecorr[c][0], ps[0], a.pe, e4, d0, kf, k, j, i0);
  psi_apply<real>(a.ecorr[c][1], ps[1], a.pe, e4, d1, kf, k, j, i0);
  disp = false;
#pragma unroll
  for (int e = 0; e < 4; ++e) disp |= valid[e] && m.v[e] >= a.ade_lo && m.v[e] < a.ade_hi;
  if (!disp) return;
  if (a.ade_P == 1) {
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
  } else {
    const long long jstride = (long long)a.B * a.jnk[c] * a.Y * a.X;
    disp = false;  // the general-pole update writes its currents itself
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      if (!(valid[e] && m.v[e] >= a.ade_lo && m.v[e] < a.ade_hi)) continue;
      e4.v[e] = ade_cell(e4.v[e], e0.v[e], cf[e].cbe, cf[e].beta0, m.v[e], a.J[c], jindex(a, c, b, k, j, i0) + e,
                         jstride, a.ade_kp,
                         a.ade_onekp, a.ade_beta, a.ade_P);
    }
  }
}

template <typename real>
__global__ void __launch_bounds__(kSlabThreads, 2)
    slab_e_kernel(const __grid_constant__ SweepArgs<real> a, const __grid_constant__ SlabLaunch L) {
  const SlabWork w = slab_work(L, a.nx);
  if (!w.live || w.k0 >= w.k1) return;
  const int X = a.X, Y = a.Y, Z = a.nz + 2, b = w.b, j = w.j, i0 = w.i0;
  const long long sz = (long long)X * Y;
  const long long base = (long long)b * a.bs;
  const real* Hx = a.H[0] + base;
  const real* Hy = a.H[1] + base;
  const real* Hz = a.H[2] + base;
  const Quad<real> idx4 = ld4(a.idd[0] + i0);
  const real idy = a.idd[1][j];
  long long q = (long long)w.k0 * sz + (long long)j * X + i0;  // offset within one member
  Quad<real> hx_m = ld4(Hx + q - sz), hy_m = ld4(Hy + q - sz);
  for (int k = w.k0; k < w.k1; ++k, q += sz) {
    // ---- loads
    const real idz = a.idd[2][k];
    const Quad<real> hx = ld4(Hx + q), hy = ld4(Hy + q), hz = ld4(Hz + q);
    const Quad<real> hzy = ld4(Hz + q - X), hxy = ld4(Hx + q - X);
    const real hz_l = Hz[q - 1], hy_l = Hy[q - 1];
    Quad<uint16_t> m[3];
    Quad<real> ev[3], jv[3];
    PsiQuad<real> ps[3][2];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      m[c] = ld4(a.mat[c] + q);
      ev[c] = ld4(a.E[c] + base + q);
      jv[c] = zero4<real>();
      if (a.ade_P == 1 && k >= a.jk0[c] && k < a.jk0[c] + a.jnk[c]) jv[c] = ld4(a.J[c] + jindex(a, c, b, k, j, i0));
#pragma unroll
      for (int t = 0; t < 2; ++t) {
        ps[c][t].sd = -1;
        if (a.has_cpml) psi_load<real>(a.ecorr[c][t], ps[c][t], b, k, j, i0, X, Y, Z);
      }
    }
    // ---- arithmetic
    bool disp[3];
    real d0[4], d1[4];
    // Ex: terms (a = y, +Hz) then (a = z, -Hy)
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      d0[e] = (hz.v[e] - hzy.v[e]) * idy;
      d1[e] = (hy.v[e] - hy_m.v[e]) * idz;
    }
    e_update<real>(a, 0, ev[0], m[0], d0, d1, true, ps[0], jv[0], disp[0], i0, j, k, b);
    // Ey: terms (a = z, +Hx) then (a = x, -Hz); d0 is the x term, d1 the z term
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const real hzl = e > 0 ? hz.v[e - 1] : hz_l;
      d0[e] = (hz.v[e] - hzl) * idx4.v[e];
      d1[e] = (hx.v[e] - hx_m.v[e]) * idz;
    }
    e_update<real>(a, 1, ev[1], m[1], d0, d1, false, ps[1], jv[1], disp[1], i0, j, k, b);
    // Ez: terms (a = x, +Hy) then (a = y, -Hx)
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const real hyl = e > 0 ? hy.v[e - 1] : hy_l;
      d0[e] = (hy.v[e] - hyl) * idx4.v[e];
      d1[e] = (hx.v[e] - hxy.v[e]) * idy;
    }
    e_update<real>(a, 2, ev[2], m[2], d0, d1, true, ps[2], jv[2], disp[2], i0, j, k, b);
    // ---- stores
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      st4(a.E[c] + base + q, ev[c]);
      if (disp[c]) st4(a.J[c] + jindex(a, c, b, k, j, i0), jv[c]);
#pragma unroll
      for (int t = 0; t < 2; ++t) psi_store<real>(a.ecorr[c][t], ps[c][t], b, k, j, i0, X, Y, Z);
    }
    hx_m = hx;
    hy_m = hy;
  }
}

// ------------------------------------------------------------------------------------- H
template <typename real>
__device__ __forceinline__ void h_update(const SweepArgs<real>& a, int c, Quad<real>& h, const real (&d0)[4],
                                         const real (&d1)[4], const real (&acc)[4], int ilast,
                                         PsiQuad<real> (&ps)[2], int i0, int j, int k) {
  const real dtmu = a.dtmu;
  real kf[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int i = i0 + e;
    kf[e] = dtmu;
    if (i >= 1 && i <= ilast) h.v[e] = h.v[e] + dtmu * acc[e];
  }
  psi_apply<real>(a.hcorr[c][0], ps[0], a.ph, h, d0, kf, k, j, i0);
  psi_apply<real>(a.hcorr[c][1], ps[1], a.ph, h, d1, kf, k, j, i0);
}

template <typename real>
__global__ void __launch_bounds__(kSlabThreads, 2)
    slab_h_kernel(const __grid_constant__ SweepArgs<real> a, const __grid_constant__ SlabLaunch L) {
  const SlabWork w = slab_work(L, a.nx);
  if (!w.live || w.k0 >= w.k1) return;
  const int X = a.X, Y = a.Y, Z = a.nz + 2, nx = a.nx, ny = a.ny, nz = a.nz, b = w.b, j = w.j, i0 = w.i0;
  const long long sz = (long long)X * Y;
  const long long base = (long long)b * a.bs;
  const real* Ex = a.E[0] + base;
  const real* Ey = a.E[1] + base;
  const real* Ez = a.E[2] + base;
  const Quad<real> ipx = ld4(a.ip[0] + i0);
  const real ipy = a.ip[1][j];
  const bool right = i0 + 4 < X;  // the x + 1 neighbour of element 3 is in the row
  const bool jin = j <= ny;
  long long q = (long long)w.k0 * sz + (long long)j * X + i0;
  Quad<real> ex = ld4(Ex + q), ey = ld4(Ey + q);
  for (int k = w.k0; k < w.k1; ++k, q += sz) {
    // ---- loads
    const bool kin = k <= nz;
    const real ipz = a.ip[2][k];
    Quad<real> ex1 = zero4<real>(), ey1 = zero4<real>(), ezy = zero4<real>(), exy = zero4<real>();
    if (kin) {
      ex1 = ld4(Ex + q + sz);
      ey1 = ld4(Ey + q + sz);
    }
    if (jin) {
      ezy = ld4(Ez + q + X);
      exy = ld4(Ex + q + X);
    }
    const Quad<real> ez = ld4(Ez + q);
    const real ez_r = right ? Ez[q + 4] : (real)0, ey_r = right ? Ey[q + 4] : (real)0;
    Quad<real> hv[3];
    PsiQuad<real> ps[3][2];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      hv[c] = ld4(a.H[c] + base + q);
#pragma unroll
      for (int t = 0; t < 2; ++t) {
        ps[c][t].sd = -1;
        if (a.has_cpml) psi_load<real>(a.hcorr[c][t], ps[c][t], b, k, j, i0, X, Y, Z);
      }
    }
    // ---- arithmetic
    real d0[4], d1[4], acc[4];
    const bool upd[3] = {jin && kin, kin, jin};
    if (upd[0]) {  // Hx: node along x (1..nx+1), cell along y and z
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        d0[e] = (ezy.v[e] - ez.v[e]) * ipy;  // axis y
        d1[e] = (ey1.v[e] - ey.v[e]) * ipz;  // axis z
        acc[e] = (-d0[e]) + d1[e];
      }
      h_update<real>(a, 0, hv[0], d0, d1, acc, nx + 1, ps[0], i0, j, k);
    }
    if (upd[1]) {  // Hy: cell along x (1..nx), node along y (1..ny+1), cell along z
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const real ezr = e < 3 ? ez.v[e + 1] : ez_r;
        d0[e] = (ezr - ez.v[e]) * ipx.v[e];  // axis x
        d1[e] = (ex1.v[e] - ex.v[e]) * ipz;  // axis z
        acc[e] = (-d1[e]) + d0[e];
      }
      h_update<real>(a, 1, hv[1], d0, d1, acc, nx, ps[1], i0, j, k);
    }
    if (upd[2]) {  // Hz: cell along x and y, node along z (1..nz+1)
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const real eyr = e < 3 ? ey.v[e + 1] : ey_r;
        d0[e] = (eyr - ey.v[e]) * ipx.v[e];  // axis x
        d1[e] = (exy.v[e] - ex.v[e]) * ipy;  // axis y
        acc[e] = (-d0[e]) + d1[e];
      }
      h_update<real>(a, 2, hv[2], d0, d1, acc, nx, ps[2], i0, j, k);
    }
    // ---- stores
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      if (!upd[c]) continue;
      st4(a.H[c] + base + q, hv[c]);
#pragma unroll
      for (int t = 0; t < 2; ++t) psi_store<real>(a.hcorr[c][t], ps[c][t], b, k, j, i0, X, Y, Z);
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
    L.nch[L.n] = (bx.k1 - bx.k0 + kSlabPlanes - 1) / kSlabPlanes;
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
