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

#include <algorithm>

#include "device_common.cuh"

namespace oafdtd {

constexpr int kSlabThreads = 256;
// Planes marched per thread. The slab boxes are thin (CPML slabs of ~10 cells): short marches
// give the kernel enough independent threads to hide its load latency.
constexpr int kSlabPlanes = 4;


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

// Where a thread works: field component, member, box, quad column and plane range. The
// component is the fastest-varying block index, so the three components of a region run side by
// side and share their source-field reads through L1 and L2.
struct SlabWork {
  int comp, b, j, i0, k0, k1;
  bool live;
};

__device__ __forceinline__ SlabWork slab_work(const SlabLaunch& L, int nx, int block) {
  const int blk = block / 3;
  int s = 0;
  while (s + 1 < L.n && blk >= L.first[s + 1]) ++s;
  const Span3 bx = L.box[s];
  int r = blk - L.first[s];
  const int cb = r % L.cblk[s];
  r /= L.cblk[s];
  const int ch = r % L.nch[s];
  SlabWork w;
  w.comp = block % 3;
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

// One E component on one quad column. Per plane: every load first (H, E, index, Debye current,
// psi), then the arithmetic, then every store, so no load waits behind a store it cannot be proven
// not to alias. C: 0 Ex (terms y +Hz, z -Hy), 1 Ey (z +Hx, x -Hz), 2 Ez (x +Hy, y -Hx); d0 is
// the derivative along the first axis in ascending order, d1 along the second.
// kMulti: more than one Debye pole (the general update, a call); single-pole runs compile without
// it, so their registers never spill around the call.
template <typename real, int C, bool kMulti>
__device__ __forceinline__ void slab_e_column(const SweepArgs<real>& a, const SlabWork& w) {
  const int X = a.X, Y = a.Y, Z = a.nz + 2, nx = a.nx, b = w.b, j = w.j, i0 = w.i0;
  const long long sz = (long long)X * Y;
  const long long base = (long long)b * a.bs;
  const real* Hx = a.Ho[0] + base;  // H^{n+1/2}
  const real* Hy = a.Ho[1] + base;
  const real* Hz = a.Ho[2] + base;
  const real* E = a.E[C] + base;     // E^n
  real* Eo = a.Eo[C] + base;         // E^{n+1}
  const Quad<real> idx4 = ld4(a.idd[0] + i0);
  const real idy = a.idd[1][j];
  long long q = (long long)w.k0 * sz + (long long)j * X + i0;  // offset within one member
  // the z-derivative source at plane k - 1, carried (Ex: Hy, Ey: Hx)
  Quad<real> hm = zero4<real>();
  if (C == 0) hm = ld4(Hy + q - sz);
  if (C == 1) hm = ld4(Hx + q - sz);
  for (int k = w.k0; k < w.k1; ++k, q += sz) {
    // ---- loads
    Quad<real> s0, s1, s2;  // sources of the two derivatives
    real sl = (real)0;      // x - 1 neighbour of element 0
    if (C == 0) {
      s0 = ld4(Hz + q);
      s1 = ld4(Hz + q - X);
      s2 = ld4(Hy + q);
    } else if (C == 1) {
      s0 = ld4(Hz + q);
      if (i0 > 0) sl = Hz[q - 1];  // cell 0 is never updated: no neighbour from the row before
      s2 = ld4(Hx + q);
    } else {
      s0 = ld4(Hy + q);
      if (i0 > 0) sl = Hy[q - 1];
      s2 = ld4(Hx + q);
      s1 = ld4(Hx + q - X);
    }
    const Quad<uint16_t> m = ld4(a.mat[C] + q);
    Quad<real> e4 = ld4(E + q);
    const bool jrange = a.ade_P == 1 && k >= a.jk0[C] && k < a.jk0[C] + a.jnk[C];
    Quad<real> j4 = zero4<real>();
    if (jrange) j4 = ld4(a.J[C] + jindex(a, C, b, k, j, i0));
    PsiQuad<real> ps[2];
    ps[0].sd = ps[1].sd = -1;
    if (a.has_cpml) {
      psi_load<real>(a.ecorr[C][0], ps[0], b, k, j, i0, X, Y, Z);
      psi_load<real>(a.ecorr[C][1], ps[1], b, k, j, i0, X, Y, Z);
    }
    // ---- arithmetic
    real d0[4], d1[4];
    const real idz = a.idd[2][k];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      if (C == 0) {
        d0[e] = (s0.v[e] - s1.v[e]) * idy;  // y: Hz
        d1[e] = (s2.v[e] - hm.v[e]) * idz;  // z: Hy
      } else if (C == 1) {
        const real l = e > 0 ? s0.v[e - 1] : sl;
        d0[e] = (s0.v[e] - l) * idx4.v[e];  // x: Hz
        d1[e] = (s2.v[e] - hm.v[e]) * idz;  // z: Hx
      } else {
        const real l = e > 0 ? s0.v[e - 1] : sl;
        d0[e] = (s0.v[e] - l) * idx4.v[e];  // x: Hy
        d1[e] = (s2.v[e] - s1.v[e]) * idy;  // y: Hx
      }
    }
    const bool first_plus = C != 1;  // the reference's term order: (d0, -d1), for Ey (d1, -d0)
    const Quad<real> e0 = e4;
    real kf[4];
    bool valid[4], dis[4];
    bool disp = false;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int i = i0 + e;
      const Coef<real> cf = ldg_coef(a.coef + m.v[e]);
      kf[e] = cf.cb;
      valid[e] = i >= 1 && i <= nx + 1;
      const real acc = first_plus ? d0[e] + (-d1[e]) : d1[e] + (-d0[e]);
      if (valid[e]) e4.v[e] = cf.ca * e4.v[e] + cf.cb * acc;
      dis[e] = valid[e] && m.v[e] >= a.ade_lo && m.v[e] < a.ade_hi;
      disp |= dis[e];
    }
    psi_apply<real>(a.ecorr[C][0], ps[0], a.pe, e4, d0, kf, k, j, i0);
    psi_apply<real>(a.ecorr[C][1], ps[1], a.pe, e4, d1, kf, k, j, i0);
    if (disp) {
      if constexpr (!kMulti) {
        const real onekp = a.ade_onekp[0], kp = a.ade_kp[0];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          if (!dis[e]) continue;
          const Coef<real> cf = ldg_coef(a.coef + m.v[e]);  // the Debye coefficients (cbe, beta_0)
          const real jt = (real)0.5 * (onekp * j4.v[e]);
          const real en = e4.v[e] - cf.cbe * jt;
          const real de = en - e0.v[e];
          j4.v[e] = kp * j4.v[e] + cf.beta0 * de;
          e4.v[e] = en;
        }
      } else {
        const long long jstride = (long long)a.B * a.jnk[C] * Y * X;
        const long long jq = jindex(a, C, b, k, j, i0);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          if (!dis[e]) continue;
          const Coef<real> cf = ldg_coef(a.coef + m.v[e]);
          e4.v[e] = ade_cell(e4.v[e], e0.v[e], cf.cbe, cf.beta0, m.v[e], a.J[C], jq + e, jstride, a.ade_kp,
                             a.ade_onekp, a.ade_beta, a.ade_P);
        }
      }
    }
    // ---- stores
    st4(Eo + q, e4);
    if (!kMulti && disp) st4(a.J[C] + jindex(a, C, b, k, j, i0), j4);
    psi_store<real>(a.ecorr[C][0], ps[0], b, k, j, i0, X, Y, Z);
    psi_store<real>(a.ecorr[C][1], ps[1], b, k, j, i0, X, Y, Z);
    if (C == 0) hm = s2;
    if (C == 1) hm = s2;
  }
}

template <typename real, bool kMulti>
__device__ __forceinline__ void slab_e_body(const SweepArgs<real>& a, const SlabLaunch& L, int block) {
  const SlabWork w = slab_work(L, a.nx, block);
  if (!w.live || w.k0 >= w.k1) return;
  if (w.comp == 0)
    slab_e_column<real, 0, kMulti>(a, w);
  else if (w.comp == 1)
    slab_e_column<real, 1, kMulti>(a, w);
  else
    slab_e_column<real, 2, kMulti>(a, w);
}

template <typename real, bool kMulti>
__global__ void __launch_bounds__(kSlabThreads, 3)
    slab_e_kernel(const __grid_constant__ SweepArgs<real> a, const __grid_constant__ SlabLaunch L) {
  slab_e_body<real, kMulti>(a, L, (int)blockIdx.x);
}

// Several engines' E slab updates in one launch: engine e's arguments at A[e] and L[e].
template <typename real, bool kMulti>
__global__ void __launch_bounds__(kSlabThreads, 3)
    slab_e_batch_kernel(const SweepArgs<real>* __restrict__ A, const SlabLaunch* __restrict__ L, const BatchGrid G) {
  __shared__ __align__(16) unsigned char args[sizeof(SweepArgs<real>)];
  __shared__ __align__(16) unsigned char launch[sizeof(SlabLaunch)];
  int e;
  const uint3 bid = G.block(&e);
  const SlabLaunch& l = stage_args(L + e, launch);
  slab_e_body<real, kMulti>(stage_args(A + e, args), l, (int)bid.x);
}

// ------------------------------------------------------------------------------------- H
// One H component on one quad column. C: 0 Hx (terms y -Ez, z +Ey), 1 Hy (z -Ex, x +Ez),
// 2 Hz (x -Ey, y +Ex); d0 along the first axis in ascending order, d1 along the second.
template <typename real, int C>
__device__ __forceinline__ void slab_h_column(const SweepArgs<real>& a, const SlabWork& w) {
  const int X = a.X, Y = a.Y, Z = a.nz + 2, nx = a.nx, ny = a.ny, nz = a.nz, b = w.b, j = w.j, i0 = w.i0;
  // the cells this component updates: Hx i in 1..nx+1, j <= ny, k <= nz; Hy i <= nx, k <= nz;
  // Hz i <= nx, j <= ny
  if ((C == 0 || C == 2) && j > ny) return;
  const int ilast = C == 0 ? nx + 1 : nx;
  const long long sz = (long long)X * Y;
  const long long base = (long long)b * a.bs;
  const real* Ex = a.E[0] + base;
  const real* Ey = a.E[1] + base;
  const real* Ez = a.E[2] + base;
  const real* H = a.H[C] + base;  // H^{n-1/2}
  real* Ho = a.Ho[C] + base;      // H^{n+1/2}
  const Quad<real> ipx = ld4(a.ip[0] + i0);
  const real ipy = a.ip[1][j];
  const bool right = i0 + 4 < X;  // the x + 1 neighbour of element 3 is in the row
  const real dtmu = a.dtmu;
  long long q = (long long)w.k0 * sz + (long long)j * X + i0;
  // the z-derivative source at plane k, carried from the previous plane's k + 1 (Hx: Ey, Hy: Ex)
  Quad<real> sc = zero4<real>();
  if (C == 0) sc = ld4(Ey + q);
  if (C == 1) sc = ld4(Ex + q);
  for (int k = w.k0; k < w.k1; ++k, q += sz) {
    if (C != 2 && k > nz) break;
    // ---- loads
    Quad<real> s0, s1, s2;
    real sr = (real)0;  // x + 1 neighbour of element 3
    if (C == 0) {
      s0 = ld4(Ez + q + X);   // y: Ez(j + 1)
      s1 = ld4(Ez + q);
      s2 = ld4(Ey + q + sz);  // z: Ey(k + 1)
    } else if (C == 1) {
      s0 = ld4(Ez + q);       // x: Ez
      sr = right ? Ez[q + 4] : (real)0;
      s2 = ld4(Ex + q + sz);  // z: Ex(k + 1)
    } else {
      s0 = ld4(Ey + q);       // x: Ey
      sr = right ? Ey[q + 4] : (real)0;
      s2 = ld4(Ex + q + X);   // y: Ex(j + 1)
      s1 = ld4(Ex + q);
    }
    Quad<real> h = ld4(H + q);
    PsiQuad<real> ps[2];
    ps[0].sd = ps[1].sd = -1;
    if (a.has_cpml) {
      psi_load<real>(a.hcorr[C][0], ps[0], b, k, j, i0, X, Y, Z);
      psi_load<real>(a.hcorr[C][1], ps[1], b, k, j, i0, X, Y, Z);
    }
    // ---- arithmetic
    const real ipz = a.ip[2][k];
    real d0[4], d1[4], kf[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      real acc;
      if (C == 0) {
        d0[e] = (s0.v[e] - s1.v[e]) * ipy;  // y
        d1[e] = (s2.v[e] - sc.v[e]) * ipz;  // z
        acc = (-d0[e]) + d1[e];
      } else if (C == 1) {
        const real r = e < 3 ? s0.v[e + 1] : sr;
        d0[e] = (r - s0.v[e]) * ipx.v[e];   // x
        d1[e] = (s2.v[e] - sc.v[e]) * ipz;  // z
        acc = (-d1[e]) + d0[e];
      } else {
        const real r = e < 3 ? s0.v[e + 1] : sr;
        d0[e] = (r - s0.v[e]) * ipx.v[e];   // x
        d1[e] = (s2.v[e] - s1.v[e]) * ipy;  // y
        acc = (-d0[e]) + d1[e];
      }
      const int i = i0 + e;
      kf[e] = dtmu;
      if (i >= 1 && i <= ilast) h.v[e] = h.v[e] + dtmu * acc;
    }
    psi_apply<real>(a.hcorr[C][0], ps[0], a.ph, h, d0, kf, k, j, i0);
    psi_apply<real>(a.hcorr[C][1], ps[1], a.ph, h, d1, kf, k, j, i0);
    // ---- stores
    st4(Ho + q, h);
    psi_store<real>(a.hcorr[C][0], ps[0], b, k, j, i0, X, Y, Z);
    psi_store<real>(a.hcorr[C][1], ps[1], b, k, j, i0, X, Y, Z);
    if (C != 2) sc = s2;
  }
}

template <typename real>
__device__ __forceinline__ void slab_h_body(const SweepArgs<real>& a, const SlabLaunch& L, int block) {
  const SlabWork w = slab_work(L, a.nx, block);
  if (!w.live || w.k0 >= w.k1) return;
  if (w.comp == 0)
    slab_h_column<real, 0>(a, w);
  else if (w.comp == 1)
    slab_h_column<real, 1>(a, w);
  else
    slab_h_column<real, 2>(a, w);
}

template <typename real>
__global__ void __launch_bounds__(kSlabThreads, 4)
    slab_h_kernel(const __grid_constant__ SweepArgs<real> a, const __grid_constant__ SlabLaunch L) {
  slab_h_body<real>(a, L, (int)blockIdx.x);
}

// Several engines' H slab updates in one launch.
template <typename real>
__global__ void __launch_bounds__(kSlabThreads, 4)
    slab_h_batch_kernel(const SweepArgs<real>* __restrict__ A, const SlabLaunch* __restrict__ L, const BatchGrid G) {
  __shared__ __align__(16) unsigned char args[sizeof(SweepArgs<real>)];
  __shared__ __align__(16) unsigned char launch[sizeof(SlabLaunch)];
  int e;
  const uint3 bid = G.block(&e);
  const SlabLaunch& l = stage_args(L + e, launch);
  slab_h_body<real>(stage_args(A + e, args), l, (int)bid.x);
}

// ------------------------------------------------------------------------------------- launch
template <typename real>
cudaError_t slab_plan(const SweepArgs<real>& a, int kind, SlabLaunch* L, long long* blocks) {
  *L = SlabLaunch{};
  L->n = 0;
  *blocks = 0;
  long long total = 0;
  for (int n = 0; n < a.n_slab[kind]; ++n) {
    Span3 bx = a.slab[kind][n];
    bx.q1 = std::min(bx.q1, (a.nx + 1) / 4 + 1);  // quads past the last updated cell hold no work
    const long long cols = (long long)(bx.q1 - bx.q0) * (bx.j1 - bx.j0);
    if (cols <= 0 || bx.k1 <= bx.k0) continue;
    L->box[L->n] = bx;
    L->first[L->n] = (int)total;
    L->cblk[L->n] = (int)((cols + kSlabThreads - 1) / kSlabThreads);
    L->nch[L->n] = (bx.k1 - bx.k0 + kSlabPlanes - 1) / kSlabPlanes;
    total += (long long)L->cblk[L->n] * L->nch[L->n] * a.B;
    ++L->n;
  }
  if (L->n == 0) return cudaSuccess;
  if (3 * total > 2147483647LL) return cudaErrorInvalidConfiguration;
  L->first[L->n] = (int)total;
  *blocks = 3 * total;  // one block per component of every column block
  return cudaSuccess;
}

template <typename real>
cudaError_t launch_slab(const SweepArgs<real>& a, int kind, cudaStream_t s) {
  SlabLaunch L;
  long long blocks = 0;
  if (const cudaError_t e = slab_plan(a, kind, &L, &blocks)) return e;
  if (blocks == 0) return cudaSuccess;
  if (kind == 0 && a.ade_P > 1)
    slab_e_kernel<real, true><<<(unsigned)blocks, kSlabThreads, 0, s>>>(a, L);
  else if (kind == 0)
    slab_e_kernel<real, false><<<(unsigned)blocks, kSlabThreads, 0, s>>>(a, L);
  else
    slab_h_kernel<real><<<(unsigned)blocks, kSlabThreads, 0, s>>>(a, L);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_slab_batch(const SweepArgs<real>* A, const SlabLaunch* L, const BatchGrid& G, int blocks, int kind,
                              bool multi_pole, cudaStream_t s) {
  if (blocks <= 0) return cudaSuccess;
  if (kind == 0 && multi_pole)
    slab_e_batch_kernel<real, true><<<blocks, kSlabThreads, 0, s>>>(A, L, G);
  else if (kind == 0)
    slab_e_batch_kernel<real, false><<<blocks, kSlabThreads, 0, s>>>(A, L, G);
  else
    slab_h_batch_kernel<real><<<blocks, kSlabThreads, 0, s>>>(A, L, G);
  return cudaGetLastError();
}

template <typename real>
cudaError_t preload_slab() {
  cudaFuncAttributes fa;
  const void* fns[] = {
      reinterpret_cast<const void*>(slab_e_kernel<real, false>),
      reinterpret_cast<const void*>(slab_e_kernel<real, true>),
      reinterpret_cast<const void*>(slab_h_kernel<real>),
      reinterpret_cast<const void*>(slab_e_batch_kernel<real, false>),
      reinterpret_cast<const void*>(slab_e_batch_kernel<real, true>),
      reinterpret_cast<const void*>(slab_h_batch_kernel<real>),
  };
  for (const void* f : fns) {
    const cudaError_t err = cudaFuncGetAttributes(&fa, f);
    if (err != cudaSuccess) return err;
  }
  return cudaSuccess;
}

template cudaError_t preload_slab<float>();
template cudaError_t preload_slab<double>();
template cudaError_t slab_plan<float>(const SweepArgs<float>&, int, SlabLaunch*, long long*);
template cudaError_t slab_plan<double>(const SweepArgs<double>&, int, SlabLaunch*, long long*);
template cudaError_t launch_slab_batch<float>(const SweepArgs<float>*, const SlabLaunch*, const BatchGrid&, int, int,
                                              bool, cudaStream_t);
template cudaError_t launch_slab_batch<double>(const SweepArgs<double>*, const SlabLaunch*, const BatchGrid&, int, int,
                                               bool, cudaStream_t);
template cudaError_t launch_slab<float>(const SweepArgs<float>&, int, cudaStream_t);
template cudaError_t launch_slab<double>(const SweepArgs<double>&, int, cudaStream_t);

}  // namespace oafdtd
