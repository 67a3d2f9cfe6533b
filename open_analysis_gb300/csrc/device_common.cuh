// Device helpers shared by the sweep kernels: 4-cell vectors ("quads"), async copies and the
// general-pole Debye update.
#pragma once

#include "oafdtd_internal.cuh"

namespace oafdtd {

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

// One entry of the combined material table through the read-only data path (the table does
// not change during a run).
__device__ __forceinline__ Coef<float> ldg_coef(const Coef<float>* p) {
  const float4 t = __ldg(reinterpret_cast<const float4*>(p));
  return Coef<float>{t.x, t.y, t.z, t.w};
}
__device__ __forceinline__ Coef<double> ldg_coef(const Coef<double>* p) {
  const double2 a = __ldg(reinterpret_cast<const double2*>(p));
  const double2 b = __ldg(reinterpret_cast<const double2*>(p) + 1);
  return Coef<double>{a.x, a.y, b.x, b.y};
}

template <typename real>
__device__ __forceinline__ Quad<real> zero4() {
  return Quad<real>{{(real)0, (real)0, (real)0, (real)0}};
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

// ---------------------------------------------------------------------------- E update of a quad
// A z-term correction of one quad: psi <- b psi + c d; F <- F + (sign k)(ek d + psi), with the
// plane's coefficients and psi staged in shared memory, for the cells of the correction box; the
// updated psi row goes back to global memory.
template <typename real>
struct ZTerm {
  const real* sm;  // staged psi of the quad
  real* g;         // psi of the quad in global memory
  real eb, ec, ek, sign;
  int lo0, hi0;
  bool on;         // the row and plane lie in the correction box
};

template <typename real>
__device__ __forceinline__ ZTerm<real> z_term(const SweepArgs<real>& a, const CpmlTerm<real>& T, int sd,
                                              const real* sm, int b, int k, int j, int i0, int kind) {
  ZTerm<real> z;
  z.on = false;
  if (sd < 0) return z;
  const CpmlSide<real>& s = sd == 0 ? T.side[0] : T.side[1];
  z.on = j >= s.lo[1] && j < s.hi[1] && k >= s.lo[2] && k < s.hi[2];
  if (!z.on) return z;
  const int w = s.hi[2] - s.lo[2];
  z.sm = sm;
  z.g = s.psi + ((((long long)b * w + (k - s.lo[2])) * a.Y + j) * a.X + i0);
  const real* const* co = kind == 0 ? a.pe[2] : a.ph[2];
  z.eb = __ldg(co[0] + k);
  z.ec = __ldg(co[1] + k);
  z.ek = __ldg(co[2] + k);
  z.sign = T.sign;
  z.lo0 = s.lo[0];
  z.hi0 = s.hi[0];
  return z;
}

template <typename real>
__device__ __forceinline__ void z_apply(const ZTerm<real>& z, Quad<real>& f, const real (&d)[4], const real (&kf)[4],
                                        int i0) {
  if (!z.on) return;
  Quad<real> ps = ld4(z.sm);
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int i = i0 + e;
    if (i < z.lo0 || i >= z.hi0) continue;
    real p = ps.v[e] * z.eb;
    p = p + z.ec * d[e];
    ps.v[e] = p;
    const real upd = z.ek * d[e] + p;
    f.v[e] = f.v[e] + (z.sign * kf[e]) * upd;
  }
  st4(z.g, ps);
}

// Bulk update, z correction (z sweeps) and the Debye update of one E component on one quad, in
// the reference's order. d0/d1 are the derivatives along the component's two axes in ascending
// order; the reference's term order is (d0, -d1) when first_plus, else (d1, -d0). j4 holds the
// prefetched Debye current (P = 1).
template <typename real, bool kZ, bool kMulti>
__device__ __forceinline__ void e_apply(const SweepArgs<real>& a, int c, real* __restrict__ E, long long p,
                                        const Quad<real>& e_old, const uint16_t* m, const real (&d0)[4],
                                        const real (&d1)[4], bool first_plus, const Quad<real>& j4in,
                                        const ZTerm<real>& zt, int i0, int j, int k, int b,
                                        const Coef<real>* ctab = nullptr) {
  const int X = a.X, Y = a.Y, nx = a.nx;
  const Coef<real>* tab = ctab != nullptr ? ctab : a.coef;  // the table staged in shared memory, or global
  Quad<real> e4 = e_old;
  Coef<real> cf[4];
  real kf[4];
  bool valid[4];
  bool disp = false;
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int i = i0 + e;
    cf[e] = tab[m[e]];
    kf[e] = cf[e].cb;
    valid[e] = i >= 1 && i <= nx + 1;
    const real acc = first_plus ? d0[e] + (-d1[e]) : d1[e] + (-d0[e]);
    if (valid[e]) e4.v[e] = cf[e].ca * e4.v[e] + cf[e].cb * acc;
    disp |= valid[e] && m[e] >= a.ade_lo && m[e] < a.ade_hi;
  }
  if constexpr (kZ) z_apply(zt, e4, d1, kf, i0);
  if (disp) {
    const long long jstride = (long long)a.B * a.jnk[c] * Y * X;
    const long long jq = (((long long)b * a.jnk[c] + (k - a.jk0[c])) * Y + j) * X + i0;
    real* J = a.J[c];
    if constexpr (!kMulti) {
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

}  // namespace oafdtd
