// Device helpers shared by the sweep kernels: 4-cell vectors ("quads"), async copies, the CPML
// correction of a quad and the general-pole Debye update.
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

template <typename real>
__device__ __forceinline__ Quad<real> zero4() {
  return Quad<real>{{(real)0, (real)0, (real)0, (real)0}};
}

enum : int { kBulk = 0, kSlabPlanes = 1, kSlabColumns = 2 };

// The CPML corrections of one component on one quad: for each derivative axis (ascending) whose
// slab holds the cell, psi <- b psi + c d; f += (sign k) (ek d + psi). Slabs along y and z hold
// whole quads, so their psi moves as one vector; x slabs are handled cell by cell.
template <typename real, int KIND>
__device__ __forceinline__ void cpml_quad(const SweepArgs<real>& a, const CpmlTerm<real> (&terms)[2],
                                          const real* const (&co)[3][3], Quad<real>& f, const real (&d0)[4],
                                          const real (&d1)[4], const real (&kfac)[4], const bool (&valid)[4],
                                          int i0, int j, int k, int b) {
  const int X = a.X, Y = a.Y, Z = a.nz + 2;
#pragma unroll
  for (int t = 0; t < 2; ++t) {
    const CpmlTerm<real>& T = terms[t];
    if (T.side[0].psi == nullptr) continue;
    const int ax = T.axis;
    const real* cb_ = co[ax][0];
    const real* cc_ = co[ax][1];
    const real* ck_ = co[ax][2];
    if (ax == 0) {
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int i = i0 + e;
        const int s = a.side[KIND][0][i];
        if (!valid[e] || s < 0) continue;
        const CpmlSide<real>& S = T.side[s];
        if (j < S.lo[1] || j >= S.hi[1] || k < S.lo[2] || k >= S.hi[2] || i < S.lo[0] || i >= S.hi[0]) continue;
        const int w = S.hi[0] - S.lo[0];
        const long long q = (((long long)b * Z + k) * Y + j) * w + (i - S.lo[0]);
        const real d = t == 0 ? d0[e] : d1[e];
        real ps = S.psi[q];
        ps = ps * cb_[i];
        ps = ps + cc_[i] * d;
        S.psi[q] = ps;
        const real upd = ck_[i] * d + ps;
        f.v[e] = f.v[e] + (T.sign * kfac[e]) * upd;
      }
    } else {
      const int ia = ax == 1 ? j : k;
      const int s = a.side[KIND][ax][ia];
      if (s < 0) continue;
      const CpmlSide<real>& S = T.side[s];
      const int other = ax == 1 ? k : j;
      const int oax = ax == 1 ? 2 : 1;
      if (other < S.lo[oax] || other >= S.hi[oax] || ia < S.lo[ax] || ia >= S.hi[ax]) continue;
      const int w = S.hi[ax] - S.lo[ax];
      const long long q0 = ax == 1 ? (((long long)b * Z + k) * w + (j - S.lo[1])) * X + i0
                                   : (((long long)b * w + (k - S.lo[2])) * Y + j) * X + i0;
      Quad<real> ps4 = ld4(S.psi + q0);
      const real pb = cb_[ia], pc = cc_[ia], pk = ck_[ia];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int i = i0 + e;
        if (!valid[e] || i < S.lo[0] || i >= S.hi[0]) continue;
        const real d = t == 0 ? d0[e] : d1[e];
        real ps = ps4.v[e] * pb;
        ps = ps + pc * d;
        ps4.v[e] = ps;
        const real upd = pk * d + ps;
        f.v[e] = f.v[e] + (T.sign * kfac[e]) * upd;
      }
      st4(S.psi + q0, ps4);
    }
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

}  // namespace oafdtd
