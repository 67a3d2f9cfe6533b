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

}  // namespace oafdtd
