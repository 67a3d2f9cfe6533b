// CPML correction passes.
//
// After a sweep has given every cell its bulk update, the corrections of the slab cells are
// applied by three passes, one per derivative axis in ascending order (x, then y, then z), each
// covering both slab sides and every component with a term on that axis. A cell in a slab corner
// therefore receives its corrections in the reference's order (packages/oa-fdtd/src/oa_fdtd/
// reference.py:182-207, the corrections of oa_fdtd.pml.build_pml in axis order), each rounded
// to the field precision: psi <- b psi + c d; F += (sign k) (ek d + psi), with d recomputed from
// the source field (unchanged during the pass) exactly as the bulk update computed it.
//
// Every thread owns one cell (x slabs) or one quad of four x cells (y and z slabs, whose psi rows
// are contiguous in x) and nothing else, so the passes have no carried dependency and keep many
// loads in flight.
//
// Debye edges inside an E slab: the reference applies the CPML correction t before the Debye
// update, whose current update J_p = k_p J_p + beta_p (E^{n+1} - E^n) depends on it; the sweep
// has already done the Debye update without t. Adding t to E and beta_p t to every J_p gives the
// same E^{n+1} and J^{n+1}; only the rounding of these edges differs from the reference's order.
// (Dispersive edges with injection are updated by the edge pass, after the corrections, in the
// reference's order.)

#include "device_common.cuh"

namespace oafdtd {

template <typename real>
struct CorrItem {
  real* F;          // corrected field component
  const real* S;    // source component of the derivative
  real* psi;        // (B, Z', Y', X') with the slab on the derivative axis
  int c;            // corrected component (E: material index array)
  real sign;
  int lo[3], hi[3]; // box
};

template <typename real>
struct CorrArgs {
  CorrItem<real> item[4];
  int n_items;
  int kind;         // 0 E, 1 H
  int axis;
  const real* cb_;  // psi coefficients of the axis
  const real* cc_;
  const real* ck_;
  const real* inv;  // inverse lengths along the axis (dual for E, primal for H)
  real dtmu;
  const uint16_t* mat[3];
  const Coef<real>* coef;
  int ade_lo, ade_hi, ade_P;
  const real* ade_beta;     // [entry * P + p]
  real* J[3];
  int jk0[3], jnk[3];
  int X, Y, Z, B;
  long long bs;
};

// E^{n+1} of a dispersive edge has moved by t after its Debye update: move every J_p by beta_p t.
template <typename real>
__device__ __forceinline__ void debye_shift(const CorrArgs<real>& a, int c, int m, real t, int b, int k, int j,
                                            int i) {
  if (m < a.ade_lo || m >= a.ade_hi) return;
  const long long plane = (long long)a.Y * a.X;
  const long long jq = ((long long)b * a.jnk[c] + (k - a.jk0[c])) * plane + (long long)j * a.X + i;
  const long long stride = (long long)a.B * a.jnk[c] * plane;
  for (int p = 0; p < a.ade_P; ++p) {
    const real beta = p == 0 ? a.coef[m].beta0 : a.ade_beta[(long long)m * a.ade_P + p];
    a.J[c][jq + p * stride] = a.J[c][jq + p * stride] + beta * t;
  }
}

template <typename real>
__global__ void __launch_bounds__(256) cpml_pass_kernel(const __grid_constant__ CorrArgs<real> a) {
  const CorrItem<real>& it = a.item[blockIdx.y];
  const int ax = a.axis;
  const int X = a.X, Y = a.Y, Z = a.Z;
  const int lx = it.lo[0], hx = it.hi[0];
  const int ny_ = it.hi[1] - it.lo[1], nz_ = it.hi[2] - it.lo[2];
  // x slabs: one cell per thread; y and z slabs: one quad (aligned to 4) per thread
  const int q0 = ax == 0 ? lx : (lx & ~3);
  const int nxq = ax == 0 ? (hx - lx) : ((hx - q0 + 3) >> 2);
  const long long per_b = (long long)nxq * ny_ * nz_;
  const long long total = per_b * a.B;
  const long long sa = ax == 0 ? 1 : (ax == 1 ? (long long)X : (long long)X * Y);
  const bool is_h = a.kind == 1;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(t / per_b);
    long long r = t - (long long)b * per_b;
    const int xq = (int)(r % nxq);
    r /= nxq;
    const int jj = (int)(r % ny_);
    const int kk = (int)(r / ny_);
    const int j = it.lo[1] + jj, k = it.lo[2] + kk;
    const int ia = ax == 1 ? j : k;
    if (ax == 0) {
      const int i = lx + xq;
      const long long q = (long long)k * X * Y + (long long)j * X + i;
      const long long p = (long long)b * a.bs + q;
      const real d = is_h ? (it.S[p + sa] - it.S[p]) * a.inv[i] : (it.S[p] - it.S[p - sa]) * a.inv[i];
      const int w = hx - lx;
      const long long pq = (((long long)b * Z + k) * Y + j) * w + (i - lx);
      real ps = it.psi[pq];
      ps = ps * a.cb_[i];
      ps = ps + a.cc_[i] * d;
      it.psi[pq] = ps;
      const real upd = a.ck_[i] * d + ps;
      if (is_h) {
        it.F[p] = it.F[p] + (it.sign * a.dtmu) * upd;
      } else {
        const int m = a.mat[it.c][q];
        const real tc = (it.sign * a.coef[m].cb) * upd;
        it.F[p] = it.F[p] + tc;
        debye_shift(a, it.c, m, tc, b, k, j, i);
      }
    } else {
      const int i0 = q0 + 4 * xq;
      const long long q = (long long)k * X * Y + (long long)j * X + i0;
      const long long p = (long long)b * a.bs + q;
      const Quad<real> s0 = ld4(it.S + p);
      const Quad<real> s1 = is_h ? ld4(it.S + p + sa) : ld4(it.S + p - sa);
      Quad<real> f = ld4(it.F + p);
      const int w = it.hi[ax] - it.lo[ax];
      const long long pq = ax == 1 ? (((long long)b * Z + k) * w + (j - it.lo[1])) * X + i0
                                   : (((long long)b * w + (k - it.lo[2])) * Y + j) * X + i0;
      Quad<real> ps = ld4(it.psi + pq);
      Quad<uint16_t> m{};
      if (!is_h) m = ld4(a.mat[it.c] + q);
      const real inv = a.inv[ia], pb = a.cb_[ia], pc = a.cc_[ia], pk = a.ck_[ia];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int i = i0 + e;
        if (i < lx || i >= hx) continue;
        const real d = is_h ? (s1.v[e] - s0.v[e]) * inv : (s0.v[e] - s1.v[e]) * inv;
        real v = ps.v[e] * pb;
        v = v + pc * d;
        ps.v[e] = v;
        const real upd = pk * d + v;
        if (is_h) {
          f.v[e] = f.v[e] + (it.sign * a.dtmu) * upd;
        } else {
          const real tc = (it.sign * a.coef[m.v[e]].cb) * upd;
          f.v[e] = f.v[e] + tc;
          debye_shift(a, it.c, m.v[e], tc, b, k, j, i);
        }
      }
      st4(it.psi + pq, ps);
      st4(it.F + p, f);
    }
  }
}

template <typename real>
cudaError_t launch_cpml_pass(const CpmlPass<real>& pass, const SweepArgs<real>& a, int kind, cudaStream_t s) {
  for (int ax = 0; ax < 3; ++ax) {
    const CpmlAxisPass<real>& ap = pass.axis[kind][ax];
    if (ap.n == 0) continue;
    CorrArgs<real> c{};
    c.n_items = ap.n;
    long long most = 0;
    for (int n = 0; n < ap.n; ++n) {
      const CpmlSide<real>& sd = *ap.side[n];
      CorrItem<real>& it = c.item[n];
      const int comp = ap.comp[n], src = ap.src[n];
      it.F = kind == 0 ? a.E[comp] : a.H[comp];
      it.S = kind == 0 ? a.H[src] : a.E[src];
      it.psi = sd.psi;
      it.c = comp;
      it.sign = ap.sign[n];
      for (int d = 0; d < 3; ++d) {
        it.lo[d] = sd.lo[d];
        it.hi[d] = sd.hi[d];
      }
      const int lx = it.lo[0], hx = it.hi[0];
      const int q0 = ax == 0 ? lx : (lx & ~3);
      const long long nxq = ax == 0 ? (hx - lx) : ((hx - q0 + 3) >> 2);
      const long long items = nxq * (it.hi[1] - it.lo[1]) * (it.hi[2] - it.lo[2]) * a.B;
      most = items > most ? items : most;
    }
    c.kind = kind;
    c.axis = ax;
    const real* const* co = kind == 0 ? a.pe[ax] : a.ph[ax];
    c.cb_ = co[0];
    c.cc_ = co[1];
    c.ck_ = co[2];
    c.inv = kind == 0 ? a.idd[ax] : a.ip[ax];
    c.dtmu = a.dtmu;
    for (int d = 0; d < 3; ++d) {
      c.mat[d] = a.mat[d];
      c.J[d] = a.J[d];
      c.jk0[d] = a.jk0[d];
      c.jnk[d] = a.jnk[d];
    }
    c.coef = a.coef;
    c.ade_lo = a.ade_lo;
    c.ade_hi = a.ade_hi;
    c.ade_P = a.ade_P;
    c.ade_beta = a.ade_beta;
    c.X = a.X;
    c.Y = a.Y;
    c.Z = a.nz + 2;
    c.B = a.B;
    c.bs = a.bs;
    long long blocks = (most + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    if (blocks < 1) blocks = 1;
    cpml_pass_kernel<real><<<dim3((unsigned)blocks, ap.n), 256, 0, s>>>(c);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return err;
  }
  return cudaSuccess;
}

template cudaError_t launch_cpml_pass<float>(const CpmlPass<float>&, const SweepArgs<float>&, int, cudaStream_t);
template cudaError_t launch_cpml_pass<double>(const CpmlPass<double>&, const SweepArgs<double>&, int, cudaStream_t);

}  // namespace oafdtd
