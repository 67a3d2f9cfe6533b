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
  int X, Y, Z, B;
  long long bs;
};

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
      const real kf = is_h ? a.dtmu : a.coef[a.mat[it.c][q]].cb;
      it.F[p] = it.F[p] + (it.sign * kf) * upd;
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
        const real kf = is_h ? a.dtmu : a.coef[m.v[e]].cb;
        f.v[e] = f.v[e] + (it.sign * kf) * upd;
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
    for (int d = 0; d < 3; ++d) c.mat[d] = a.mat[d];
    c.coef = a.coef;
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
