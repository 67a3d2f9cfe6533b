// FDTD time-step kernels for sm_103a.
//
// One time step is: h_sweep -> [ghosts] -> [pre_e] -> e_sweep -> [edges] -> [probe_e].
//  * h_sweep, e_sweep: the Yee sweeps with CPML, and Debye ADE fused (sweeps.cu).
//  * ghosts: PMC mirror planes, one launch per wall in wall order.
//  * pre_e: H probe sums + running DFT at (n + 1/2) dt; saves E^n of dispersive edges that also
//    receive injection (their ADE update runs after the injection, in the edge pass).
//  * sibc, edges: surface impedance on its edge list, then injection and the deferred Debye
//    updates on theirs.
//  * probe_e: E probe sums + running DFT at (n + 1) dt.
//
// Arithmetic follows the reference engine (packages/oa-fdtd/src/oa_fdtd/reference.py:115-249)
// operation by operation; the library is built with -fmad=false, so float32 fields agree bit for
// bit with the float32 oracle. Fusing the CPML corrections into the sweeps keeps the reference's
// order (bulk update, then the corrections in ascending derivative axis, each rounded to the field
// precision), so fusion changes no rounding.

#include "oafdtd_internal.cuh"

namespace oafdtd {

// ----------------------------------------------------------------------------- PMC ghosts
// h[dst plane] = -h[src plane] over the whole plane (every storage index of the other axes).
template <typename real>
__global__ void ghost_kernel(real* H0, real* H1, int axis, int dst, int src, int X, int Y, int Z,
                             int B) {
  const int ext[3] = {X, Y, Z};
  const int u_ax = axis == 0 ? 1 : 0;
  const int v_ax = axis == 2 ? 1 : 2;
  const long long nu = ext[u_ax], nv = ext[v_ax];
  const long long total = nu * nv * B;
  const long long st[3] = {1, X, (long long)X * Y};
  const long long bs = (long long)X * Y * Z;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const long long u = t % nu;
    const long long r = t / nu;
    const long long v = r % nv;
    const long long b = r / nv;
    const long long off = b * bs + u * st[u_ax] + v * st[v_ax];
    const long long pd = off + dst * st[axis], ps = off + src * st[axis];
    H0[pd] = -H0[ps];
    H1[pd] = -H1[ps];
  }
}

// ----------------------------------------------------------------------------- probes
// Weighted float64 sum of one probe for one batch member (fixed-order reduction), then the
// running DFT acc[f] += exp(-j w t) dt V with t = (n + offset) dt.
template <typename real>
__device__ void probe_block(const ProbeArgs<real>& a, int pid, int b, long long step, double toff) {
  __shared__ double warp_sum[32];
  const real* F = a.F[(a.kind[pid] == 0 ? 0 : 3) + a.comp[pid]] + (long long)b * a.bs;
  double acc = 0.0;
  for (long long e = a.off[pid] + threadIdx.x; e < a.off[pid + 1]; e += blockDim.x)
    acc += (double)F[a.flat[e]] * a.w[e];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) warp_sum[warp] = acc;
  __syncthreads();
  __shared__ double total;
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += warp_sum[w];
    total = s;
    if (a.series != nullptr) a.series[((long long)pid * a.B + b) * a.max_steps + step] = s;
  }
  __syncthreads();
  const double v = total;
  const double t = ((double)step + toff) * a.dt;
  double2* out = a.acc + ((long long)pid * a.B + b) * a.n_freq;
  for (int f = threadIdx.x; f < a.n_freq; f += blockDim.x) {
    double sn, cs;
    sincos(a.omega[f] * t, &sn, &cs);
    double2 cur = out[f];
    cur.x += (cs * a.dt) * v;
    cur.y += (-(sn * a.dt)) * v;
    out[f] = cur;
  }
}

template <typename real>
__device__ __forceinline__ void pre_e_body(const ProbeArgs<real>& a, int off, int block) {
  const long long step = *a.step_base + off;
  const int nprobe_blocks = a.n_kind[1] * a.B;
  if (block < nprobe_blocks) {
    const int pi = block / a.B, b = block % a.B;
    probe_block(a, a.list[1][pi], b, step, 0.5);
    return;
  }
  const int t = (block - nprobe_blocks) * blockDim.x + threadIdx.x;
  if (t >= a.n_def) return;
  const real* E = a.E[a.def_comp[t]];
  for (int b = 0; b < a.B; ++b) a.eold[(long long)b * a.n_def + t] = E[(long long)b * a.bs + a.def_flat[t]];
}

template <typename real>
__global__ void __launch_bounds__(256) pre_e_kernel(const __grid_constant__ ProbeArgs<real> a, int off) {
  pre_e_body(a, off, (int)blockIdx.x);
}

template <typename real>
__device__ __forceinline__ void probe_e_body(const ProbeArgs<real>& a, int off, int block) {
  const long long step = *a.step_base + off;
  const int pi = block / a.B, b = block % a.B;
  probe_block(a, a.list[0][pi], b, step, 1.0);
}

template <typename real>
__global__ void __launch_bounds__(256) probe_e_kernel(const __grid_constant__ ProbeArgs<real> a, int off) {
  probe_e_body(a, off, (int)blockIdx.x);
}

// Several engines' deferred-E saves and H-probe DFTs, and E-probe DFTs, in one launch each.
template <typename real>
__global__ void __launch_bounds__(256) pre_e_batch_kernel(const ProbeArgs<real>* __restrict__ A, const BatchGrid G,
                                                          int off) {
  __shared__ __align__(16) unsigned char args[sizeof(ProbeArgs<real>)];
  int e;
  const uint3 bid = G.block(&e);
  pre_e_body(stage_args(A + e, args), off, (int)bid.x);
}

template <typename real>
__global__ void __launch_bounds__(256) probe_e_batch_kernel(const ProbeArgs<real>* __restrict__ A, const BatchGrid G,
                                                            int off) {
  __shared__ __align__(16) unsigned char args[sizeof(ProbeArgs<real>)];
  int e;
  const uint3 bid = G.block(&e);
  probe_e_body(stage_args(A + e, args), off, (int)bid.x);
}

// ----------------------------------------------------------------------------- surface impedance
// E_face = r0 J + sum_p v_p, v_p = alpha_p (J - J_prev) + g_p v_p, J = sum of the signed outside
// H samples (reference.py:129-150). One thread per edge handles every batch member; BB and PP
// unroll the batch and pole loops so all loads of an edge are issued together.
template <typename real, int BB, int PP>
__device__ __forceinline__ void sibc_body(const SibcArgs<real>& a, int block, int lo, int hi) {
  const int s = lo + block * (int)blockDim.x + (int)threadIdx.x;
  if (s >= hi) return;
  const SibcEdge<real> ed = a.edge[s];
  const real* __restrict__ alpha = a.alpha + (long long)ed.mat * PP;
  const long long n = a.n;
  // every load of this edge first (the stores below would otherwise order them one by one)
  real vv[BB][PP], hs[BB][2], jp[BB];
#pragma unroll
  for (int b = 0; b < BB; ++b) {
    const long long off = (long long)b * a.bs;
    const long long be = (long long)b * n + s;
    hs[b][0] = ed.sign[0] != (real)0 ? a.H[ed.hcomp0][off + ed.hflat[0]] : (real)0;
    hs[b][1] = ed.sign[1] != (real)0 ? a.H[ed.hcomp1][off + ed.hflat[1]] : (real)0;
    jp[b] = a.jprev[be];
#pragma unroll
    for (int p = 0; p < PP; ++p) vv[b][p] = a.v[((long long)p * BB) * n + be];
  }
  const real r0 = a.r0[ed.mat];
#pragma unroll
  for (int b = 0; b < BB; ++b) {
    real jj = (real)0;
    if (ed.sign[0] != (real)0) jj = jj + ed.sign[0] * hs[b][0];
    if (ed.sign[1] != (real)0) jj = jj + ed.sign[1] * hs[b][1];
    const real dj = jj - jp[b];
    real vsum = (real)0;
#pragma unroll
    for (int p = 0; p < PP; ++p) {
      const real nv = alpha[p] * dj + a.gp[p] * vv[b][p];
      vv[b][p] = nv;
      vsum = p == 0 ? nv : vsum + nv;
    }
    const long long be = (long long)b * n + s;
#pragma unroll
    for (int p = 0; p < PP; ++p) a.v[((long long)p * BB) * n + be] = vv[b][p];
    a.jprev[be] = jj;
    a.E[ed.comp][(long long)b * a.bs + ed.flat] = r0 * jj + vsum;
  }
}

template <typename real, int BB, int PP>
__global__ void __launch_bounds__(128) sibc_kernel(const __grid_constant__ SibcArgs<real> a, int lo, int hi) {
  sibc_body<real, BB, PP>(a, (int)blockIdx.x, lo, hi);
}

// Any batch size and pole count (loops not unrolled).
template <typename real>
__device__ __forceinline__ void sibc_generic_body(const SibcArgs<real>& a, int block, int lo, int hi) {
  const int s = lo + block * (int)blockDim.x + (int)threadIdx.x;
  if (s >= hi) return;
  const SibcEdge<real> ed = a.edge[s];
  const int B = a.B, P = a.P;
  const real* __restrict__ alpha = a.alpha + (long long)ed.mat * P;
  const long long n = a.n;
  for (int b = 0; b < B; ++b) {
    const long long off = (long long)b * a.bs;
    real jj = (real)0;
    if (ed.sign[0] != (real)0) jj = jj + ed.sign[0] * a.H[ed.hcomp0][off + ed.hflat[0]];
    if (ed.sign[1] != (real)0) jj = jj + ed.sign[1] * a.H[ed.hcomp1][off + ed.hflat[1]];
    const long long be = (long long)b * n + s;
    const real dj = jj - a.jprev[be];
    real vsum = (real)0;
    for (int p = 0; p < P; ++p) {
      real* vp = a.v + ((long long)p * B) * n + be;
      const real nv = alpha[p] * dj + a.gp[p] * (*vp);
      *vp = nv;
      vsum = p == 0 ? nv : vsum + nv;
    }
    a.jprev[be] = jj;
    a.E[ed.comp][off + ed.flat] = a.r0[ed.mat] * jj + vsum;
  }
}

template <typename real>
__global__ void __launch_bounds__(128) sibc_generic_kernel(const __grid_constant__ SibcArgs<real> a, int lo, int hi) {
  sibc_generic_body(a, (int)blockIdx.x, lo, hi);
}

// Several engines' surface-impedance updates in one launch (engines of one kernel variant).
template <typename real, int BB, int PP>
__global__ void __launch_bounds__(128) sibc_batch_kernel(const SibcArgs<real>* __restrict__ A, const BatchGrid G) {
  __shared__ __align__(16) unsigned char args[sizeof(SibcArgs<real>)];
  int e;
  const uint3 bid = G.block(&e);
  const SibcArgs<real>& a = stage_args(A + e, args);
  if constexpr (BB == 0)
    sibc_generic_body(a, (int)bid.x, 0, a.n);
  else
    sibc_body<real, BB, PP>(a, (int)bid.x, 0, a.n);
}

template <typename real>
int sibc_variant(const SibcArgs<real>& a) {
  return a.P == 16 && (a.B == 1 || a.B == 2 || a.B == 4) ? a.B : 0;
}

template <typename real>
int sibc_blocks(const SibcArgs<real>& a) {
  return (int)((a.n + 127) / 128);
}

template <typename real>
cudaError_t launch_sibc_batch(const SibcArgs<real>* A, const BatchGrid& G, int blocks, int variant, cudaStream_t s) {
  if (blocks <= 0) return cudaSuccess;
  if (variant == 2)
    sibc_batch_kernel<real, 2, 16><<<blocks, 128, 0, s>>>(A, G);
  else if (variant == 1)
    sibc_batch_kernel<real, 1, 16><<<blocks, 128, 0, s>>>(A, G);
  else if (variant == 4)
    sibc_batch_kernel<real, 4, 16><<<blocks, 128, 0, s>>>(A, G);
  else
    sibc_batch_kernel<real, 0, 16><<<blocks, 128, 0, s>>>(A, G);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_sibc(const SibcArgs<real>& a, cudaStream_t s, int lo, int hi) {
  if (hi < 0) hi = a.n;
  if (hi <= lo) return cudaSuccess;
  const unsigned blocks = (unsigned)((hi - lo + 127) / 128);
  if (a.B == 2 && a.P == 16)
    sibc_kernel<real, 2, 16><<<blocks, 128, 0, s>>>(a, lo, hi);
  else if (a.B == 1 && a.P == 16)
    sibc_kernel<real, 1, 16><<<blocks, 128, 0, s>>>(a, lo, hi);
  else if (a.B == 4 && a.P == 16)
    sibc_kernel<real, 4, 16><<<blocks, 128, 0, s>>>(a, lo, hi);
  else
    sibc_generic_kernel<real><<<blocks, 128, 0, s>>>(a, lo, hi);
  return cudaGetLastError();
}

// ----------------------------------------------------------------------------- injection pass
// Injection (reference.py:223-234) and the Debye update of dispersive edges with injection
// (reference.py:119-127), in the reference's order after the surface impedance.
template <typename real>
__device__ __forceinline__ void edge_body(const EdgeArgs<real>& a, int off, int block) {
  const int e = block * blockDim.x + threadIdx.x;
  if (e >= a.n) return;
  const long long step = *a.step_base + off;
  const int c = a.comp[e];
  const long long f = a.flat[e];
  const int ib = a.inj_beg[e], ie = a.inj_end[e];
  const int ds = a.def_slot[e];
  for (int b = 0; b < a.B; ++b) {
    real* Ec = a.E[c] + (long long)b * a.bs;
    real val = Ec[f];
    for (int t = ib; t < ie; ++t) {
      const int ch = a.i_chan[t];
      const double w = a.wave[(long long)ch * a.max_steps + step];
      val = val + (real)((a.drive[b * a.n_chan + ch] * w) * a.i_amp[t]);
    }
    if (ds >= 0) {
      const long long q = f;
      const int m = a.mat[c][q];
      const int kk = (int)(q / ((long long)a.X * a.Y));
      const long long rem = q - (long long)kk * a.X * a.Y;
      const long long jstride = (long long)a.B * a.jnk[c] * a.Y * a.X;
      const long long jq = ((long long)b * a.jnk[c] + (kk - a.jk0[c])) * a.Y * a.X + rem;
      real* J = a.J[c];
      const int AP = a.ade_P;
      real jt = (real)0;
      for (int p = 0; p < AP; ++p) jt = jt + a.ade_onekp[p] * J[jq + p * jstride];
      jt = (real)0.5 * jt;
      const real en = val - a.coef[m].cbe * jt;
      const real de = en - a.eold[(long long)b * a.n_def + ds];
      for (int p = 0; p < AP; ++p) {
        const long long qq = jq + p * jstride;
        const real beta = p == 0 ? a.coef[m].beta0 : a.ade_beta[(long long)m * AP + p];
        J[qq] = a.ade_kp[p] * J[qq] + beta * de;
      }
      val = en;
    }
    Ec[f] = val;
  }
}

template <typename real>
__global__ void __launch_bounds__(128) edge_kernel(const __grid_constant__ EdgeArgs<real> a, int off) {
  edge_body(a, off, (int)blockIdx.x);
}

// Several engines' injection passes in one launch.
template <typename real>
__global__ void __launch_bounds__(128) edge_batch_kernel(const EdgeArgs<real>* __restrict__ A, const BatchGrid G,
                                                         int off) {
  __shared__ __align__(16) unsigned char args[sizeof(EdgeArgs<real>)];
  int e;
  const uint3 bid = G.block(&e);
  edge_body(stage_args(A + e, args), off, (int)bid.x);
}

// ----------------------------------------------------------------------------- energy
// Float-float arithmetic (a value is hi + lo, two float32 with |lo| <= ulp(hi) / 2): products
// from the float32 multiply and its exact error (one fused multiply-add, written out: the
// library is built without contraction), sums by Knuth's two-sum. About 2^-46 relative error
// per operation.
__device__ __forceinline__ float2 ff_mul(float2 a, float2 b) {
  const float p = a.x * b.x;
  float e = __fmaf_rn(a.x, b.x, -p);
  e = __fmaf_rn(a.x, b.y, e);
  e = __fmaf_rn(a.y, b.x, e);
  const float s = p + e;
  return make_float2(s, e - (s - p));
}
__device__ __forceinline__ float2 ff_add(float2 a, float2 b) {
  const float s = a.x + b.x;
  const float bb = s - a.x;
  const float err = (a.x - (s - bb)) + (b.x - bb);
  const float lo = (err + a.y) + b.y;
  const float h = s + lo;
  return make_float2(h, lo - (h - s));
}

// Energy sums 1/2 sum eps E^2 V (and sum H^2 V) per component, in float64 or, for float32
// fields, in float-float: GB300's float64 rate is a small fraction of its float32 rate, and a
// float64 product chain per cell made this kernel compute-bound (3.3 ms at 400x400x120, batch
// 2; the fields are read in 0.15 ms). A float32 field value squares exactly into a float-float
// pair; the weights come as float-float pairs; the terms of a thread are summed in float-float
// and the thread's sum converted to float64 once. Each term is then exact to about 1e-13 relative,
// so the sum is too (every term is positive). The fields are scaled by 2^32 and the weights by
// 2^40 (exact) so that squares of fields down to 1e-28 and weights down to 1e-30 stay normal;
// the thread's sum is scaled back by 2^-104. Fields above 4e9 would overflow the square.
template <typename real>
__global__ void __launch_bounds__(256) energy_kernel(const __grid_constant__ EnergyArgs<real> a,
                                                     double* partial) {
  __shared__ double warp_sum[8];
  const int cc = blockIdx.y;  // 0..2 E, 3..5 H
  const real* F = a.F[cc];
  const double* wx = a.w[cc][0];
  const double* wy = a.w[cc][1];
  const double* wz = a.w[cc][2];
  const long long rows = (long long)a.B * a.Z * a.Y;
  const long long bs = (long long)a.Z * a.Y * a.X;
  double acc = 0.0;
  if constexpr (sizeof(real) == 4) {
    // one quad (four cells, 16-byte loads) per thread and iteration, quads of consecutive rows
    // on consecutive threads: enough loads in flight to stream the fields
    const float vscale = ldexpf(1.0f, kEnergyVShift);
    const float2* wxf = a.wxf[cc];
    const float2* wyzf = a.wyzf[cc];
    const int Q = a.X / 4;
    const long long quads = rows * Q;
    float2 sum = make_float2(0.0f, 0.0f);
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < quads;
         t += (long long)gridDim.x * blockDim.x) {
      const long long r = t / Q;
      const int i0 = 4 * (int)(t - r * Q);
      const long long plane = r % ((long long)a.Z * a.Y);
      const long long q = r * a.X + i0;
      const float4 f4 = *reinterpret_cast<const float4*>(F + q);
      const float2 wyz = wyzf[plane];
      ushort4 m4 = make_ushort4(0, 0, 0, 0);
      if (cc < 3) m4 = *reinterpret_cast<const ushort4*>(a.mat[cc] + (q % bs));
      const float fv[4] = {f4.x, f4.y, f4.z, f4.w};
      const unsigned short mv[4] = {m4.x, m4.y, m4.z, m4.w};
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float v = fv[e] * vscale;
        const float p = v * v;
        const float2 v2 = make_float2(p, __fmaf_rn(v, v, -p));
        float2 w = ff_mul(wxf[i0 + e], wyz);
        if (cc < 3) w = ff_mul(w, a.epsf[mv[e]]);
        sum = ff_add(sum, ff_mul(w, v2));
      }
    }
    acc = ldexp((double)sum.x + (double)sum.y, -(kEnergyVShift * 2 + kEnergyWShift));
  } else {
    for (long long r = blockIdx.x; r < rows; r += gridDim.x) {
      const long long plane = r % ((long long)a.Z * a.Y);
      const int k = (int)(plane / a.Y), j = (int)(plane % a.Y);
      const double wyz = wy[j] * wz[k];
      const long long row = r * a.X;
      double racc = 0.0;
      for (int i = threadIdx.x; i < a.X; i += blockDim.x) {
        const double v = (double)F[row + i];
        double term = wx[i] * wyz * v * v;
        if (cc < 3) term *= a.eps[a.mat[cc][(row % bs) + i]];
        racc += term;
      }
      acc += racc;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < 8; ++w) s += warp_sum[w];
    partial[(long long)cc * gridDim.x + blockIdx.x] = s;
  }
}

__global__ void energy_final_kernel(const double* partial, int nblocks, double* out) {
  const int cc = threadIdx.x;
  if (cc >= 6) return;
  double s = 0.0;
  for (int k = 0; k < nblocks; ++k) s += partial[(long long)cc * nblocks + k];
  out[cc] = s;
}

__global__ void bump_kernel(long long* step_base, int n) { *step_base += n; }

__global__ void bump_batch_kernel(long long* const* step_base, int n_eng, int n) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n_eng) *step_base[e] += n;
}

// ----------------------------------------------------------------------------- launchers
static inline unsigned ceil_div(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

template <typename real>
cudaError_t launch_ghosts(real* const H[3], int pmc_mask, int nx, int ny, int nz, int X, int Y, int B,
                          cudaStream_t s) {
  const int n[3] = {nx, ny, nz};
  const int Z = nz + 2;
  for (int axis = 0; axis < 3; ++axis) {
    for (int side = 0; side < 2; ++side) {
      if (!(pmc_mask & (1 << (2 * axis + side)))) continue;
      const int dst = side == 0 ? 0 : n[axis] + 1;
      const int src = side == 0 ? 1 : n[axis];
      real* h0 = H[axis == 0 ? 1 : 0];
      real* h1 = H[axis == 2 ? 1 : 2];
      ghost_kernel<real><<<152 * 4, 256, 0, s>>>(h0, h1, axis, dst, src, X, Y, Z, B);
      cudaError_t err = cudaGetLastError();
      if (err != cudaSuccess) return err;
    }
  }
  return cudaSuccess;
}

template <typename real>
int pre_e_blocks(const ProbeArgs<real>& a) {
  return a.n_kind[1] * a.B + (int)ceil_div(a.n_def, 256);
}

template <typename real>
int probe_e_blocks(const ProbeArgs<real>& a) {
  return a.n_kind[0] * a.B;
}

template <typename real>
int edge_blocks(const EdgeArgs<real>& a) {
  return a.n == 0 ? 0 : (int)ceil_div(a.n, 128);
}

template <typename real>
cudaError_t launch_pre_e_batch(const ProbeArgs<real>* A, const BatchGrid& G, int blocks, int off, cudaStream_t s) {
  if (blocks <= 0) return cudaSuccess;
  pre_e_batch_kernel<real><<<blocks, 256, 0, s>>>(A, G, off);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_probe_e_batch(const ProbeArgs<real>* A, const BatchGrid& G, int blocks, int off, cudaStream_t s) {
  if (blocks <= 0) return cudaSuccess;
  probe_e_batch_kernel<real><<<blocks, 256, 0, s>>>(A, G, off);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_edges_batch(const EdgeArgs<real>* A, const BatchGrid& G, int blocks, int off, cudaStream_t s) {
  if (blocks <= 0) return cudaSuccess;
  edge_batch_kernel<real><<<blocks, 128, 0, s>>>(A, G, off);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_pre_e(const ProbeArgs<real>& a, int off, cudaStream_t s) {
  const int blocks = pre_e_blocks(a);
  if (blocks == 0) return cudaSuccess;
  pre_e_kernel<real><<<blocks, 256, 0, s>>>(a, off);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_probe_e(const ProbeArgs<real>& a, int off, cudaStream_t s) {
  const int blocks = a.n_kind[0] * a.B;
  if (blocks == 0) return cudaSuccess;
  probe_e_kernel<real><<<blocks, 256, 0, s>>>(a, off);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_edges(const EdgeArgs<real>& a, int off, cudaStream_t s) {
  if (a.n == 0) return cudaSuccess;
  edge_kernel<real><<<ceil_div(a.n, 128), 128, 0, s>>>(a, off);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_energy(const EnergyArgs<real>& a, double* partial, int nblocks, double* out,
                          cudaStream_t s) {
  energy_kernel<real><<<dim3(nblocks, 6), 256, 0, s>>>(a, partial);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  energy_final_kernel<<<1, 32, 0, s>>>(partial, nblocks, out);
  return cudaGetLastError();
}

cudaError_t launch_bump(long long* step_base, int n, cudaStream_t s) {
  bump_kernel<<<1, 1, 0, s>>>(step_base, n);
  return cudaGetLastError();
}

cudaError_t launch_bump_batch(long long* const* step_base, int n_eng, int n, cudaStream_t s) {
  if (n_eng <= 0) return cudaSuccess;
  bump_batch_kernel<<<(unsigned)ceil_div(n_eng, 128), 128, 0, s>>>(step_base, n_eng, n);
  return cudaGetLastError();
}

#define OAFDTD_INSTANTIATE(real)                                                                   \
  template cudaError_t launch_ghosts<real>(real* const[3], int, int, int, int, int, int, int,      \
                                           cudaStream_t);                                           \
  template cudaError_t launch_pre_e<real>(const ProbeArgs<real>&, int, cudaStream_t);              \
  template cudaError_t launch_probe_e<real>(const ProbeArgs<real>&, int, cudaStream_t);            \
  template cudaError_t launch_edges<real>(const EdgeArgs<real>&, int, cudaStream_t);               \
  template cudaError_t launch_sibc<real>(const SibcArgs<real>&, cudaStream_t, int, int);            \
  template int pre_e_blocks<real>(const ProbeArgs<real>&);                                          \
  template int probe_e_blocks<real>(const ProbeArgs<real>&);                                        \
  template int edge_blocks<real>(const EdgeArgs<real>&);                                            \
  template int sibc_blocks<real>(const SibcArgs<real>&);                                            \
  template int sibc_variant<real>(const SibcArgs<real>&);                                           \
  template cudaError_t launch_pre_e_batch<real>(const ProbeArgs<real>*, const BatchGrid&, int, int, \
                                                cudaStream_t);                                      \
  template cudaError_t launch_probe_e_batch<real>(const ProbeArgs<real>*, const BatchGrid&, int, int, \
                                                  cudaStream_t);                                    \
  template cudaError_t launch_edges_batch<real>(const EdgeArgs<real>*, const BatchGrid&, int, int,  \
                                                cudaStream_t);                                      \
  template cudaError_t launch_sibc_batch<real>(const SibcArgs<real>*, const BatchGrid&, int, int,   \
                                               cudaStream_t);                                       \
  template cudaError_t preload_kernels<real>();                                                     \
  template cudaError_t launch_energy<real>(const EnergyArgs<real>&, double*, int, double*,         \
                                           cudaStream_t);

template <typename real>
cudaError_t preload_kernels() {
  cudaFuncAttributes fa;
  const void* fns[] = {
      reinterpret_cast<const void*>(ghost_kernel<real>),
      reinterpret_cast<const void*>(pre_e_kernel<real>),
      reinterpret_cast<const void*>(probe_e_kernel<real>),
      reinterpret_cast<const void*>(sibc_kernel<real, 2, 16>),
      reinterpret_cast<const void*>(sibc_kernel<real, 1, 16>),
      reinterpret_cast<const void*>(sibc_kernel<real, 4, 16>),
      reinterpret_cast<const void*>(sibc_generic_kernel<real>),
      reinterpret_cast<const void*>(edge_kernel<real>),
      reinterpret_cast<const void*>(energy_kernel<real>),
      reinterpret_cast<const void*>(energy_final_kernel),
      reinterpret_cast<const void*>(bump_kernel),
      reinterpret_cast<const void*>(bump_batch_kernel),
      reinterpret_cast<const void*>(pre_e_batch_kernel<real>),
      reinterpret_cast<const void*>(probe_e_batch_kernel<real>),
      reinterpret_cast<const void*>(sibc_batch_kernel<real, 2, 16>),
      reinterpret_cast<const void*>(sibc_batch_kernel<real, 1, 16>),
      reinterpret_cast<const void*>(sibc_batch_kernel<real, 4, 16>),
      reinterpret_cast<const void*>(sibc_batch_kernel<real, 0, 16>),
      reinterpret_cast<const void*>(edge_batch_kernel<real>),
  };
  for (const void* f : fns) {
    const cudaError_t err = cudaFuncGetAttributes(&fa, f);
    if (err != cudaSuccess) return err;
  }
  return cudaSuccess;
}

OAFDTD_INSTANTIATE(float)
OAFDTD_INSTANTIATE(double)

}  // namespace oafdtd
