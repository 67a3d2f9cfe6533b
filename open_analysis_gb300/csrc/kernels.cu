// FDTD time-step kernels for sm_103a.
//
// One time step is: h_sweep -> [ghosts] -> [pre_e] -> e_sweep -> [edges] -> [probe_e].
//  * h_sweep: H update with every CPML-H correction fused, one thread per (i, j) column marching
//    up a z chunk; E at k + 1 is carried in registers to the next plane.
//  * e_sweep: E update from the combined material index, CPML-E corrections and the Debye ADE
//    update fused (E^n stays in a register); H at k - 1 is carried.
//  * ghosts: PMC mirror planes, one launch per wall in wall order.
//  * pre_e: H probe sums + running DFT at (n + 1/2) dt; saves E^n of dispersive edges that also
//    receive injection (their ADE update runs after the injection, in the edge pass).
//  * edges: surface impedance, injection and the deferred ADE updates on the edge list.
//  * probe_e: E probe sums + running DFT at (n + 1) dt.
//
// Arithmetic follows the reference engine (packages/oa-fdtd/src/oa_fdtd/reference.py:115-249)
// operation by operation; the library is built with -fmad=false, so float32 fields agree bit for
// bit with the float32 oracle. Fusing the CPML corrections into the sweeps keeps the reference's
// order (bulk update, then the corrections in ascending derivative axis, each rounded to the field
// precision), so fusion changes no rounding.

#include "oafdtd_internal.cuh"

namespace oafdtd {

template <typename real>
__device__ __forceinline__ void apply_cpml(real& f, const CpmlTerm<real>& t, int i, int j, int k, int b,
                                           real d, real kfac, const real* cb_, const real* cc_,
                                           const real* ck_) {
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const CpmlSide<real>& sd = t.side[s];
    if (sd.psi == nullptr) continue;
    if (i < sd.lo[0] || i >= sd.hi[0] || j < sd.lo[1] || j >= sd.hi[1] || k < sd.lo[2] ||
        k >= sd.hi[2])
      continue;
    const int ia = t.axis == 0 ? i : (t.axis == 1 ? j : k);
    const int ni = sd.hi[0] - sd.lo[0], nj = sd.hi[1] - sd.lo[1], nk = sd.hi[2] - sd.lo[2];
    const long long q =
        (((long long)b * nk + (k - sd.lo[2])) * nj + (j - sd.lo[1])) * (long long)ni + (i - sd.lo[0]);
    real ps = sd.psi[q];
    ps = ps * cb_[ia];
    ps = ps + cc_[ia] * d;
    sd.psi[q] = ps;
    const real upd = ck_[ia] * d + ps;
    f = f + (t.sign * kfac) * upd;
  }
}

// ----------------------------------------------------------------------------- H sweep
template <typename real>
__global__ void __launch_bounds__(256) h_sweep_kernel(const __grid_constant__ SweepArgs<real> a) {
  const int i = blockIdx.x * 32 + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int b = blockIdx.z % a.B;
  const int kc = blockIdx.z / a.B;
  const int nx = a.nx, ny = a.ny, nz = a.nz;
  if (i < 1 || i > nx + 1 || j > ny + 1) return;
  const int k0 = 1 + kc * a.tile_z;
  const int k1 = min(k0 + a.tile_z, nz + 2);
  const long long sy = a.X, sz = (long long)a.X * a.Y;
  const long long base = (long long)b * a.bs;
  const real* __restrict__ Ex = a.E[0] + base;
  const real* __restrict__ Ey = a.E[1] + base;
  const real* __restrict__ Ez = a.E[2] + base;
  real* __restrict__ Hx = a.H[0] + base;
  real* __restrict__ Hy = a.H[1] + base;
  real* __restrict__ Hz = a.H[2] + base;
  const real ipx = a.ip[0][i], ipy = a.ip[1][j];
  const real dtmu = a.dtmu;
  long long p = (long long)k0 * sz + (long long)j * sy + i;
  real ex_c = Ex[p], ey_c = Ey[p];
  for (int k = k0; k < k1; ++k, p += sz) {
    const bool kin = k <= nz;
    const real ex_n = kin ? Ex[p + sz] : (real)0;
    const real ey_n = kin ? Ey[p + sz] : (real)0;
    const real ez = Ez[p];
    const real ipz = a.ip[2][k];
    if (j <= ny && kin) {  // Hx: node along x, cell along y and z
      const real dy = (Ez[p + sy] - ez) * ipy;
      const real dz = (ey_n - ey_c) * ipz;
      const real acc = (-dy) + dz;
      real h = Hx[p] + dtmu * acc;
      if (a.has_cpml) {
        apply_cpml(h, a.hcorr[0][0], i, j, k, b, dy, dtmu, a.ph[1][0], a.ph[1][1], a.ph[1][2]);
        apply_cpml(h, a.hcorr[0][1], i, j, k, b, dz, dtmu, a.ph[2][0], a.ph[2][1], a.ph[2][2]);
      }
      Hx[p] = h;
    }
    if (i <= nx && kin) {  // Hy
      const real dz = (ex_n - ex_c) * ipz;
      const real dx = (Ez[p + 1] - ez) * ipx;
      const real acc = (-dz) + dx;
      real h = Hy[p] + dtmu * acc;
      if (a.has_cpml) {
        apply_cpml(h, a.hcorr[1][0], i, j, k, b, dx, dtmu, a.ph[0][0], a.ph[0][1], a.ph[0][2]);
        apply_cpml(h, a.hcorr[1][1], i, j, k, b, dz, dtmu, a.ph[2][0], a.ph[2][1], a.ph[2][2]);
      }
      Hy[p] = h;
    }
    if (i <= nx && j <= ny) {  // Hz: node along z (k up to nz + 1)
      const real dx = (Ey[p + 1] - ey_c) * ipx;
      const real dy = (Ex[p + sy] - ex_c) * ipy;
      const real acc = (-dx) + dy;
      real h = Hz[p] + dtmu * acc;
      if (a.has_cpml) {
        apply_cpml(h, a.hcorr[2][0], i, j, k, b, dx, dtmu, a.ph[0][0], a.ph[0][1], a.ph[0][2]);
        apply_cpml(h, a.hcorr[2][1], i, j, k, b, dy, dtmu, a.ph[1][0], a.ph[1][1], a.ph[1][2]);
      }
      Hz[p] = h;
    }
    ex_c = ex_n;
    ey_c = ey_n;
  }
}

// ----------------------------------------------------------------------------- E sweep
template <typename real>
__device__ __forceinline__ real ade_update(real e, real e0, const SweepArgs<real>& a, int c, int m,
                                           long long jq, long long jstride) {
  // jt = 1/2 sum_p (1 + k_p) J_p ; E^{n+1} = e - cbe jt ; J_p = k_p J_p + beta_p (E^{n+1} - E^n)
  real* J = a.J[c];
  const int P = a.ade_P;
  real jt = (real)0;
  for (int p = 0; p < P; ++p) jt = jt + a.ade_onekp[p] * J[jq + p * jstride];
  jt = (real)0.5 * jt;
  const real en = e - a.ade_cbe[m] * jt;
  const real de = en - e0;
  for (int p = 0; p < P; ++p) {
    const long long q = jq + p * jstride;
    J[q] = a.ade_kp[p] * J[q] + a.ade_beta[m * P + p] * de;
  }
  return en;
}

template <typename real>
__global__ void __launch_bounds__(256) e_sweep_kernel(const __grid_constant__ SweepArgs<real> a) {
  const int i = blockIdx.x * 32 + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int b = blockIdx.z % a.B;
  const int kc = blockIdx.z / a.B;
  const int nx = a.nx, ny = a.ny, nz = a.nz;
  if (i < 1 || i > nx + 1 || j > ny + 1) return;
  const int k0 = 1 + kc * a.tile_z;
  const int k1 = min(k0 + a.tile_z, nz + 2);
  const long long sy = a.X, sz = (long long)a.X * a.Y;
  const long long base = (long long)b * a.bs;
  real* __restrict__ Ex = a.E[0] + base;
  real* __restrict__ Ey = a.E[1] + base;
  real* __restrict__ Ez = a.E[2] + base;
  const real* __restrict__ Hx = a.H[0] + base;
  const real* __restrict__ Hy = a.H[1] + base;
  const real* __restrict__ Hz = a.H[2] + base;
  const real idx_ = a.idd[0][i], idy = a.idd[1][j];
  long long q = (long long)k0 * sz + (long long)j * sy + i;  // in-plane (batch-free) index
  real hx_m = Hx[q - sz], hy_m = Hy[q - sz];
  for (int k = k0; k < k1; ++k, q += sz) {
    const real hx = Hx[q], hy = Hy[q], hz = Hz[q];
    const real idz = a.idd[2][k];
    {  // Ex
      const real dy = (hz - Hz[q - sy]) * idy;
      const real dz = (hy - hy_m) * idz;
      const real acc = dy + (-dz);
      const int m = a.mat[0][q];
      const real e0 = Ex[q];
      const real cbm = a.cb[m];
      real e = a.ca[m] * e0 + cbm * acc;
      if (a.has_cpml) {
        apply_cpml(e, a.ecorr[0][0], i, j, k, b, dy, cbm, a.pe[1][0], a.pe[1][1], a.pe[1][2]);
        apply_cpml(e, a.ecorr[0][1], i, j, k, b, dz, cbm, a.pe[2][0], a.pe[2][1], a.pe[2][2]);
      }
      if (a.flag[m] == kFlagAde)
        e = ade_update(e, e0, a, 0, m,
                       (((long long)b * a.jnk[0] + (k - a.jk0[0])) * a.Y + j) * a.X + i,
                       (long long)a.B * a.jnk[0] * a.Y * a.X);
      Ex[q] = e;
    }
    {  // Ey
      const real dz = (hx - hx_m) * idz;
      const real dx = (hz - Hz[q - 1]) * idx_;
      const real acc = dz + (-dx);
      const int m = a.mat[1][q];
      const real e0 = Ey[q];
      const real cbm = a.cb[m];
      real e = a.ca[m] * e0 + cbm * acc;
      if (a.has_cpml) {
        apply_cpml(e, a.ecorr[1][0], i, j, k, b, dx, cbm, a.pe[0][0], a.pe[0][1], a.pe[0][2]);
        apply_cpml(e, a.ecorr[1][1], i, j, k, b, dz, cbm, a.pe[2][0], a.pe[2][1], a.pe[2][2]);
      }
      if (a.flag[m] == kFlagAde)
        e = ade_update(e, e0, a, 1, m,
                       (((long long)b * a.jnk[1] + (k - a.jk0[1])) * a.Y + j) * a.X + i,
                       (long long)a.B * a.jnk[1] * a.Y * a.X);
      Ey[q] = e;
    }
    {  // Ez
      const real dx = (hy - Hy[q - 1]) * idx_;
      const real dy = (hx - Hx[q - sy]) * idy;
      const real acc = dx + (-dy);
      const int m = a.mat[2][q];
      const real e0 = Ez[q];
      const real cbm = a.cb[m];
      real e = a.ca[m] * e0 + cbm * acc;
      if (a.has_cpml) {
        apply_cpml(e, a.ecorr[2][0], i, j, k, b, dx, cbm, a.pe[0][0], a.pe[0][1], a.pe[0][2]);
        apply_cpml(e, a.ecorr[2][1], i, j, k, b, dy, cbm, a.pe[1][0], a.pe[1][1], a.pe[1][2]);
      }
      if (a.flag[m] == kFlagAde)
        e = ade_update(e, e0, a, 2, m,
                       (((long long)b * a.jnk[2] + (k - a.jk0[2])) * a.Y + j) * a.X + i,
                       (long long)a.B * a.jnk[2] * a.Y * a.X);
      Ez[q] = e;
    }
    hx_m = hx;
    hy_m = hy;
  }
}

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
__global__ void __launch_bounds__(256) pre_e_kernel(const __grid_constant__ ProbeArgs<real> a, int off) {
  const long long step = *a.step_base + off;
  const int nprobe_blocks = a.n_kind[1] * a.B;
  if ((int)blockIdx.x < nprobe_blocks) {
    const int pi = blockIdx.x / a.B, b = blockIdx.x % a.B;
    probe_block(a, a.list[1][pi], b, step, 0.5);
    return;
  }
  const int t = (blockIdx.x - nprobe_blocks) * blockDim.x + threadIdx.x;
  if (t >= a.n_def) return;
  const real* E = a.E[a.def_comp[t]];
  for (int b = 0; b < a.B; ++b) a.eold[(long long)b * a.n_def + t] = E[(long long)b * a.bs + a.def_flat[t]];
}

template <typename real>
__global__ void __launch_bounds__(256) probe_e_kernel(const __grid_constant__ ProbeArgs<real> a, int off) {
  const long long step = *a.step_base + off;
  const int pi = blockIdx.x / a.B, b = blockIdx.x % a.B;
  probe_block(a, a.list[0][pi], b, step, 1.0);
}

// ----------------------------------------------------------------------------- edge pass
template <typename real>
__global__ void __launch_bounds__(128) edge_kernel(const __grid_constant__ EdgeArgs<real> a, int off) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a.n) return;
  const long long step = *a.step_base + off;
  const int c = a.comp[e];
  const long long f = a.flat[e];
  const int ss = a.sibc_slot[e];
  const int ib = a.inj_beg[e], ie = a.inj_end[e];
  const int ds = a.def_slot[e];
  const int ns = a.sibc_n, P = a.sibc_P;
  for (int b = 0; b < a.B; ++b) {
    real* Ec = a.E[c] + (long long)b * a.bs;
    real val = Ec[f];
    if (ss >= 0) {
      // J = sum of the signed outside H samples; v_p = alpha_p (J - J_prev) + g_p v_p;
      // E = r0 J + sum_p v_p  (reference.py:129-150)
      real jj = (real)0;
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        const real sg = a.s_hsign[2 * ss + s];
        if (sg != (real)0)
          jj = jj + sg * a.H[a.s_hcomp[2 * ss + s]][(long long)b * a.bs + a.s_hflat[2 * ss + s]];
      }
      const int m = a.s_mat[ss];
      const long long be = (long long)b * ns + ss;
      const real dj = jj - a.s_jprev[be];
      real vsum = (real)0;
      for (int p = 0; p < P; ++p) {
        real* vp = a.s_v + (long long)p * a.B * ns + be;
        const real nv = a.s_alpha[m * P + p] * dj + a.s_gp[p] * (*vp);
        *vp = nv;
        vsum = p == 0 ? nv : vsum + nv;
      }
      a.s_jprev[be] = jj;
      val = a.s_r0[m] * jj + vsum;
    }
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
      const real en = val - a.ade_cbe[m] * jt;
      const real de = en - a.eold[(long long)b * a.n_def + ds];
      for (int p = 0; p < AP; ++p) {
        const long long qq = jq + p * jstride;
        J[qq] = a.ade_kp[p] * J[qq] + a.ade_beta[m * AP + p] * de;
      }
      val = en;
    }
    Ec[f] = val;
  }
}

// ----------------------------------------------------------------------------- energy
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

// ----------------------------------------------------------------------------- launchers
static inline unsigned ceil_div(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

template <typename real>
cudaError_t launch_h_sweep(const SweepArgs<real>& a, int tile_y, cudaStream_t s) {
  const int nkc = (a.nz + 1 + a.tile_z - 1) / a.tile_z;
  dim3 block(32, tile_y);
  dim3 grid(ceil_div(a.nx + 2, 32), ceil_div(a.ny + 1, tile_y), nkc * a.B);
  h_sweep_kernel<real><<<grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_e_sweep(const SweepArgs<real>& a, int tile_y, cudaStream_t s) {
  const int nkc = (a.nz + 1 + a.tile_z - 1) / a.tile_z;
  dim3 block(32, tile_y);
  dim3 grid(ceil_div(a.nx + 2, 32), ceil_div(a.ny + 1, tile_y), nkc * a.B);
  e_sweep_kernel<real><<<grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

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
cudaError_t launch_pre_e(const ProbeArgs<real>& a, int off, cudaStream_t s) {
  const int blocks = a.n_kind[1] * a.B + (int)ceil_div(a.n_def, 256);
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

#define OAFDTD_INSTANTIATE(real)                                                                   \
  template cudaError_t launch_h_sweep<real>(const SweepArgs<real>&, int, cudaStream_t);            \
  template cudaError_t launch_e_sweep<real>(const SweepArgs<real>&, int, cudaStream_t);            \
  template cudaError_t launch_ghosts<real>(real* const[3], int, int, int, int, int, int, int,      \
                                           cudaStream_t);                                           \
  template cudaError_t launch_pre_e<real>(const ProbeArgs<real>&, int, cudaStream_t);              \
  template cudaError_t launch_probe_e<real>(const ProbeArgs<real>&, int, cudaStream_t);            \
  template cudaError_t launch_edges<real>(const EdgeArgs<real>&, int, cudaStream_t);               \
  template cudaError_t launch_energy<real>(const EnergyArgs<real>&, double*, int, double*,         \
                                           cudaStream_t);

OAFDTD_INSTANTIATE(float)
OAFDTD_INSTANTIATE(double)

}  // namespace oafdtd
