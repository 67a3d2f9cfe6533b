// The fused sweep (variant 3): H^{n+1/2} and E^{n+1} of the interior in one z-march per block.
//
// The separate sweeps move 72 bytes per cell and member and time step: the H sweep reads E and
// reads and writes H, the E sweep reads H and reads and writes E. This sweep reads E^n and
// H^{n-1/2} once and writes H^{n+1/2} and E^{n+1} once: 48 bytes. It needs two buffers per field.
// A block's E update at its tile edge needs H^{n+1/2} one cell outside the tile (x - 1, y - 1),
// which the block recomputes from E^n and H^{n-1/2}; with one buffer the neighbouring block could
// already have overwritten those with E^{n+1} and H^{n+1/2}. So every block reads the current
// buffers, which nothing writes during the step, and writes the other ones; the engine swaps them
// after each step. The same holds in z: a block's first plane needs H^{n+1/2} of the plane below,
// which it recomputes (for its own cells) before it starts.
//
// A block owns a tile of 32 quads (128 x cells) by 8 rows and a chunk of z planes. Per plane it
// stages, by TMA tensor copies into shared memory: E^n of the plane above (with a one-quad and
// one-row halo on every side; the plane itself is still staged from the previous step of the
// march), H^{n-1/2} of the plane (with a halo on the low sides) and the material index. Each warp
// waits for the copies itself; one block barrier per plane (after the H update) also agrees on
// whether every wait succeeded, and the warps release their slots through an mbarrier that the
// leader waits on before it refills them. It then
//   1. updates H of its cells (and of the halo column x0 - 1 and row y0 - 1) in shared memory,
//      with the H sweep's arithmetic (packages/oa-fdtd/src/oa_fdtd/reference.py:152-165);
//   2. updates E of its cells from the new H (and the carried H of the plane below), with the
//      bulk and Debye arithmetic of the E sweep (reference.py:167-180, :119-127);
//   3. writes H^{n+1/2} and E^{n+1} of its cells to the other buffers.
// The fused box holds no CPML correction cell of either field, its halo cells hold none of H and
// are not ghosts, so every cell gets exactly the arithmetic the separate sweeps give it, bit for
// bit. The z-slab planes and the x/y slabs around the box are swept by the staged and slab
// kernels, out of place as well; the engine runs the H part of those beside this kernel and the E
// part after it.
//
// Every mbarrier wait is bounded: a block whose copies do not arrive sets bit 0 of the status
// word, waits (bounded again) for the copies it issued and returns; the host reports
// OAFDTD_E_TIMEOUT.

#include "tma.cuh"

namespace oafdtd {

namespace {

constexpr int kFQ = 32;            // quads per tile row
constexpr int kFY = 8;             // rows per tile
constexpr int kFW = 4 * kFQ;       // tile width in cells (128)
constexpr int kEW = kFW + 8;       // staged E width: one quad each side (136)
constexpr int kEH = kFY + 2;       // staged E rows: one each side (10)
constexpr int kHW = kFW + 4;       // staged H width: one quad on the low side (132)
constexpr int kHH = kFY + 1;       // staged H rows: one on the low side (9)
constexpr int kSE = 3;             // E slots: the plane, the one above, one in flight
constexpr int kSH = 2;             // H + index slots: the plane, one in flight

template <typename real>
struct EPlane {
  Box<real, kEH, kEW> e[3];
};
template <typename real>
struct HPlane {
  Box<real, kHH, kHW> h[3];
  Box<uint16_t, kFY, kFW> m[3];
};
template <typename real>
struct FusedSmem {
  EPlane<real> e[kSE];
  HPlane<real> h[kSH];
  Coef<real> coef[kCoefSmem];  // the combined material table (the E update's 12 gathers per quad)
};

template <typename real>
__device__ __forceinline__ void issue_e(const FusedMaps& tm, EPlane<real>& s, unsigned long long* bar, int x0, int y0,
                                        int k, int b) {
  mbar_expect_tx(bar, 3u * kEH * kEW * sizeof(real));
#pragma unroll
  for (int c = 0; c < 3; ++c) tma_load4(&s.e[c], &tm.e_halo[c], bar, x0 - 4, y0 - 1, k, b);
}

template <typename real>
__device__ __forceinline__ void issue_h(const FusedMaps& tm, HPlane<real>& s, unsigned long long* bar, int x0, int y0,
                                        int k, int b) {
  mbar_expect_tx(bar, 3u * (kHH * kHW * sizeof(real) + kFY * kFW * sizeof(uint16_t)));
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    tma_load4(&s.h[c], &tm.h_halo[c], bar, x0 - 4, y0 - 1, k, b);
    tma_load3(&s.m[c], &tm.mat[c], bar, x0, y0, k);
  }
}

// A wait gave up: the leader records it and waits (bounded) for every copy it issued that has not
// been seen to arrive, so no copy lands after the block has exited.
__device__ __noinline__ void abort_fused(unsigned long long* bar_e, unsigned long long* bar_h, int e_seen, int e_issued,
                                         int h_seen, int h_issued, int* status, bool leader) {
  if (!leader) return;
  if (status) atomicOr(status, kStatusWaitTimeout);
  for (int u = e_seen; u < e_issued; ++u) mbar_wait(&bar_e[u % kSE], (unsigned)((u / kSE) & 1), kDrainNs);
  for (int u = h_seen; u < h_issued; ++u) mbar_wait(&bar_h[u % kSH], (unsigned)((u / kSH) & 1), kDrainNs);
}

// The sweep of block bid of the fused box (a plain launch passes blockIdx; a batched one the
// block of its engine).
template <typename real, bool kMulti>
__device__ __forceinline__ void fused_body(const SweepArgs<real>& a, const FusedMaps& tm, const uint3 bid) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ unsigned long long bar_e[kSE], bar_h[kSH];
  __shared__ unsigned long long bar_done;  // one arrival per warp when it is done with a plane
  FusedSmem<real>& sm = *reinterpret_cast<FusedSmem<real>*>(align_smem(smem_raw));
  const int tx = threadIdx.x, ty = threadIdx.y;
  const bool leader = tx == 0 && ty == 0;
  const Span3 F = a.fused;
  const int nx = a.nx, ny = a.ny, nz = a.nz, X = a.X, Y = a.Y;
  const int nkc = (F.k1 - F.k0 + a.tile_z - 1) / a.tile_z;
  const int b = (int)bid.z / nkc;
  const int kc0 = F.k0 + ((int)bid.z % nkc) * a.tile_z;
  const int kc1 = min(kc0 + a.tile_z, F.k1);
  const int x0 = 4 * (F.q0 + (int)bid.x * kFQ);
  const int y0 = F.j0 + (int)bid.y * kFY;
  if (kc1 <= kc0 || x0 >= 4 * F.q1 || y0 >= F.j1) return;
  const int ks = kc0 - 1;            // the plane below the chunk: H only, for the carry
  const int n_planes = kc1 - ks;     // planes of the march, ks .. kc1 - 1
  const int n_e = n_planes + 1;      // E planes staged, ks .. kc1 (kc1 <= nz + 1 < Z)
  const int i0 = x0 + 4 * tx, j = y0 + ty;
  const bool live = i0 < 4 * F.q1 && j < F.j1;
  const long long base = (long long)b * a.bs;
  const real dtmu = a.dtmu;
  const Quad<real> ipx = i0 < X ? ld4(a.ip[0] + i0) : Quad<real>{};
  const Quad<real> idx4 = i0 < X ? ld4(a.idd[0] + i0) : Quad<real>{};
  const real ipy = a.ip[1][min(j, Y - 1)];
  const real idy = a.idd[1][min(j, Y - 1)];
  const real ipy_h = a.ip[1][y0 - 1];  // the halo row
  const real ipx_h = a.ip[0][x0 - 1];  // the halo column
  const int cc = 4 + 4 * tx;           // own first cell in the staged E and H rows
  // the halo row's cells, 128 of them: lanes 0-15 of every warp, cell hc of the tile row
  const int hc = 16 * ty + tx;
  const bool halo_live = tx < 16 && x0 + 4 * (hc / 4) < 4 * F.q1;
  const real ipx_c = halo_live ? a.ip[0][x0 + hc] : (real)0;
  if (leader) {
#pragma unroll
    for (int s = 0; s < kSE; ++s) mbar_init(&bar_e[s], 1);
#pragma unroll
    for (int s = 0; s < kSH; ++s) mbar_init(&bar_h[s], 1);
    mbar_init(&bar_done, kFY);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      prefetch_map(&tm.e_halo[c]);
      prefetch_map(&tm.h_halo[c]);
      prefetch_map(&tm.mat[c]);
    }
  }
  for (int e = ty * kFQ + tx; e < a.n_coef; e += kFQ * kFY) sm.coef[e] = a.coef[e];
  __syncthreads();
  int e_issued = 0, h_issued = 0;
  if (leader) {
    for (; e_issued < kSE && e_issued < n_e; ++e_issued)
      issue_e(tm, sm.e[e_issued], &bar_e[e_issued], x0, y0, ks + e_issued, b);
    for (; h_issued < kSH && h_issued < n_planes; ++h_issued)
      issue_h(tm, sm.h[h_issued], &bar_h[h_issued], x0, y0, ks + h_issued, b);
  }
  // E(ks) first; each step of the march then waits for the plane above and its own H and index
  bool ok = mbar_wait(&bar_e[0], 0u, kWaitNs);
  if (__syncthreads_or(!ok)) {
    abort_fused(bar_e, bar_h, 0, e_issued, 0, h_issued, a.status, leader);
    return;
  }
  Quad<real> hx_m{}, hy_m{};  // H^{n+1/2} of the plane below at the own cells, carried
  Quad<real> jcur[3], jnext[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) jcur[c] = Quad<real>{};
  if (live && a.ade_P == 1) {
#pragma unroll
    for (int c = 0; c < 3; ++c)
      if (kc0 >= a.jk0[c] && kc0 < a.jk0[c] + a.jnk[c])
        jcur[c] = ld4(a.J[c] + (((long long)b * a.jnk[c] + (kc0 - a.jk0[c])) * Y + j) * X + i0);
  }
  for (int t = 0; t < n_planes; ++t) {
    const int k = ks + t;
    const bool inner = k >= kc0;  // a plane of the fused box (else the carry plane below it)
#pragma unroll
    for (int c = 0; c < 3; ++c) jnext[c] = Quad<real>{};
    if (inner && live && a.ade_P == 1 && k + 1 < kc1) {
#pragma unroll
      for (int c = 0; c < 3; ++c)
        if (k + 1 >= a.jk0[c] && k + 1 < a.jk0[c] + a.jnk[c])
          jnext[c] = ld4(a.J[c] + (((long long)b * a.jnk[c] + (k + 1 - a.jk0[c])) * Y + j) * X + i0);
    }
    // each thread acquires the plane's copies itself; whether every wait succeeded is agreed on
    // at the block's one barrier of the plane, before any global store
    ok = ok && mbar_wait(&bar_e[(t + 1) % kSE], (unsigned)(((t + 1) / kSE) & 1), kWaitNs);
    if (ok) ok = mbar_wait(&bar_h[t % kSH], (unsigned)((t / kSH) & 1), kWaitNs);
    const EPlane<real>& ec = sm.e[t % kSE];         // E^n of plane k
    const EPlane<real>& en = sm.e[(t + 1) % kSE];   // E^n of plane k + 1
    HPlane<real>& hs = sm.h[t % kSH];               // H^{n-1/2} of plane k, updated in place
    const bool kin = k <= nz;
    const real ipz = a.ip[2][k];
    // ---- 1. H^{n+1/2} of the own quad (the H sweep's arithmetic), kept in shared memory
    Quad<real> hx_n{}, hy_n{}, hz_n{};
    if (live) {
      const Quad<real> ex = ld4(&ec.e[0].v[ty + 1][cc]), ey = ld4(&ec.e[1].v[ty + 1][cc]);
      const Quad<real> ez = ld4(&ec.e[2].v[ty + 1][cc]);
      const real ez_r = ec.e[2].v[ty + 1][cc + 4], ey_r = ec.e[1].v[ty + 1][cc + 4];
      hx_n = ld4(&hs.h[0].v[ty + 1][cc]);
      hy_n = ld4(&hs.h[1].v[ty + 1][cc]);
      hz_n = ld4(&hs.h[2].v[ty + 1][cc]);
      if (j <= ny && kin) {  // Hx: node along x (1..nx+1), cell along y and z
        const Quad<real> ezy = ld4(&ec.e[2].v[ty + 2][cc]);
        const Quad<real> ey1 = ld4(&en.e[1].v[ty + 1][cc]);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int i = i0 + e;
          const real d0 = (ezy.v[e] - ez.v[e]) * ipy;  // axis y
          const real d1 = (ey1.v[e] - ey.v[e]) * ipz;  // axis z
          if (i >= 1 && i <= nx + 1) hx_n.v[e] = hx_n.v[e] + dtmu * ((-d0) + d1);
        }
      }
      if (kin) {  // Hy: cell along x (1..nx), node along y, cell along z
        const Quad<real> ex1 = ld4(&en.e[0].v[ty + 1][cc]);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int i = i0 + e;
          const real ezr = e < 3 ? ez.v[e + 1] : ez_r;
          const real d0 = (ezr - ez.v[e]) * ipx.v[e];  // axis x
          const real d1 = (ex1.v[e] - ex.v[e]) * ipz;  // axis z
          if (i >= 1 && i <= nx) hy_n.v[e] = hy_n.v[e] + dtmu * ((-d1) + d0);
        }
      }
      if (j <= ny) {  // Hz: cell along x and y, node along z
        const Quad<real> exy = ld4(&ec.e[0].v[ty + 2][cc]);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int i = i0 + e;
          const real eyr = e < 3 ? ey.v[e + 1] : ey_r;
          const real d0 = (eyr - ey.v[e]) * ipx.v[e];  // axis x
          const real d1 = (exy.v[e] - ex.v[e]) * ipy;  // axis y
          if (i >= 1 && i <= nx) hz_n.v[e] = hz_n.v[e] + dtmu * ((-d0) + d1);
        }
      }
      if (inner) {
        st4(&hs.h[0].v[ty + 1][cc], hx_n);
        st4(&hs.h[1].v[ty + 1][cc], hy_n);
        st4(&hs.h[2].v[ty + 1][cc], hz_n);
      }
    }
    if (inner && halo_live) {  // the halo row y0 - 1: Hx and Hz, one cell per lane, every warp a share
      const int jh = y0 - 1, i = x0 + hc, ch = 4 + hc;
      real hx = hs.h[0].v[0][ch], hz = hs.h[2].v[0][ch];
      const real ex = ec.e[0].v[0][ch], ey = ec.e[1].v[0][ch], ez = ec.e[2].v[0][ch];
      const real ezy = ec.e[2].v[1][ch], exy = ec.e[0].v[1][ch];
      const real ey1 = en.e[1].v[0][ch], eyr = ec.e[1].v[0][ch + 1];
      if (jh <= ny && kin) {
        const real d0 = (ezy - ez) * ipy_h;
        const real d1 = (ey1 - ey) * ipz;
        if (i >= 1 && i <= nx + 1) hx = hx + dtmu * ((-d0) + d1);
      }
      if (jh <= ny) {
        const real d0 = (eyr - ey) * ipx_c;
        const real d1 = (exy - ex) * ipy_h;
        if (i >= 1 && i <= nx) hz = hz + dtmu * ((-d0) + d1);
      }
      hs.h[0].v[0][ch] = hx;
      hs.h[2].v[0][ch] = hz;
    }
    if (inner && live && tx == 0) {  // the halo column x0 - 1: Hy and Hz
      const int ih = x0 - 1;
      real hy = hs.h[1].v[ty + 1][3], hz = hs.h[2].v[ty + 1][3];
      if (kin && ih >= 1 && ih <= nx) {
        const real d0 = (ec.e[2].v[ty + 1][4] - ec.e[2].v[ty + 1][3]) * ipx_h;
        const real d1 = (en.e[0].v[ty + 1][3] - ec.e[0].v[ty + 1][3]) * ipz;
        hy = hy + dtmu * ((-d1) + d0);
      }
      if (j <= ny && ih >= 1 && ih <= nx) {
        const real d0 = (ec.e[1].v[ty + 1][4] - ec.e[1].v[ty + 1][3]) * ipx_h;
        const real d1 = (ec.e[0].v[ty + 2][3] - ec.e[0].v[ty + 1][3]) * ipy;
        hz = hz + dtmu * ((-d0) + d1);
      }
      hs.h[1].v[ty + 1][3] = hy;
      hs.h[2].v[ty + 1][3] = hz;
    }
    // the new H of the plane (halo included) is complete
    if (__syncthreads_or(!ok)) {
      abort_fused(bar_e, bar_h, t + 1, e_issued, t, h_issued, a.status, leader);
      return;
    }
    // ---- 2. E^{n+1} of the own quad, and the stores
    if (inner && live) {
      const long long p = base + (long long)k * X * Y + (long long)j * X + i0;
      const long long q = (long long)k * X * Y + (long long)j * X + i0;
      const real idz = a.idd[2][k];
      const Quad<real> hzy = ld4(&hs.h[2].v[ty][cc]), hxy = ld4(&hs.h[0].v[ty][cc]);
      const real hz_l = hs.h[2].v[ty + 1][cc - 1], hy_l = hs.h[1].v[ty + 1][cc - 1];
      ZTerm<real> none;
      none.on = false;
      real d0[4], d1[4];
      // Ex: terms (a = y, +Hz) then (a = z, -Hy)
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        d0[e] = (hz_n.v[e] - hzy.v[e]) * idy;
        d1[e] = (hy_n.v[e] - hy_m.v[e]) * idz;
      }
      e_apply<real, false, kMulti>(a, 0, a.Eo[0] + base, q, ld4(&ec.e[0].v[ty + 1][cc]), &hs.m[0].v[ty][4 * tx], d0,
                                   d1, true, jcur[0], none, i0, j, k, b, sm.coef);
      // Ey: terms (a = z, +Hx) then (a = x, -Hz)
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const real hzl = e > 0 ? hz_n.v[e - 1] : hz_l;
        d0[e] = (hz_n.v[e] - hzl) * idx4.v[e];
        d1[e] = (hx_n.v[e] - hx_m.v[e]) * idz;
      }
      e_apply<real, false, kMulti>(a, 1, a.Eo[1] + base, q, ld4(&ec.e[1].v[ty + 1][cc]), &hs.m[1].v[ty][4 * tx], d0,
                                   d1, false, jcur[1], none, i0, j, k, b, sm.coef);
      // Ez: terms (a = x, +Hy) then (a = y, -Hx)
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const real hyl = e > 0 ? hy_n.v[e - 1] : hy_l;
        d0[e] = (hy_n.v[e] - hyl) * idx4.v[e];
        d1[e] = (hx_n.v[e] - hxy.v[e]) * idy;
      }
      e_apply<real, false, kMulti>(a, 2, a.Eo[2] + base, q, ld4(&ec.e[2].v[ty + 1][cc]), &hs.m[2].v[ty][4 * tx], d0,
                                   d1, true, jcur[2], none, i0, j, k, b, sm.coef);
      if (j <= ny && kin) st4(a.Ho[0] + p, hx_n);
      if (kin) st4(a.Ho[1] + p, hy_n);
      if (j <= ny) st4(a.Ho[2] + p, hz_n);
    }
    hx_m = hx_n;
    hy_m = hy_n;
    if (inner) {  // the carry plane keeps the currents of the chunk's first plane
#pragma unroll
      for (int c = 0; c < 3; ++c) jcur[c] = jnext[c];
    }
    // This warp is done with E(k) and the H / index slot of plane k: its reads and writes of
    // the slots are ordered before the copies that refill them, and the warp moves on to the
    // next plane without waiting for the others. The leader refills the slots once every warp
    // has arrived (phase t of bar_done; phase t + 1 cannot complete before the leader has passed
    // the next plane's barrier).
    fence_proxy_async();
    __syncwarp();
    if (tx == 0) mbar_arrive(&bar_done);
    if (leader && ok && (e_issued < n_e || h_issued < n_planes)) {
      // a wait that gives up is reported at the next plane's barrier; nothing more is issued
      ok = mbar_wait(&bar_done, (unsigned)(t & 1), kWaitNs);
      if (ok && e_issued < n_e) {  // E(k + 3) into the slot of E(k)
        issue_e(tm, sm.e[e_issued % kSE], &bar_e[e_issued % kSE], x0, y0, ks + e_issued, b);
        ++e_issued;
      }
      if (ok && h_issued < n_planes) {  // H and index of plane k + 2 into the slot of plane k
        issue_h(tm, sm.h[h_issued % kSH], &bar_h[h_issued % kSH], x0, y0, ks + h_issued, b);
        ++h_issued;
      }
    }
  }
}

template <typename real, bool kMulti>
__global__ void __launch_bounds__(256, 2)
    fused_kernel(const __grid_constant__ SweepArgs<real> a, const __grid_constant__ FusedMaps tm) {
  fused_body<real, kMulti>(a, tm, blockIdx);
}

// Several engines' fused sweeps in one launch: engine e's arguments at A[e] and M[e].
template <typename real, bool kMulti>
__global__ void __launch_bounds__(256, 2)
    fused_batch_kernel(const SweepArgs<real>* __restrict__ A, const FusedMaps* __restrict__ M, const BatchGrid G) {
  __shared__ __align__(16) unsigned char args[sizeof(SweepArgs<real>)];
  int e;
  const uint3 bid = G.block(&e);
  fused_body<real, kMulti>(stage_args(A + e, args), M[e], bid);
}

}  // namespace

template <typename real>
cudaError_t fused_grid(const SweepArgs<real>& a, dim3* grid) {
  const Span3 F = a.fused;
  *grid = dim3(0, 0, 0);
  if (F.q1 <= F.q0 || F.j1 <= F.j0 || F.k1 <= F.k0) return cudaSuccess;
  if (F.q0 % 2 != 0 || F.q0 < 2 || F.j0 < 2 || F.k0 < 2 || F.k1 > a.nz + 1) return cudaErrorInvalidValue;
  const int nkc = (F.k1 - F.k0 + a.tile_z - 1) / a.tile_z;
  *grid = dim3((F.q1 - F.q0 + kFQ - 1) / kFQ, (F.j1 - F.j0 + kFY - 1) / kFY, nkc * a.B);
  return cudaSuccess;
}

template <typename real>
cudaError_t launch_fused_batch(const SweepArgs<real>* A, const FusedMaps* M, const BatchGrid& G, int blocks,
                               bool multi_pole, cudaStream_t s) {
  if (blocks <= 0) return cudaSuccess;
  const size_t bytes = sizeof(FusedSmem<real>) + 128;
  auto kern = multi_pole ? fused_batch_kernel<real, true> : fused_batch_kernel<real, false>;
  const cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (err != cudaSuccess) return err;
  kern<<<blocks, dim3(kFQ, kFY), bytes, s>>>(A, M, G);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_fused_sweep(const SweepArgs<real>& a, const FusedMaps& m, cudaStream_t s) {
  dim3 grid;
  if (const cudaError_t e = fused_grid(a, &grid)) return e;
  if (grid.x == 0) return cudaSuccess;
  const dim3 block(kFQ, kFY);
  const size_t bytes = sizeof(FusedSmem<real>) + 128;
  auto kern = a.ade_P > 1 ? fused_kernel<real, true> : fused_kernel<real, false>;
  const cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (err != cudaSuccess) return err;
  kern<<<grid, block, bytes, s>>>(a, m);
  return cudaGetLastError();
}

template <typename real>
bool encode_fused_maps(const SweepArgs<real>& a, FusedMaps* m, std::string* why) {
  const CUtensorMapDataType dt = sizeof(real) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
  const cuuint64_t X = (cuuint64_t)a.X, Y = (cuuint64_t)a.Y, Z = (cuuint64_t)a.nz + 2, B = (cuuint64_t)a.B;
  const cuuint64_t dims[4] = {X, Y, Z, B};
  const cuuint64_t rs = sizeof(real);
  const cuuint64_t strides[3] = {X * rs, X * Y * rs, X * Y * Z * rs};
  const cuuint32_t ebox[4] = {kEW, kEH, 1, 1};
  const cuuint32_t hbox[4] = {kHW, kHH, 1, 1};
  const cuuint32_t mbox[3] = {kFW, kFY, 1};
  const cuuint64_t mdims[3] = {X, Y, Z};
  const cuuint64_t mstrides[2] = {X * 2, X * Y * 2};
  for (int c = 0; c < 3; ++c) {
    if (!encode_tensor_map(&m->e_halo[c], dt, 4, a.E[c], dims, strides, ebox, "E halo", why) ||
        !encode_tensor_map(&m->h_halo[c], dt, 4, a.H[c], dims, strides, hbox, "H halo", why) ||
        !encode_tensor_map(&m->mat[c], CU_TENSOR_MAP_DATA_TYPE_UINT16, 3, a.mat[c], mdims, mstrides, mbox, "mat",
                           why))
      return false;
  }
  return true;
}

template <typename real>
cudaError_t preload_fused() {
  cudaFuncAttributes fa;
  const void* fns[] = {reinterpret_cast<const void*>(fused_kernel<real, false>),
                       reinterpret_cast<const void*>(fused_kernel<real, true>),
                       reinterpret_cast<const void*>(fused_batch_kernel<real, false>),
                       reinterpret_cast<const void*>(fused_batch_kernel<real, true>)};
  for (const void* f : fns) {
    const cudaError_t err = cudaFuncGetAttributes(&fa, f);
    if (err != cudaSuccess) return err;
  }
  return cudaSuccess;
}

static_assert((kEW * sizeof(float)) % 16 == 0 && (kHW * sizeof(float)) % 16 == 0 && (kFW * sizeof(uint16_t)) % 16 == 0,
              "TMA box rows are whole 16-byte units");
static_assert(sizeof(FusedSmem<float>) + 128 <= 113 * 1024, "two fused blocks per SM in float32");
static_assert(sizeof(FusedSmem<double>) + 128 <= 227 * 1024, "one fused block per SM in float64");

template cudaError_t fused_grid<float>(const SweepArgs<float>&, dim3*);
template cudaError_t fused_grid<double>(const SweepArgs<double>&, dim3*);
template cudaError_t launch_fused_batch<float>(const SweepArgs<float>*, const FusedMaps*, const BatchGrid&, int, bool,
                                               cudaStream_t);
template cudaError_t launch_fused_batch<double>(const SweepArgs<double>*, const FusedMaps*, const BatchGrid&, int,
                                                bool, cudaStream_t);
template cudaError_t launch_fused_sweep<float>(const SweepArgs<float>&, const FusedMaps&, cudaStream_t);
template cudaError_t launch_fused_sweep<double>(const SweepArgs<double>&, const FusedMaps&, cudaStream_t);
template bool encode_fused_maps<float>(const SweepArgs<float>&, FusedMaps*, std::string*);
template bool encode_fused_maps<double>(const SweepArgs<double>&, FusedMaps*, std::string*);
template cudaError_t preload_fused<float>();
template cudaError_t preload_fused<double>();

}  // namespace oafdtd
