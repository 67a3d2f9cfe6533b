// Internal types shared by the engine's host code and its kernels.
//
// Device data layout (HBM):
//  * fields: six arrays E0..E2, H0..H2, each (B, Z, Y, X) with Z = nz + 2, Y = ny + 2, X = pitch;
//    x rows are 128-byte aligned (pitch is a multiple of 32 elements).
//  * mat[c]: uint16 per E edge (Z, Y, X), index into the combined table. The combined table
//    holds, per entry, the update coefficients ca/cb of the averaged material, its permittivity
//    (energy) and, for dispersive edges, the Debye ADE coefficients (cbe, beta_p). Entries are
//    ordered plain, dispersive, dispersive-with-injection, so the kind of an edge follows from
//    its index. It replaces both the reference's material index and its per-edge ADE arrays:
//    the E sweep reads one 2-byte index per edge, shared by every batch member.
//  * psi: one array per CPML correction, (B, Z', Y', X') with the slab width along the
//    derivative axis and the full storage extent along the other two axes, so psi rows of y and z
//    slabs line up with the field rows.
//  * J[c]: dense Debye currents (P, B, nzA, Y, X) over the z range that holds dispersive edges.
//  * edge list (surface impedance, injection, dispersive edges with injection), sorted by
//    (component, flat index), one thread per edge.
#pragma once

#include <cuda.h>  // CUtensorMap (the descriptors are encoded through the runtime's driver entry point)
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

namespace oafdtd {

constexpr int kChunk = 64;        // steps per captured graph (the reference's CHUNK)
constexpr int kMaxAdePoles = 16;  // Debye poles handled by the fused sweep
constexpr int kCoefSmem = 256;    // table entries the fused sweep keeps in shared memory

template <typename real>
struct CpmlSide {
  real* psi;         // nullptr: side absent
  int lo[3], hi[3];  // storage box [lo, hi) per x, y, z
};

template <typename real>
struct CpmlTerm {    // the correction of one (kind, component, derivative axis)
  int axis;
  int src;           // source component of the derivative
  real sign;
  CpmlSide<real> side[2];
};

// A box of the update domain: quads [q0, q1) (x cells 4 q0 .. 4 q1), rows [j0, j1), planes
// [k0, k1).
struct Span3 {
  int q0, q1, j0, j1, k0, k1;
};

// One entry of the combined material table: update coefficients of the averaged material and,
// for dispersive entries, the Debye coefficients (cbe, beta of the first pole).
template <typename real>
struct __align__(4 * sizeof(real)) Coef {
  real ca, cb, cbe, beta0;
};

// Field pointers of a time step. The H sweeps read E (E^n) and H (H^{n-1/2}) and write Ho
// (H^{n+1/2}); the E sweeps read Ho (H^{n+1/2}) and E (E^n) and write Eo (E^{n+1}). In place,
// Eo == E and Ho == H; with two buffers per field (the fused sweep), E and H are the current
// buffers and Eo, Ho the other ones, and the engine swaps them after each step.
template <typename real>
struct SweepArgs {
  real* E[3];
  real* H[3];
  real* Eo[3];
  real* Ho[3];
  const uint16_t* mat[3];
  const Coef<real>* coef;   // [entry]; entries [ade_lo, ade_hi) are dispersive, then deferred ones
  int n_coef;               // entries in the table
  int ade_lo, ade_hi;
  const real* ade_beta;     // [entry * P + p]
  const real* ade_kp;       // [p]
  const real* ade_onekp;    // [p]: 1 + kp in the field precision
  int ade_P;
  real* J[3];
  int jk0[3];
  int jnk[3];
  const real* ip[3];        // inverse primal lengths
  const real* idd[3];       // inverse dual lengths
  const real* pe[3][3];     // per axis: eb, ec, ek
  const real* ph[3][3];     // per axis: hb, hc, hk
  CpmlTerm<real> ecorr[3][2];  // [component][ascending derivative axis]
  CpmlTerm<real> hcorr[3][2];
  int has_cpml;
  real dtmu;
  int nx, ny, nz, X, Y;
  long long bs;             // Z * Y * X
  int B;
  int tile_z;       // planes marched per block by the staged sweeps
  int staged;       // 3: fused H + E sweep of the interior, the rest as 2; 2: staged by TMA
                    // tensor copies; 1: staged by cp.async; 0: slab kernel only
  int* status;      // device status word: bit 0 set when a bounded wait of a sweep gave up
  // Per kind ([0] E, [1] H): the interior box, which holds no CPML correction cell and is swept
  // by the staged kernels; the z-slab planes over the interior's x-y extent ([low, high]), swept
  // by the staged kernels with their z corrections; and up to six disjoint boxes covering the rest
  // of the update domain, marched by the slab kernel (bulk update, corrections, Debye update).
  Span3 inner[2];
  Span3 fused;       // the box both fields of which the fused sweep updates (variant 3)
  Span3 zin[2][2];
  int zsd[2][2][2];  // [kind][low/high][component 0/1]: side of the z-term psi, -1 if none
  Span3 slab[2][6];
  int n_slab[2];
};

// TMA descriptors of the staged sweeps: per component, the field arrays as 4-D tensors
// (x, y, z, batch) with a wide box (132 x 9: the tile plus its one-quad / one-row halo) and a
// tile box (128 x 8), and the material index arrays (x, y, z) with a 128 x 8 box. E wide and
// E tile describe E (the H sweep's source, the E sweep's old values), H tile describes H (the H
// sweep's old values) and H wide describes Ho (the E sweep's source).
struct SweepMaps {
  CUtensorMap e_wide[3], e_tile[3];
  CUtensorMap h_wide[3], h_tile[3];
  CUtensorMap mat[3];
  // z-term psi of the two components that have one (E: Ex, Ey; H: Hx, Hy) as (x, y, z', batch)
  // tensors with a tile box: [kind][component][low/high]
  CUtensorMap psi_z[2][2][2];
};

// TMA descriptors of the fused sweep, on the current buffers: E with a one-quad and one-row halo
// on every side (136 x 10), H with a halo on the low sides (132 x 9), and the material index
// (128 x 8).
struct FusedMaps {
  CUtensorMap e_halo[3];
  CUtensorMap h_halo[3];
  CUtensorMap mat[3];
};

constexpr int kStatusWaitTimeout = 1;

// One surface-impedance edge: the E edge it sets and its two outside H samples (weight 0: unused).
template <typename real>
struct __align__(16) SibcEdge {
  int flat;                  // storage index of the E edge (one batch member)
  int hflat[2];
  int mat;                   // row of the impedance tables
  real sign[2];
  unsigned char comp, hcomp0, hcomp1, pad;
};

template <typename real>
struct SibcArgs {
  real* E[3];
  const real* H[3];
  int n, P;                  // edges, poles
  const SibcEdge<real>* edge;
  const real* r0;            // [m]
  const real* alpha;         // [m * P + p] = rp * cp (rounded once to the field precision)
  const real* gp;            // [p]
  real* jprev;               // (B, n)
  real* v;                   // (P, B, n)
  long long bs;
  int B;
};

// Injection and the Debye update of dispersive edges with injection, after the surface
// impedance pass, on the edges that have either.
template <typename real>
struct EdgeArgs {
  real* E[3];
  const real* H[3];
  int n;                     // edges of this list
  const int8_t* comp;
  const long long* flat;
  const int* inj_beg;
  const int* inj_end;
  const int* def_slot;       // -1: none
  // injection contributions, ordered by edge then channel
  const int* i_chan;
  const double* i_amp;
  const double* wave;        // (n_chan, max_steps)
  const double* drive;       // (B, n_chan)
  int n_chan, max_steps;
  // deferred ADE
  int n_def;
  real* eold;                // (B, n_def)
  const uint16_t* mat[3];
  const Coef<real>* coef;
  const real* ade_beta;
  const real* ade_kp;
  const real* ade_onekp;
  int ade_P;
  real* J[3];
  int jk0[3];
  int jnk[3];
  const long long* def_flat; // (n_def)
  const int8_t* def_comp;
  long long bs;
  int X, Y, B;
  const long long* step_base;
};

template <typename real>
struct ProbeArgs {
  const real* F[6];          // E0..E2, H0..H2
  int n_probe;
  const int* kind;
  const int* comp;
  const long long* off;
  const long long* flat;
  const double* w;
  const int* list[2];        // probe ids of kind E / H
  int n_kind[2];
  int n_freq;
  const double* omega;
  double dt;
  double2* acc;              // (n_probe, B, F)
  double* series;            // (n_probe, B, max_steps) or nullptr
  int max_steps;
  long long bs;
  int B;
  const long long* step_base;
  // deferred-ADE save (in the pre-E launch)
  int n_def;
  real* eold;
  const long long* def_flat;
  const int8_t* def_comp;
  const real* E[3];
};

template <typename real>
struct EnergyArgs {
  const real* F[6];
  const uint16_t* mat[3];
  const double* eps;         // [entry] eps_r * eps0
  const double* w[6][3];     // per component, per axis: node or cell weights
  int X, Y, Z, B;
  // float32 fields: the same weights as float-float pairs (hi, lo), the y-z product per plane and
  // row pre-multiplied by 2^kEnergyWShift (kept clear of float32 underflow)
  const float2* wxf[6];      // [i]
  const float2* wyzf[6];     // [k * Y + j]
  const float2* epsf;        // [entry]
};
constexpr int kEnergyWShift = 40;  // weights scaled by 2^40 ...
constexpr int kEnergyVShift = 32;  // ... and fields by 2^32 (squares by 2^64) in the float-float sum

// Launch geometry of the slab kernel: the boxes of one kind with their first block.
struct SlabLaunch {
  Span3 box[6];
  int n;
  int first[7];  // first block of each box; first[n] = total blocks
  int cblk[6];   // column blocks per (box, chunk, member)
  int nch[6];    // z chunks per box
};

// The blocks of one launch that covers several engines (a batched sweep): block b of the launch
// is block (x, y, z) = (blk[b].y, blk[b].z, blk[b].w) of engine blk[b].x in that engine's own
// grid (one 16-byte load per block). The per-engine arguments sit in device arrays indexed by
// the engine.
struct BatchGrid {
  const int4* blk;
#ifdef __CUDACC__
  __device__ __forceinline__ uint3 block(int* e) const {
    const int4 t = __ldg(blk + blockIdx.x);
    *e = t.x;
    return make_uint3((unsigned)t.y, (unsigned)t.z, (unsigned)t.w);
  }
#endif
};

#ifdef __CUDACC__
// A batched kernel's arguments of this block's engine, copied once per block from device memory
// into shared memory (buf: sizeof(T) bytes, 16-byte aligned), so that the kernel body reads them
// as cheaply as launch parameters instead of holding them in registers.
template <typename T>
__device__ __forceinline__ const T& stage_args(const T* __restrict__ src, unsigned char* buf) {
  static_assert(sizeof(T) % 4 == 0, "argument blocks are whole words");
  const int* s = reinterpret_cast<const int*>(src);
  int* d = reinterpret_cast<int*>(buf);
  const int tid = (int)(threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z));
  const int nt = (int)(blockDim.x * blockDim.y * blockDim.z);
  for (int i = tid; i < (int)(sizeof(T) / 4); i += nt) d[i] = __ldg(s + i);
  __syncthreads();
  return *reinterpret_cast<const T*>(buf);
}
#endif

// Per-engine launch grids of the step's kernel classes (the single launchers use the same), and
// the batched launchers: one launch of a class over the blocks of every engine in G, the
// arguments of engine e at A[e] (and M[e], L[e]) in device memory. A grid with no blocks is empty.
template <typename real>
cudaError_t fused_grid(const SweepArgs<real>& a, dim3* grid);
template <typename real>
cudaError_t staged_grids(const SweepArgs<real>& a, int kind, dim3* inner, dim3* z);
template <typename real>
cudaError_t slab_plan(const SweepArgs<real>& a, int kind, SlabLaunch* L, long long* blocks);
template <typename real>
int pre_e_blocks(const ProbeArgs<real>& a);
template <typename real>
int probe_e_blocks(const ProbeArgs<real>& a);
template <typename real>
int edge_blocks(const EdgeArgs<real>& a);
template <typename real>
int sibc_blocks(const SibcArgs<real>& a);
// the SIBC kernel variant of an engine: 0 generic, else the unrolled batch size (poles 16)
template <typename real>
int sibc_variant(const SibcArgs<real>& a);
template <typename real>
cudaError_t launch_fused_batch(const SweepArgs<real>* A, const FusedMaps* M, const BatchGrid& G, int blocks,
                               bool multi_pole, cudaStream_t s);
template <typename real>
cudaError_t launch_staged_batch(const SweepArgs<real>* A, const SweepMaps* M, const BatchGrid& G, int blocks, bool h,
                                bool tma, bool z, bool multi_pole, cudaStream_t s);
template <typename real>
cudaError_t launch_slab_batch(const SweepArgs<real>* A, const SlabLaunch* L, const BatchGrid& G, int blocks, int kind,
                              bool multi_pole, cudaStream_t s);
template <typename real>
cudaError_t launch_pre_e_batch(const ProbeArgs<real>* A, const BatchGrid& G, int blocks, int off, cudaStream_t s);
template <typename real>
cudaError_t launch_probe_e_batch(const ProbeArgs<real>* A, const BatchGrid& G, int blocks, int off, cudaStream_t s);
template <typename real>
cudaError_t launch_edges_batch(const EdgeArgs<real>* A, const BatchGrid& G, int blocks, int off, cudaStream_t s);
template <typename real>
cudaError_t launch_sibc_batch(const SibcArgs<real>* A, const BatchGrid& G, int blocks, int variant, cudaStream_t s);
// step_base[e] += n for the n_eng engines' device step counters (an array of device pointers)
cudaError_t launch_bump_batch(long long* const* step_base, int n_eng, int n, cudaStream_t s);

// kernel launchers (kernels.cu)
template <typename real>
cudaError_t launch_h_sweep(const SweepArgs<real>& a, const SweepMaps& m, cudaStream_t s);
template <typename real>
cudaError_t launch_e_sweep(const SweepArgs<real>& a, const SweepMaps& m, cudaStream_t s);
template <typename real>
cudaError_t launch_slab(const SweepArgs<real>& a, int kind, cudaStream_t s);
template <typename real>
cudaError_t launch_ghosts(real* const H[3], int pmc_mask, int nx, int ny, int nz, int X, int Y, int B,
                          cudaStream_t s);
template <typename real>
cudaError_t launch_pre_e(const ProbeArgs<real>& a, int off, cudaStream_t s);
template <typename real>
cudaError_t launch_edges(const EdgeArgs<real>& a, int off, cudaStream_t s);
// the surface-impedance edges [lo, hi) (hi < 0: to the last)
template <typename real>
cudaError_t launch_sibc(const SibcArgs<real>& a, cudaStream_t s, int lo = 0, int hi = -1);
template <typename real>
cudaError_t launch_probe_e(const ProbeArgs<real>& a, int off, cudaStream_t s);
template <typename real>
cudaError_t launch_energy(const EnergyArgs<real>& a, double* partial, int nblocks, double* out,
                          cudaStream_t s);
cudaError_t launch_bump(long long* step_base, int n, cudaStream_t s);
template <typename real>
cudaError_t launch_staged_sweep(const SweepArgs<real>& a, const SweepMaps& m, cudaStream_t s, bool h);
// The fused H + E sweep of a.fused (variant 3, two buffers per field).
template <typename real>
cudaError_t launch_fused_sweep(const SweepArgs<real>& a, const FusedMaps& m, cudaStream_t s);
template <typename real>
bool encode_fused_maps(const SweepArgs<real>& a, FusedMaps* m, std::string* why);
template <typename real>
cudaError_t preload_fused();
// One tiled TMA descriptor (dims and box innermost first, strides in bytes of dims 1..rank-1,
// no interleave or swizzle, zero fill); false with a message when the driver's encoder is missing
// or rejects it.
bool encode_tensor_map(CUtensorMap* m, CUtensorMapDataType dt, int rank, const void* base, const cuuint64_t* dims,
                       const cuuint64_t* strides, const cuuint32_t* box, const char* what, std::string* why,
                       CUtensorMapSwizzle swizzle = CU_TENSOR_MAP_SWIZZLE_NONE);
// The tcgen05 GEMM of the surrogate (umma.cu), grouped: C_g = A_g . B_g^T for row-major A_g
// (M x K) and B_g (N x K), g < groups, each operand's groups a fixed number of elements apart.
struct UmmaProblem {
  const void* A;
  const void* B;
  float* C32;          // FP32 result (nullable), ldc
  void* C16;           // BF16 result (nullable), ldc
  void* C16T;          // BF16 result transposed, N x M (nullable), ldct
  const float* bias;   // per column (nullable)
  const void* mask;    // epilogues 2 and 4: BF16 in the layout of C
  int M, N, K, lda, ldb, ldc, ldct, act, groups;
  long long sA, sB, sC, sCT, sBias;  // elements between consecutive groups
  float beta;
  int* status;         // set nonzero when a bounded wait gave up (nullable)
};
// Whether a problem suits the kernel: M a multiple of 128, N of 64, K of 64; leading dimensions
// and group strides multiples of 8 elements; 16-byte aligned operands; beta 0.
bool umma_shape_ok(const UmmaProblem& p);
cudaError_t launch_umma_gemm(const UmmaProblem& p, cudaStream_t s, std::string* why);
cudaError_t preload_umma();
// Encodes the TMA descriptors of the staged sweeps for the fields and indices in a; false (with
// a message) when the driver entry point is missing or rejects a descriptor.
template <typename real>
bool encode_sweep_maps(const SweepArgs<real>& a, SweepMaps* m, std::string* why);

// Loads every kernel of one precision on the current device now (cudaFuncGetAttributes), so
// that no kernel is loaded lazily at its first launch: a lazy load synchronises the device and
// would serialise engines that run side by side on their own streams.
template <typename real>
cudaError_t preload_kernels();
template <typename real>
cudaError_t preload_staged();
template <typename real>
cudaError_t preload_slab();

// Message returned by oafdtd_last_error() on the calling thread.
void set_last_error(const std::string& msg);

constexpr int kEnergyBlocks = 1216;  // 8 per SM on a 152-SM GB300; fixed for a deterministic sum

}  // namespace oafdtd
