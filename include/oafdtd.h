/*
 * oafdtd — GB300 (sm_103a) FDTD time-stepping engine, C ABI.
 *
 * This is the drop-in boundary for the engine layer of the oa-fdtd solver. The reference engine
 * is a Python class driven by the run loop (packages/oa-fdtd/src/oa_fdtd/run.py:46-137):
 * CupyEngine (packages/oa-fdtd/src/oa_fdtd/engine.py:67-506) and NumpyEngine
 * (packages/oa-fdtd/src/oa_fdtd/reference.py:41-331). Both consume a compiled problem
 * (`Compiled`, packages/oa-fdtd/src/oa_fdtd/model.py:246-269) and expose
 * step / energy / results / series / get_fields / peak_bytes. Each function below replaces one
 * of those methods; the comment on each names the reference method.
 *
 * Conventions
 *  - Plain C types and host pointers only. The caller owns every host buffer for the duration of
 *    a call; the library copies what it needs and owns all device memory of a handle.
 *  - Every function returns an int status: OAFDTD_OK (0) or a negative OAFDTD_E_* code.
 *    oafdtd_last_error() returns a message for the last failure on the calling thread.
 *  - One handle = one CUDA stream on the device that was current at creation. Calls on one handle
 *    are not re-entrant; different handles may be used from different threads.
 *  - oafdtd_step() returns after the stream has synchronised, as the reference engine's step()
 *    does (engine.py:437).
 *  - Storage layout of every field component: (batch, nz + 2, ny + 2, pitch), x fastest,
 *    storage index = cell/node index + 1, ghost planes at 0 and n + 1 (oa_fdtd/grid.py:1-10).
 */
#ifndef OAFDTD_H
#define OAFDTD_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OAFDTD_ABI_VERSION 1

enum {
  OAFDTD_OK = 0,
  OAFDTD_E_INVALID = -1,      /* bad descriptor or argument (ModelError analogue) */
  OAFDTD_E_OOM = -2,          /* device allocation failed (ACCEL_OUT_OF_MEMORY analogue) */
  OAFDTD_E_CUDA = -3,         /* a CUDA runtime call failed */
  OAFDTD_E_RANGE = -4,        /* step past max_steps (the wave table length) */
  OAFDTD_E_TABLE = -5,        /* more than 65535 combined material entries */
  OAFDTD_E_NODEVICE = -6,     /* no CUDA device */
  OAFDTD_E_TIMEOUT = -7       /* a bounded device-side wait gave up */
};

/* One CPML curl-term correction (oa_fdtd/pml.py:56-70): kind 0 = E, 1 = H; corrected component
 * c, derivative (slab) axis a, source component b, sign, storage box [lo, hi) per x, y, z. */
typedef struct oafdtd_correction {
  int32_t kind, c, a, b;
  double sign;
  int32_t lo[3], hi[3];
} oafdtd_correction;

/* A compiled problem (oa_fdtd/model.py:246-269), flattened to plain arrays. */
typedef struct oafdtd_problem {
  int32_t abi_version;   /* OAFDTD_ABI_VERSION */
  int32_t real_bytes;    /* 4: float32 fields (the production mode), 8: float64 */
  int32_t nx, ny, nz;    /* cells per axis */
  int32_t pitch;         /* padded storage x extent */
  int32_t batch;         /* excitations advanced together */
  double dt;             /* time step [s] */
  double dtmu;           /* dt / mu0 */
  /* materials: per-E-component uint16 index into the averaged-material table (0 = PEC) */
  const uint16_t* idx[3];          /* each (nz+2)*(ny+2)*pitch */
  int32_t n_mat;
  const double* ca_tab;            /* n_mat */
  const double* cb_tab;            /* n_mat */
  const double* eps_tab;           /* n_mat, relative permittivity (energy only) */
  /* 1-D metrics over the storage index of each axis (length pitch, ny+2, nz+2) */
  const double* inv_primal[3];
  const double* inv_dual[3];
  const double* node_w[3];
  const double* cell_w[3];
  int32_t pmc_mask;                /* bit (2*axis + side) set for a PMC wall */
  /* CPML */
  int32_t n_corr;
  const oafdtd_correction* corr;   /* n_corr, in application order */
  const double* pml[3][6];         /* per axis: eb, ec, ek, hb, hc, hk (NULL: no CPML on axis) */
  /* sources: every (channel, edge) contribution in channel order */
  int32_t n_chan;
  int32_t max_steps;
  const double* wave;              /* (n_chan, max_steps): s((n + 1/2) dt) */
  const double* drive;             /* (batch, n_chan) */
  int64_t n_inj;
  const int32_t* inj_comp;
  const int64_t* inj_flat;
  const double* inj_amp;
  const int32_t* inj_chan;
  /* probes: kind 0 = E, 1 = H */
  int32_t n_probe;
  const int32_t* probe_kind;
  const int32_t* probe_comp;
  const int64_t* probe_off;        /* n_probe + 1 */
  const int64_t* probe_flat;
  const double* probe_w;
  int32_t n_freq;
  const double* omega;             /* 2 pi f */
  int32_t record_series;
  /* Debye ADE (oa_fdtd/model.py:218-226) */
  int32_t ade_poles;
  const double* ade_kp;            /* ade_poles */
  int64_t ade_n[3];                /* dispersive edges per component (0: none) */
  const int64_t* ade_flat[3];
  const double* ade_beta[3];       /* (ade_poles, ade_n[c]) */
  const double* ade_cbe[3];        /* ade_n[c] */
  /* surface impedance (oa_fdtd/model.py:230-242) */
  int64_t sibc_n;
  int32_t sibc_poles;
  int32_t sibc_nmat;
  const int32_t* sibc_comp;
  const int64_t* sibc_flat;
  const int32_t* sibc_hcomp;       /* (sibc_n, 2) */
  const int64_t* sibc_hflat;       /* (sibc_n, 2) */
  const double* sibc_hsign;        /* (sibc_n, 2) */
  const int32_t* sibc_mat;
  const double* sibc_r0;           /* sibc_nmat */
  const double* sibc_rp;           /* (sibc_nmat, sibc_poles) */
  const double* sibc_cp;           /* sibc_poles */
  const double* sibc_gp;           /* sibc_poles */
} oafdtd_problem;

typedef struct oafdtd_engine oafdtd_engine;
typedef struct oafdtd_batch oafdtd_batch;

/* Library ABI version (OAFDTD_ABI_VERSION). */
int32_t oafdtd_abi_version(void);

/* Message of the last failure on this thread ("" when none). */
const char* oafdtd_last_error(void);

/* Number of CUDA devices visible (0 when none); never fails. */
int32_t oafdtd_device_count(void);

/* Make `device` the current CUDA device of the calling thread for this library (the device
 * oafdtd_create builds on). One process per GPU calls it with its local rank. */
int oafdtd_set_device(int32_t device);

/* Name, compute capability and memory of the current device (the oa_accel AccelReport fields
 * that CupyEngine's backend fills, packages/oa-accel/src/oa_accel/report.py:13-34, and the free
 * memory that MemoryBudget.require checks against, packages/oa-accel/src/oa_accel/memory.py:82). */
int oafdtd_device_info(char* name, int32_t name_len, int32_t* cc_major, int32_t* cc_minor,
                       int64_t* free_bytes, int64_t* total_bytes, int32_t* runtime_version);

/* Build an engine on the current device: replaces CupyEngine.__init__ (engine.py:73-119), which
 * copies the Compiled arrays to the device, builds the edge lists and allocates psi/J/v state. */
int oafdtd_create(const oafdtd_problem* problem, oafdtd_engine** out);

/* Release every device resource of the handle. Replaces dropping the CupyEngine object. */
int oafdtd_destroy(oafdtd_engine* engine);

/* Advance n time steps: replaces CupyEngine.step (engine.py:418-437). Full 64-step chunks replay
 * a captured CUDA graph (use_graph != 0, set by oafdtd_set_graph). OAFDTD_E_RANGE when the total
 * would pass max_steps (the reference raises ValueError there). */
int oafdtd_step(oafdtd_engine* engine, int64_t n);

/* oafdtd_step with the elapsed device time of its launches (CUDA events recorded on the
 * handle's stream before the first and after the last launch) written to *device_ms. */
int oafdtd_step_timed(oafdtd_engine* engine, int64_t n, double* device_ms);

/* Steps taken so far. */
int oafdtd_step_count(const oafdtd_engine* engine, int64_t* out);

/* Field energy 1/2 sum eps E^2 V + 1/2 mu0 sum H^2 V in float64: replaces CupyEngine.energy
 * (engine.py:440-468). */
int oafdtd_energy(oafdtd_engine* engine, double* out);

/* Probe DFT accumulators: replaces CupyEngine.results (engine.py:486-494). Writes
 * n_probe * batch * n_freq complex values as interleaved (re, im) doubles, probe-major, in the
 * order of the problem's probe list. */
int oafdtd_dft(oafdtd_engine* engine, double* out_re_im);

/* Recorded probe samples (record_series != 0): replaces CupyEngine.series (engine.py:496-503).
 * Writes n_probe * batch * steps doubles, probe-major, step fastest. */
int oafdtd_series(oafdtd_engine* engine, double* out);

/* One field component as float64, shape (batch, nz+2, ny+2, pitch): comp 0..2 = Ex..Ez,
 * 3..5 = Hx..Hz. Replaces CupyEngine.get_fields (engine.py:478-484). */
int oafdtd_fields(oafdtd_engine* engine, int32_t comp, double* out);

/* Snapshot of the run's whole device state (fields, CPML psi, Debye currents, SIBC state,
 * deferred E^n, DFT accumulators, recorded series, step counter) into a host buffer of
 * oafdtd_snapshot_bytes bytes; oafdtd_restore puts it back into a handle of the same problem and
 * configuration (OAFDTD_E_INVALID otherwise), so a run can be bisected or resumed. The reference
 * engine has no counterpart. */
int oafdtd_snapshot_bytes(oafdtd_engine* engine, int64_t* out);
int oafdtd_snapshot(oafdtd_engine* engine, void* out);
int oafdtd_restore(oafdtd_engine* engine, const void* in);

/* Queues n steps on the handle's stream and returns without waiting (oafdtd_step is this and
 * oafdtd_wait); oafdtd_wait synchronises and reports errors, including a bounded wait that gave
 * up (OAFDTD_E_TIMEOUT). Several handles on one device then run side by side (a batched sweep
 * of independent instances). Checks as oafdtd_step. No counterpart in the reference engine. */
int oafdtd_step_async(oafdtd_engine* engine, int64_t n);
int oafdtd_wait(oafdtd_engine* engine);

/* A batched sweep: n engines of one precision, device and sweep variant, at the same step, stepped
 * together. Every kernel class of a time step is then one launch over the blocks of all n engines
 * (the same kernel bodies on each engine's own arguments, so each engine's fields, DFTs and
 * S-parameters are bit for bit those of stepping it alone); whole 64-step chunks replay one
 * captured graph for the whole batch. The engines stay owned by the caller and must outlive the
 * batch; while it exists they are stepped through it only (OAFDTD_E_INVALID otherwise), and
 * their observables (oafdtd_dft, oafdtd_energy, ...) stay available, ordered after the batch's
 * work. oafdtd_batch_step_async queues n steps of every engine and returns; oafdtd_batch_wait
 * synchronises and reports errors, including a bounded wait that gave up (OAFDTD_E_TIMEOUT).
 * OAFDTD_E_RANGE past any engine's max_steps. Replaces looping the reference's engine over the
 * instances of a sweep (one CupyEngine per problem, packages/oa-fdtd/src/oa_fdtd/engine.py:390-437). */
int oafdtd_batch_create(oafdtd_engine* const* engines, int32_t n, oafdtd_batch** out);
int oafdtd_batch_step_async(oafdtd_batch* batch, int64_t n);
int oafdtd_batch_wait(oafdtd_batch* batch);
/* Kernel launches in one replay of the batch's 64-step graph (0 before the first capture). */
int oafdtd_batch_graph_kernels(const oafdtd_batch* batch, int64_t* out);
int oafdtd_batch_destroy(oafdtd_batch* batch);

/* One half of a time step, launched eagerly and synchronised: which 0 = the H half (H update,
 * CPML-H, PMC ghosts, H probes), 1 = the E half (E update, CPML-E, Debye, SIBC, injection, E
 * probes; advances the step counter). A z-slab decomposition exchanges boundary planes between
 * the halves. OAFDTD_E_RANGE past max_steps; OAFDTD_E_INVALID when the halves come out of order.
 * The reference engine has no counterpart (it steps whole steps only). */
int oafdtd_step_half(oafdtd_engine* engine, int32_t which);

/* Storage plane k (0 .. nz+1) of one component, all batch members, (batch, ny+2, pitch) as
 * float64: read (oafdtd_plane) or written, rounded to the field precision (oafdtd_set_plane).
 * The halo exchange of a z-slab decomposition; no counterpart in the reference engine. */
int oafdtd_plane(oafdtd_engine* engine, int32_t comp, int32_t k, double* out);
int oafdtd_set_plane(oafdtd_engine* engine, int32_t comp, int32_t k, const double* in);

/* The same plane in the engine's own precision (real_bytes per value), device to device: dst / src
 * is device memory holding (batch, ny+2, pitch) values, on this GPU or a peer. The copies run on
 * the handle's stream and have finished when the call returns. For the halo exchange of a z-slab
 * decomposition without a trip through host memory (NCCL send/recv or peer copies of the buffer);
 * no counterpart in the reference. */
int oafdtd_plane_device(oafdtd_engine* engine, int32_t comp, int32_t k, void* dst);
int oafdtd_set_plane_device(oafdtd_engine* engine, int32_t comp, int32_t k, const void* src);

/* Overwrites one field component from float64 values in the oafdtd_fields layout, rounded to
 * the field precision (restoring fields, or starting a check from a chosen state). The reference
 * engine has no counterpart. */
int oafdtd_set_field(oafdtd_engine* engine, int32_t comp, const double* in);

/* Device bytes held by the handle: replaces CupyEngine.peak_bytes (engine.py:505-506). */
int oafdtd_peak_bytes(const oafdtd_engine* engine, int64_t* out);

/* 0: eager launches only; 1 (default): capture the first full 64-step chunk into a CUDA graph
 * and replay it (the reference's use_graph flag, engine.py:80,425-429). */
int oafdtd_set_graph(oafdtd_engine* engine, int32_t use_graph);

/* Launch shape of the sweeps: z planes marched per block (tile_z, 0 keeps the current value) and
 * the sweep variant (3: the fused sweep, which updates H and E of the interior in one z-march and
 * runs the rest as variant 2; it keeps two buffers per field, reading the current ones and writing
 * the others, and is the default where the interior is not empty and the device has room for them;
 * 2 stages the planes through shared memory with TMA tensor copies, the default otherwise where
 * the driver encodes the descriptors; 1 stages them with cp.async; 0 marches them in registers;
 * -1 keeps it). Variants 2 and 3 without descriptors, and 3 without an interior, are
 * OAFDTD_E_INVALID. The autotuner sets these. A staged sweep whose copies do not arrive within its
 * bounded wait makes the step return OAFDTD_E_TIMEOUT. */
int oafdtd_set_tuning(oafdtd_engine* engine, int32_t tile_z, int32_t variant);
/* The current launch shape: planes per block and sweep variant (as oafdtd_set_tuning takes them). */
int oafdtd_get_tuning(const oafdtd_engine* engine, int32_t* tile_z, int32_t* variant);

/* Average device time per step of each kernel class over the last oafdtd_step call, measured
 * with CUDA events when profiling is on (oafdtd_set_profiling). Writes up to n values in the
 * order: h_sweep (interior, staged; in variant 3 the z-slab planes), h_slab (CPML slabs, or
 * everything in variant 0), ghosts, pre_e, e_sweep, e_slab, edges, probe_e, fused (the fused
 * sweep of variant 3), whole step. */
int oafdtd_set_profiling(oafdtd_engine* engine, int32_t on);
int oafdtd_kernel_times(oafdtd_engine* engine, double* out_ms, int32_t n);

/* Algorithmic DRAM bytes per time step of each kernel class under the current sweep variant, in
 * the order of oafdtd_kernel_times, then their sum; up to n values. The traffic model: 9 field
 * values per grid cell and batch member for each separate sweep (E also its three uint16 indices
 * per cell and the Debye currents), 12 for the fused sweep (E and H read once and written once),
 * psi read+write per CPML cell, the surface-impedance state per edge. A diagnostic of this
 * library; the reference has no counterpart. */
int oafdtd_kernel_bytes(oafdtd_engine* engine, double* out, int32_t n);

/* Kernel launches in one replay of the captured 64-step graph (0 before the first capture). A
 * diagnostic of this library; the reference has no counterpart. */
int oafdtd_graph_kernels(oafdtd_engine* engine, int64_t* out);

/* Algorithmic DRAM bytes of one time step (all batch members) under the traffic model of the
 * separate sweeps (72 + 6 / B bytes per plain float32 cell-update, plus CPML psi, Debye J and SIBC
 * state), whatever the variant moves: the figure the roofline fraction of the step is quoted
 * against. */
int oafdtd_model_bytes(const oafdtd_engine* engine, double* out);

/* Field arrays already resident on the device, described for oafdtd_energy_noalloc: the six
 * components (E0..E2, H0..H2) of shape (batch, nz+2, ny+2, pitch) in float32 (real_bytes 4) or
 * float64 (8), the three uint16 material index arrays (nz+2, ny+2, pitch), the relative
 * permittivity table indexed by them, and the node and cell weights of each axis (float64, length
 * pitch, ny+2, nz+2). All pointers are device pointers; stream may be NULL (default stream). */
typedef struct oafdtd_energy_view {
  int32_t real_bytes;
  int32_t nx, ny, nz, pitch, batch;
  const void* field[6];
  const uint16_t* idx[3];
  const double* eps_tab;
  const double* node_w[3];
  const double* cell_w[3];
  void* stream;
} oafdtd_energy_view;

/* Field energy 1/2 sum eps E^2 V + 1/2 mu0 sum H^2 V (float64, written to the host double *out)
 * of device-resident fields, without allocating any device memory: no cudaMalloc, cudaFree or
 * allocating library call. For callers that cannot allocate on the device, such as a plugin whose
 * host application owns every device allocation, or a service that reserves its device memory at
 * start-up and must not grow it afterwards. This entry point has no counterpart in the reference.
 * Its partial sums live in a fixed device array of 65536 doubles (512 KiB, held on every GPU that
 * loads the library until the process exits): a problem with 6 * batch * (nz + 2) > 65536 is
 * rejected with OAFDTD_E_INVALID. Every call in the process shares that one array, whatever stream
 * it is given, so calls that overlap on the GPU race; serialise them. The call is synchronous: it
 * returns after a device-to-host copy of the result and a synchronise of its stream, so it cannot
 * be issued while that stream is being captured (nor on the legacy default stream while another
 * stream captures in global mode); it returns OAFDTD_E_INVALID there without launching anything.
 * The first call in a device's context looks the array's address up for that context, which may
 * load the library's module on the device. Same formula as oafdtd_energy; the summation order
 * differs (per-plane partial sums), so results agree to float64 rounding. */
int oafdtd_energy_noalloc(const oafdtd_energy_view* view, double* out);

/* ---------------------------------------------------------------------------------------------
 * Native model compiler: the volume stages of compile_model (packages/oa-fdtd/src/oa_fdtd/
 * model.py:501-768) on host threads, bit for bit equal to the NumPy stages it replaces:
 * per-cell materials (model.py:272-296), the four-cell area-weighted edge average
 * (_edge_average, model.py:300-321) with the static Debye term (model.py:534-537) and the
 * lumped-port loading (model.py:610-647), the averaged-material table and uint16 index
 * (model.py:688-722), and the Debye edge lists (_compile_ade, model.py:331-367). Host pointers;
 * no GPU is needed. The caller builds the PEC masks (walls, PEC regions, conductors).
 * ------------------------------------------------------------------------------------------- */
typedef struct oafdtd_material_desc {
  int32_t nx, ny, nz;
  const double* cell_w[3];        /* storage cell weights, length n + 2 (zero on the ghosts) */
  const double* centres[3];       /* cell centres, length n */
  int32_t n_regions;              /* dielectric (non-PEC) regions, in the model's order */
  const double* reg_lo;           /* (n_regions, 3) closed box, cells by centre */
  const double* reg_hi;           /* (n_regions, 3) */
  const double* reg_eps;          /* n_regions */
  const double* reg_sig;          /* n_regions */
  int32_t n_poles;                /* Debye relaxation times of the model (at most 8) */
  const double* reg_strength;     /* (n_regions, n_poles) pole strengths of each region */
  const double* static_fac;       /* n_poles: dt / (2 tau_p + dt) */
  const uint8_t* pec[3];          /* per component, (nz+1, ny+1, nx+1), 1 = PEC edge */
  int64_t n_loads;                /* lumped-port loading: sigma added to single edges, in order */
  const int32_t* load_comp;
  const int64_t* load_lattice;    /* (k * (ny+1) + j) * (nx+1) + i on the component's lattice */
  const double* load_sig;
  int32_t threads;                /* 0: one per hardware thread */
  double dt;                      /* time step [s] (Debye coefficients) */
  double eps0;                    /* the vacuum permittivity the caller's tables use [F/m] */
  const double* taus;             /* n_poles relaxation times [s] */
} oafdtd_material_desc;

typedef struct oafdtd_materials oafdtd_materials;

/* Build; OAFDTD_E_TABLE when more than 65534 averaged materials. */
int oafdtd_materials_build(const oafdtd_material_desc* desc, oafdtd_materials** out);

/* Table entries including the PEC entry 0, and the dispersive edges per component. */
int oafdtd_materials_sizes(const oafdtd_materials* m, int32_t* n_mat, int64_t* ade_n);

/* Copy out: the three uint16 index arrays (nz+2, ny+2, pitch), the eps and sigma tables (n_mat),
 * and per component the dispersive edges' storage flat indices (ade_n[c]), their Debye
 * coefficients beta_p = eps0 d_p / (tau_p + dt / 2) (n_poles, ade_n[c]; d_p the averaged pole
 * strength) and cbe = cb of their table entry (ade_n[c]; cb = dt / (eps0 eps) / (1 + sigma dt /
 * (2 eps0 eps)) as model.py:723-726 writes it). The lists of a component without dispersive edges
 * may be NULL. The handle's lists are released as they are copied: call it once. */
int oafdtd_materials_fetch(oafdtd_materials* m, uint16_t* idx0, uint16_t* idx1, uint16_t* idx2, double* eps_tab,
                           double* sig_tab, int64_t* flat0, int64_t* flat1, int64_t* flat2, double* beta0,
                           double* beta1, double* beta2, double* cbe0, double* cbe1, double* cbe2);

int oafdtd_materials_free(oafdtd_materials* m);

/* ---------------------------------------------------------------------------------------------
 * Learned S-parameter surrogate: the kernels its training and inference run on. The reference
 * has no surrogate; these entry points extend the engine's sweep path (parameters -> S). All
 * pointers are device pointers; BF16 buffers are passed as void*; stream may be NULL. Nothing here
 * allocates. Returns 0, or -1 for bad arguments, -3 for a CUDA launch error.
 * ------------------------------------------------------------------------------------------- */

/* C = act(op(A) . op(B) + bias) on the tensor cores: BF16 operands, FP32 accumulation.
 * op(A) is M x K: A row-major M x K (ta = 0) or row-major K x M (ta = 1), leading dimension lda;
 * op(B) is K x N: B row-major K x N (tb = 0) or row-major N x K (tb = 1), leading dimension ldb.
 * C32 (FP32, nullable) and C16 (BF16, nullable) are row-major M x N with leading dimension ldc;
 * C32 = result + beta * C32. bias: N floats (nullable). act: 0 none, 1 ReLU, 2 keep only where
 * mask (BF16, layout of C) is positive (the ReLU derivative in the backward pass), 3 tanh,
 * 4 multiply by 1 - mask^2 (the tanh derivative, mask = the stored tanh outputs). */
int oafdtd_mlp_gemm(const void* A, const void* B, float* C32, void* C16, const float* bias, const void* mask,
                    int32_t M, int32_t N, int32_t K, int32_t lda, int32_t ldb, int32_t ldc, int32_t ta, int32_t tb,
                    int32_t act, float beta, void* stream);

/* out[g * out_stride + n] = sum over m < M of X[g * x_stride + m * ld + n] for g < groups (FP32;
 * bias gradients of every ensemble member in one launch). */
int oafdtd_mlp_colsum(const float* X, int32_t M, int32_t N, int32_t ld, float* out, int32_t groups,
                      int64_t x_stride, int64_t out_stride, void* stream);

/* Mean squared error of Y against T (both M x N FP32, M = groups x rows of each group): the
 * gradient 2 (Y - T) / ((M / groups) N) of each group's mean into G32 (FP32) and G16 (BF16), and
 * the sum of squared errors of each row into row_loss[M]. */
int oafdtd_mlp_mse_grad(const float* Y, const float* T, int32_t M, int32_t N, float* G32, void* G16,
                        float* row_loss, int32_t groups, void* stream);

/* One Adam step on n FP32 weights w (moments m1, m2), refreshing the BF16 copy w16 (nullable).
 * The learning rate is read from *lr (device float) and the step number for the bias corrections
 * from *step (device int32, >= 1), so a captured step replays with both moving on. */
int oafdtd_mlp_adam(float* w, void* w16, const float* grad, float* m1, float* m2, int64_t n, const float* lr,
                    float b1, float b2, float eps, const int32_t* step, void* stream);

/* Grouped: C_g = act(A_g . B_g^T + bias_g) for g < groups, with A_g row-major M x K and B_g
 * row-major N x K (both K-contiguous), BF16 operands, FP32 accumulation, the epilogues of
 * oafdtd_mlp_gemm (ldc for C32, C16 and mask). Group g's operands start strideA, strideB, strideC
 * (C32, C16 and mask), strideCT (C16T) and strideBias elements after group g - 1's (ignored for
 * one group). Problems with M a multiple of 128, N and K multiples of 64, leading dimensions and
 * strides multiples of 8, 16-byte aligned pointers and beta 0 run on the fifth-generation tensor
 * cores (tcgen05.mma, accumulators in tensor memory, operand tiles and results moved by TMA tensor
 * copies; one persistent launch for all groups); the others on the mma.sync kernel, one launch.
 * C16T (BF16, nullable) receives the result transposed, N x M with leading dimension ldct (the next
 * layer's weight gradient reads it K-contiguous); off the tcgen05 shapes it needs C16 as well.
 * status (device int32, nullable): bit 0 is set when a bounded wait of the tcgen05 kernel gave up
 * (that launch's C is then incomplete). */
int oafdtd_mlp_gemm_tn(const void* A, const void* B, float* C32, void* C16, void* C16T, const float* bias,
                       const void* mask, int32_t M, int32_t N, int32_t K, int32_t lda, int32_t ldb, int32_t ldc,
                       int32_t ldct, int32_t act, float beta, int32_t groups, int64_t strideA, int64_t strideB,
                       int64_t strideC, int64_t strideCT, int64_t strideBias, int32_t* status, void* stream);

/* dst_g (cols x rows, leading dimension ldd) = src_g^T (rows x cols, leading dimension lds), BF16,
 * for g < groups, src_g and dst_g src_stride and dst_stride elements after group g - 1's. */
int oafdtd_mlp_transpose(const void* src, int32_t rows, int32_t cols, int32_t lds, void* dst, int32_t ldd,
                         int32_t groups, int64_t src_stride, int64_t dst_stride, void* stream);

/* *counter += 1 on the device (the Adam step number inside a captured training step). */
int oafdtd_mlp_count(int32_t* counter, void* stream);

/* Rows idx[0..rows) (device int32) of an FP32 matrix with cols columns, into dst32 (FP32) and/or
 * dst16 (BF16), each rows x cols. */
int oafdtd_mlp_gather(const float* src, int32_t cols, const int32_t* idx, int32_t rows, float* dst32, void* dst16,
                      void* stream);

#ifdef __cplusplus
}
#endif

#endif /* OAFDTD_H */
