// C ABI of the GB300 FDTD engine: device state, host-side preparation of the edge lists and the
// combined material table, the step driver (eager launches or a captured 64-step CUDA graph) and
// the observables. The public contract is include/oafdtd.h.

#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cmath>
#include <cstdio>
#include <array>
#include <cstring>
#include <future>
#include <map>
#include <memory>
#include <new>
#include <string>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "../../include/oafdtd.h"
#include "oafdtd_internal.cuh"

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

#define OA_CUDA(call)                                                                             \
  do {                                                                                            \
    cudaError_t err_ = (call);                                                                    \
    if (err_ != cudaSuccess)                                                                      \
      return fail(err_ == cudaErrorMemoryAllocation ? OAFDTD_E_OOM : OAFDTD_E_CUDA,               \
                  std::string(#call) + ": " + cudaGetErrorString(err_));                          \
  } while (0)

constexpr double kEps0 = 1.0 / (4e-7 * 3.14159265358979323846 * 299792458.0 * 299792458.0);
constexpr double kMu0 = 4e-7 * 3.14159265358979323846;

// E_TERMS of oa_fdtd/pml.py:26-33: (c, a, b, sign); H_TERMS have the opposite signs.
constexpr int kTerms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 2, 0}, {1, 0, 2}, {2, 0, 1}, {2, 1, 0}};
constexpr double kTermSign[6] = {1.0, -1.0, 1.0, -1.0, 1.0, -1.0};

struct EngineBase {
  virtual ~EngineBase() = default;
  virtual int step(int64_t n) = 0;
  virtual int energy(double* out) = 0;
  virtual int dft(double* out) = 0;
  virtual int series(double* out) = 0;
  virtual int fields(int comp, double* out) = 0;
  virtual int set_field(int comp, const double* in) = 0;
  virtual int step_half(int which) = 0;
  virtual int enqueue(int64_t n) = 0;
  virtual int snapshot(void* out, int64_t* bytes, const void* in) = 0;
  virtual int wait() = 0;
  virtual int plane(int comp, int k, double* out, const double* in) = 0;
  virtual int plane_device(int comp, int k, void* dst, const void* src) = 0;
  virtual int kernel_times(double* out, int n) = 0;
  virtual int step_timed(int64_t n, double* ms) = 0;
  // Switches the sweep variant (0..3); the fused variant allocates the second field buffers.
  virtual int set_variant(int v) = 0;
  // Waits until class_bytes / model_bytes are filled in (a host thread computes them after build).
  virtual void traffic_ready() {}
  int64_t steps = 0;
  int64_t bytes = 0;
  int use_graph = 1;
  int profiling = 0;
  int tile_z = 16;
  // 3: fused H + E sweep of the interior (two buffers per field), the rest as 2; 2: sweeps
  // staged by TMA; 1: staged by cp.async; 0: register marching
  int staged = 2;
  bool tma_ok = false;  // the TMA descriptors were encoded (variant 2 available)
  bool fused_ok = false;  // the fused box is not empty and its descriptors were encoded
  bool graph_dirty = false;  // launch shape or profiling changed: the graph is re-captured
  int64_t graph_kernels = 0;  // kernel nodes of the current captured 64-step graph (0: none)
  // kernel classes: h_sweep, h_slab, ghosts, pre_e, e_sweep, e_slab, edges, probe_e, fused
  static constexpr int kClasses = 9;
  // algorithmic bytes per step and class: [0] variant 0, [1] variants 1 and 2, [2] variant 3
  double class_bytes[3][kClasses] = {};
  double model_bytes = 0.0;
};

template <typename real>
struct Engine final : EngineBase {
  int device = 0;
  cudaStream_t stream = nullptr;
  oafdtd::Span3 inner_staged[2]{};     // interior boxes (E, H) when the staged sweeps run
  oafdtd::Span3 zin_staged[2][2]{};    // z-slab planes over the interior's x-y extent
  int zsd[2][2][2] = {};               // side of the z-term psi per (kind, low/high, component)
  oafdtd::Span3 slab_staged[2][6]{};   // the slab boxes around them
  int n_slab_staged[2] = {0, 0};
  oafdtd::Span3 whole{};               // the whole update domain (variant 0: slab kernel only)
  std::vector<void*> allocs;
  int nx = 0, ny = 0, nz = 0, X = 0, Y = 0, Z = 0, B = 0;
  long long bs = 0;
  // Field buffers [buffer][E0..E2, H0..H2]. Buffer 1 exists once the fused variant has run:
  // it then reads the current buffers and writes the other ones, and cur[] (E, H) swaps.
  real* fbuf[2][6] = {};
  int cur[2] = {0, 0};
  bool two_buffers = false;
  oafdtd::Span3 fused_box{};              // the fused sweep's box (variant 3)
  oafdtd::Span3 zin_fused[2][2]{};        // z-slab planes over its x-y extent
  oafdtd::Span3 slab_fused[2][6]{};       // the slab boxes around it
  int n_slab_fused[2] = {0, 0};
  int graph_parity = 0;                   // cur[0] at the start of the captured chunk
  int pmc_mask = 0;
  int max_steps = 0;
  int n_probe = 0, n_freq = 0, record_series = 0;
  oafdtd::SweepArgs<real> sw{};
  oafdtd::SweepMaps maps_p[2]{};  // staged-sweep descriptors of a step starting in buffer 0 / 1
  oafdtd::FusedMaps fmaps[2]{};   // fused-sweep descriptors of a step starting in buffer 0 / 1
  int* status = nullptr;  // device status word of the bounded waits
  oafdtd::EdgeArgs<real> ed{};
  oafdtd::SibcArgs<real> sb{};
  oafdtd::ProbeArgs<real> pr{};
  oafdtd::EnergyArgs<real> en{};
  long long* step_base = nullptr;
  double* energy_partial = nullptr;
  double* energy_out = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  bool graph_ready = false;
  std::vector<cudaEvent_t> events;    // (kChunk, kClasses + 1) in profiling mode
  double prof_ms[kClasses + 1] = {};
  int64_t prof_steps = 0;

  ~Engine() override {
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    for (cudaEvent_t e : events) cudaEventDestroy(e);
    if (t_start) cudaEventDestroy(t_start);
    if (t_stop) cudaEventDestroy(t_stop);
    for (void* p : allocs) cudaFree(p);
    for (cudaEvent_t e : {fork_ev, join_ev, ejoin_ev})
      if (e) cudaEventDestroy(e);
    if (side) cudaStreamDestroy(side);
    if (stream) cudaStreamDestroy(stream);
  }

  template <typename T>
  int alloc(T** out, size_t count) {
    *out = nullptr;
    if (count == 0) count = 1;
    void* p = nullptr;
    cudaError_t err = cudaMalloc(&p, count * sizeof(T));
    if (err != cudaSuccess)
      return fail(err == cudaErrorMemoryAllocation ? OAFDTD_E_OOM : OAFDTD_E_CUDA,
                  "cudaMalloc of " + std::to_string(count * sizeof(T)) + " bytes: " + cudaGetErrorString(err));
    allocs.push_back(p);
    bytes += (int64_t)(count * sizeof(T));
    err = cudaMemsetAsync(p, 0, count * sizeof(T), stream);
    if (err != cudaSuccess) return fail(OAFDTD_E_CUDA, cudaGetErrorString(err));
    *out = static_cast<T*>(p);
    return OAFDTD_OK;
  }

  // Device buffers that hold the run's state (fields, psi, Debye currents, SIBC state, deferred
  // E^n, DFT accumulators, recorded series, step counter), in registration order: a snapshot.
  std::vector<std::pair<void*, size_t>> state_bufs;
  template <typename T>
  void keep_state(T* p, size_t count) {
    state_bufs.emplace_back(static_cast<void*>(p), count * sizeof(T));
  }

  template <typename T>
  int upload(T** out, const T* host, size_t count) {
    int rc = alloc(out, count);
    if (rc) return rc;
    if (count) OA_CUDA(cudaMemcpyAsync(*out, host, count * sizeof(T), cudaMemcpyHostToDevice, stream));
    return OAFDTD_OK;
  }

  template <typename T>
  int upload_vec(T** out, const std::vector<T>& v) {
    return upload(out, v.data(), v.size());
  }

  int upload_real(const real** out, const double* host, size_t count) {
    std::vector<real> tmp(count);
    for (size_t k = 0; k < count; ++k) tmp[k] = (real)host[k];
    real* d = nullptr;
    int rc = upload_vec(&d, tmp);
    *out = d;
    return rc;
  }

  int build(const oafdtd_problem& p);
  // parts: 1 the H half (H sweeps, ghosts, pre_e), 2 the E half (E sweeps, SIBC, edges, probe_e)
  int launch_step(int off, cudaEvent_t* ev, bool capturing = false, int parts = 3);
  int step_half(int which) override;
  int plane(int comp, int k, double* out, const double* in) override;
  int plane_device(int comp, int k, void* dst, const void* src) override;
  bool half_pending = false;  // an H half ran and its E half has not
  int capture();

  int step(int64_t n) override;
  int enqueue(int64_t n) override;
  int snapshot(void* out, int64_t* bytes, const void* in) override;
  int wait() override;
  int check_status();
  // The sweep regions of variant rv: the fused box with the z-slab and slab boxes around it (3),
  // the staged interior with its z-slab and slab boxes (1, 2), or the slab kernel alone (0).
  void use_regions(int rv) {
    sw.staged = rv == 3 ? 2 : rv;
    sw.fused = rv == 3 ? fused_box : oafdtd::Span3{0, 0, 0, 0, 0, 0};
    for (int kind = 0; kind < 2; ++kind) {
      for (int zr = 0; zr < 2; ++zr)
        for (int cc = 0; cc < 2; ++cc) sw.zsd[kind][zr][cc] = zsd[kind][zr][cc];
      if (rv == 3) {
        sw.inner[kind] = oafdtd::Span3{0, 0, 0, 0, 0, 0};
        sw.zin[kind][0] = zin_fused[kind][0];
        sw.zin[kind][1] = zin_fused[kind][1];
        sw.n_slab[kind] = n_slab_fused[kind];
        for (int n = 0; n < 6; ++n) sw.slab[kind][n] = slab_fused[kind][n];
      } else if (rv) {
        sw.inner[kind] = inner_staged[kind];
        sw.zin[kind][0] = zin_staged[kind][0];
        sw.zin[kind][1] = zin_staged[kind][1];
        sw.n_slab[kind] = n_slab_staged[kind];
        for (int n = 0; n < 6; ++n) sw.slab[kind][n] = slab_staged[kind][n];
      } else {
        sw.inner[kind] = oafdtd::Span3{0, 0, 0, 0, 0, 0};
        sw.zin[kind][0] = sw.zin[kind][1] = oafdtd::Span3{0, 0, 0, 0, 0, 0};
        sw.n_slab[kind] = 1;
        sw.slab[kind][0] = whole;
      }
    }
  }
  // Pointers of a step that starts with E in buffer pe and H in buffer ph. In place (variants
  // 0-2) the step writes the buffers it reads; the fused variant writes the other ones.
  void bind(int pe, int ph) {
    const bool pp = staged == 3;
    for (int c = 0; c < 3; ++c) {
      sw.E[c] = fbuf[pe][c];
      sw.H[c] = fbuf[ph][3 + c];
      sw.Eo[c] = fbuf[pp ? 1 - pe : pe][c];
      sw.Ho[c] = fbuf[pp ? 1 - ph : ph][3 + c];
      ed.E[c] = sw.Eo[c];
      ed.H[c] = sw.Ho[c];
      sb.E[c] = sw.Eo[c];
      sb.H[c] = sw.Ho[c];
      pr.E[c] = sw.E[c];
      pr.F[c] = sw.Eo[c];
      pr.F[3 + c] = sw.Ho[c];
    }
  }
  // The current buffer of one component (0..2 E, 3..5 H).
  real* field(int comp) { return fbuf[cur[comp < 3 ? 0 : 1]][comp]; }
  // Encodes the TMA descriptors of a step starting in each buffer for the current variant.
  int encode_maps();
  // Copies the current fields into the other buffers (both then hold the same state).
  int sync_buffers();
  int set_variant(int v) override;
  int energy(double* out) override;
  int dft(double* out) override;
  int series(double* out) override;
  int fields(int comp, double* out) override;
  int set_field(int comp, const double* in) override;
  int kernel_times(double* out, int n) override;
  int step_timed(int64_t n, double* ms) override;
  cudaEvent_t t_start = nullptr, t_stop = nullptr;
  // The slab kernel runs beside the staged sweep of the same kind (they write disjoint cells and
  // read only the other field): forked onto `side` and joined back, inside the graph as well.
  cudaStream_t side = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr, ejoin_ev = nullptr;
  // The E work of a fused step that reads no H the fused sweep writes (early) or the rest: the
  // slab boxes and z-slab boxes that lie entirely below the fused box on some axis (E at
  // (i, j, k) reads H at i - 1, j - 1 and k - 1 and at the cell itself).
  oafdtd::SweepArgs<real> e_part(bool early) const {
    oafdtd::SweepArgs<real> a = sw;
    const oafdtd::Span3& F = fused_box;
    auto below = [&](const oafdtd::Span3& b) { return b.j1 <= F.j0 || b.q1 <= F.q0 || b.k1 <= F.k0; };
    int n = 0;
    for (int s = 0; s < sw.n_slab[0]; ++s)
      if (below(sw.slab[0][s]) == early) a.slab[0][n++] = sw.slab[0][s];
    a.n_slab[0] = n;
    for (int zr = 0; zr < 2; ++zr)
      if (below(sw.zin[0][zr]) != early) a.zin[0][zr] = oafdtd::Span3{0, 0, 0, 0, 0, 0};
    return a;
  }
  int sweep_pair(int kind, cudaEvent_t* ev, int slot, unsigned rec, const oafdtd::SweepMaps& mp,
                 int pre_e_off = -1);
  // The traffic model, computed on a host thread of its own while the engine is in use (it
  // scans the index arrays). Declared last: it is destroyed, and so waited for, first.
  std::future<void> traffic;
  void traffic_ready() override {
    if (traffic.valid()) traffic.wait();
  }
};

// Build phase timer: with OAFDTD_TIMING set in the environment, oafdtd_create prints the
// host time of each phase of the build to stderr (diagnostics only).
struct PhaseTimer {
  bool on = std::getenv("OAFDTD_TIMING") != nullptr;
  std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
  void mark(const char* what) {
    if (!on) return;
    const auto now = std::chrono::steady_clock::now();
    std::fprintf(stderr, "oafdtd build %-22s %8.1f ms\n", what,
                 std::chrono::duration<double, std::milli>(now - t).count());
    t = now;
  }
};

// Runs f(begin, end, part) over [0, n) split into contiguous parts, one host thread each (up to
// 16; one part below 65536 items). The split depends only on n, so two calls with the same n
// hand the same range to the same part.
constexpr int kMaxParts = 16;
template <typename F>
void parallel_parts(long long n, F&& f) {
  int T = (int)std::min<unsigned>(std::max(1u, std::thread::hardware_concurrency()), (unsigned)kMaxParts);
  if (n < (1LL << 16)) T = 1;
  const long long chunk = (n + T - 1) / T;
  std::vector<std::thread> th;
  for (int t = 1; t < T; ++t) {
    const long long b = t * chunk, e = std::min(n, b + chunk);
    if (b < e) th.emplace_back([&f, b, e, t] { f(b, e, t); });
  }
  f(0, std::min(n, chunk), 0);
  for (std::thread& x : th) x.join();
}

// ---------------------------------------------------------------------------- build
template <typename real>
int Engine<real>::build(const oafdtd_problem& p) {
  PhaseTimer timer;
  nx = p.nx;
  ny = p.ny;
  nz = p.nz;
  X = p.pitch;
  Y = ny + 2;
  Z = nz + 2;
  B = p.batch;
  bs = (long long)X * Y * Z;
  pmc_mask = p.pmc_mask;
  max_steps = p.max_steps;
  if (nx < 1 || ny < 1 || nz < 1 || B < 1 || X < nx + 2 || X % 32 != 0)
    return fail(OAFDTD_E_INVALID, "bad grid or batch size");
  if (p.n_mat < 1 || p.n_mat > 65535) return fail(OAFDTD_E_INVALID, "n_mat out of range");
  if (p.ade_poles < 0 || p.ade_poles > oafdtd::kMaxAdePoles)
    return fail(OAFDTD_E_INVALID, "at most 16 Debye poles are supported");
  OA_CUDA(cudaGetDevice(&device));
  OA_CUDA(oafdtd::preload_kernels<real>());
  OA_CUDA(oafdtd::preload_staged<real>());
  OA_CUDA(oafdtd::preload_slab<real>());
  OA_CUDA(oafdtd::preload_fused<real>());
  OA_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  OA_CUDA(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
  OA_CUDA(cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming));
  OA_CUDA(cudaEventCreateWithFlags(&join_ev, cudaEventDisableTiming));
  OA_CUDA(cudaEventCreateWithFlags(&ejoin_ev, cudaEventDisableTiming));

  auto in_range = [&](long long f) { return f >= 0 && f < bs; };

  // fields
  for (int c = 0; c < 3; ++c) {
    real* e = nullptr;
    real* h = nullptr;
    int rc = alloc(&e, (size_t)bs * B);
    if (rc) return rc;
    rc = alloc(&h, (size_t)bs * B);
    if (rc) return rc;
    fbuf[0][c] = e;
    fbuf[0][3 + c] = h;
  }
  bind(0, 0);

  timer.mark("fields");
  // ---- Debye ADE: per-edge coefficient rows and the set of dispersive edges
  const int P = p.ade_poles;
  // injection targets (component, flat)
  std::vector<std::pair<int, long long>> inj_keys;
  inj_keys.reserve((size_t)p.n_inj);
  for (int64_t t = 0; t < p.n_inj; ++t) {
    if (p.inj_comp[t] < 0 || p.inj_comp[t] > 2 || !in_range(p.inj_flat[t]) || p.inj_chan[t] < 0 ||
        p.inj_chan[t] >= p.n_chan)
      return fail(OAFDTD_E_INVALID, "injection entry out of range");
    inj_keys.emplace_back(p.inj_comp[t], p.inj_flat[t]);
  }
  std::vector<std::pair<int, long long>> inj_sorted = inj_keys;
  std::sort(inj_sorted.begin(), inj_sorted.end());
  auto injected = [&](int c, long long f) {
    return std::binary_search(inj_sorted.begin(), inj_sorted.end(), std::make_pair(c, f));
  };
  // surface-impedance edges (one bit per storage cell and component): a dispersive one is
  // updated after the surface impedance sets it
  std::vector<bool> sibc_bits;
  if (p.sibc_n > 0) {
    sibc_bits.assign((size_t)(3 * bs), false);
    for (int64_t s = 0; s < p.sibc_n; ++s) {
      const int c = p.sibc_comp[s];
      const long long f = p.sibc_flat[s];
      if (c < 0 || c > 2 || !in_range(f) || p.sibc_mat[s] < 0 || p.sibc_mat[s] >= p.sibc_nmat)
        return fail(OAFDTD_E_INVALID, "SIBC edge out of range");
      for (int k = 0; k < 2; ++k)
        if (p.sibc_hsign[2 * s + k] != 0.0 && (p.sibc_hcomp[2 * s + k] < 0 || p.sibc_hcomp[2 * s + k] > 2 ||
                                               !in_range(p.sibc_hflat[2 * s + k])))
          return fail(OAFDTD_E_INVALID, "SIBC sample out of range");
      std::vector<bool>::reference bit = sibc_bits[(size_t)(c * bs + f)];
      if (bit) return fail(OAFDTD_E_INVALID, "duplicate SIBC edge");
      bit = true;
    }
  }
  auto on_sibc = [&](int c, long long f) { return !sibc_bits.empty() && sibc_bits[(size_t)(c * bs + f)]; };

  timer.mark("ade_classify");
  // ---- combined table. Entry key: (category, material index, ADE row); categories 0 plain,
  // 1 dispersive, 2 dispersive with injection or surface impedance (deferred to the edge pass,
  // after those). The map orders entries by category, so the kernels tell dispersive entries by
  // an index range.
  // Debye rows (cbe, beta_0..P-1) in the field precision. The edges are classified in parallel
  // parts; each part finds its rows (consecutive edges mostly share one, so the last is checked
  // first and a hash finds the others) and its table keys, then the parts are merged in order.
  struct AdeEdge {
    long long f;
    int rid;
    int defer;
  };
  struct RowSet {
    std::vector<std::vector<real>> rows;
    std::unordered_map<uint64_t, std::vector<int>> by_hash;
    int last = -1;
    int find_or_add(const real* row, int n) {
      if (last >= 0 && std::memcmp(row, rows[last].data(), sizeof(real) * n) == 0) return last;
      uint64_t h = 1469598103934665603ull;
      const unsigned char* bytes = reinterpret_cast<const unsigned char*>(row);
      for (size_t q = 0; q < sizeof(real) * n; ++q) h = (h ^ bytes[q]) * 1099511628211ull;
      std::vector<int>& bucket = by_hash[h];
      for (int cand : bucket)
        if (std::memcmp(row, rows[cand].data(), sizeof(real) * n) == 0) return last = cand;
      rows.emplace_back(row, row + n);
      bucket.push_back((int)rows.size() - 1);
      return last = (int)rows.size() - 1;
    }
  };
  using Key = std::tuple<int, int, int>;  // (category, material index, Debye row)
  RowSet global_rows;
  std::vector<AdeEdge> ade_edges[3];
  std::vector<std::pair<int, long long>> deferred;  // (comp, flat) in component order
  int kmin[3] = {0, 0, 0}, kmax[3] = {-1, -1, -1};
  std::map<Key, int> entry;  // key -> combined table id
  // material indices: range check and the set of plain materials present
  std::vector<uint8_t> present(p.n_mat, 0);
  {
    std::vector<std::vector<uint8_t>> seen(kMaxParts);
    for (std::vector<uint8_t>& sv : seen) sv.assign(p.n_mat, 0);
    int bad = 0;
    for (int c = 0; c < 3 && !bad; ++c) {
      const uint16_t* idx = p.idx[c];
      std::vector<int> part_bad(kMaxParts, 0);
      parallel_parts(bs, [&](long long b0, long long e0, int t) {
        uint8_t* mark = seen[t].data();
        for (long long q = b0; q < e0; ++q) {
          const uint16_t v = idx[q];
          if (v >= p.n_mat) {
            part_bad[t] = 1;
            return;
          }
          mark[v] = 1;
        }
      });
      for (int t : part_bad) bad |= t;
    }
    if (bad) return fail(OAFDTD_E_INVALID, "material index beyond the table");
    for (const std::vector<uint8_t>& sv : seen)
      for (size_t v = 0; v < sv.size(); ++v) present[v] |= sv[v];
  }
  for (int c = 0; c < 3; ++c) {
    const uint16_t* idx = p.idx[c];
    const int64_t ne = P > 0 ? p.ade_n[c] : 0;
    ade_edges[c].resize((size_t)ne);
    struct Part {
      RowSet rows;
      std::vector<Key> keys;
      Key last_key{-1, -1, -1};
      int kmin = 1 << 30, kmax = -1;
      bool bad = false;
      std::vector<long long> defer;
      std::vector<int> remap;
    };
    std::vector<Part> parts(kMaxParts);
    AdeEdge* out = ade_edges[c].data();
    parallel_parts(ne, [&](long long b0, long long e0, int t) {
      Part& L = parts[t];
      real row[1 + oafdtd::kMaxAdePoles];
      for (long long e = b0; e < e0; ++e) {
        const long long f = p.ade_flat[c][e];
        if (!in_range(f)) {
          L.bad = true;
          return;
        }
        row[0] = (real)p.ade_cbe[c][e];
        for (int q = 0; q < P; ++q) row[1 + q] = (real)p.ade_beta[c][(size_t)q * ne + e];
        const int rid = L.rows.find_or_add(row, 1 + P);
        const int defer = (injected(c, f) || on_sibc(c, f)) ? 1 : 0;
        out[e] = AdeEdge{f, rid, defer};
        const Key key{1 + defer, idx[f], rid};
        if (key != L.last_key) {
          if (std::find(L.keys.begin(), L.keys.end(), key) == L.keys.end()) L.keys.push_back(key);
          L.last_key = key;
        }
        if (defer) L.defer.push_back(f);
        const int k = (int)(f / ((long long)X * Y));
        L.kmin = std::min(L.kmin, k);
        L.kmax = std::max(L.kmax, k);
      }
    });
    // merge in part order: global row ids, table keys, deferred edges, plane range
    for (Part& L : parts) {
      if (L.bad) return fail(OAFDTD_E_INVALID, "ADE edge out of range");
      L.remap.resize(L.rows.rows.size());
      for (size_t r = 0; r < L.rows.rows.size(); ++r)
        L.remap[r] = global_rows.find_or_add(L.rows.rows[r].data(), 1 + P);
      for (const Key& k : L.keys) entry[Key{std::get<0>(k), std::get<1>(k), L.remap[std::get<2>(k)]}] = 0;
      for (long long f : L.defer) deferred.emplace_back(c, f);
      if (L.kmax >= 0) {
        if (kmax[c] < kmin[c]) {
          kmin[c] = L.kmin;
          kmax[c] = L.kmax;
        } else {
          kmin[c] = std::min(kmin[c], L.kmin);
          kmax[c] = std::max(kmax[c], L.kmax);
        }
      }
    }
    parallel_parts(ne, [&](long long b0, long long e0, int t) {
      const std::vector<int>& remap = parts[t].remap;
      for (long long e = b0; e < e0; ++e) out[e].rid = remap[out[e].rid];
    });
  }
  const std::vector<std::vector<real>>& ade_rows = global_rows.rows;
  for (int v = 0; v < p.n_mat; ++v)
    if (present[v]) entry[{0, v, -1}] = 0;
  if (entry.size() > 65536) return fail(OAFDTD_E_TABLE, "more than 65536 combined material entries");
  std::vector<oafdtd::Coef<real>> t_coef;
  std::vector<real> t_beta;
  std::vector<double> t_eps;
  std::vector<int> plain(p.n_mat, 0);
  int ade_lo = -1, ade_hi = -1;
  for (auto& kv : entry) {
    const int cat = std::get<0>(kv.first), v = std::get<1>(kv.first), rid = std::get<2>(kv.first);
    const int id = (int)t_coef.size();
    kv.second = id;
    if (cat == 1 && ade_lo < 0) ade_lo = id;
    if (cat == 1) ade_hi = id + 1;
    if (cat == 0) plain[v] = id;
    oafdtd::Coef<real> cf;
    cf.ca = (real)p.ca_tab[v];
    cf.cb = (real)p.cb_tab[v];
    cf.cbe = rid >= 0 ? ade_rows[rid][0] : (real)0;
    cf.beta0 = (rid >= 0 && P > 0) ? ade_rows[rid][1] : (real)0;
    t_coef.push_back(cf);
    for (int q = 0; q < P; ++q) t_beta.push_back(rid >= 0 ? ade_rows[rid][1 + q] : (real)0);
    t_eps.push_back(p.eps_tab[v] * kEps0);
  }
  if (ade_lo < 0) ade_lo = ade_hi = 0;
  // the index arrays: plain entries, then each dispersive edge's entry; kept on the host for the
  // traffic model
  std::vector<uint16_t> host_mat[3];
  for (int c = 0; c < 3; ++c) {
    std::vector<uint16_t>& m = host_mat[c];
    m.resize((size_t)bs);
    const uint16_t* idx = p.idx[c];
    parallel_parts(bs, [&](long long b0, long long e0, int) {
      for (long long q = b0; q < e0; ++q) m[q] = (uint16_t)plain[idx[q]];
    });
    const AdeEdge* ae = ade_edges[c].data();
    parallel_parts((long long)ade_edges[c].size(), [&](long long b0, long long e0, int) {
      Key lk{-1, -1, -1};
      int lid = 0;
      for (long long e = b0; e < e0; ++e) {
        const Key key{1 + ae[e].defer, idx[ae[e].f], ae[e].rid};
        if (key != lk) {
          lid = entry.find(key)->second;
          lk = key;
        }
        m[ae[e].f] = (uint16_t)lid;
      }
    });
    uint16_t* dm = nullptr;
    int rc = upload_vec(&dm, m);
    if (rc) return rc;
    sw.mat[c] = dm;
    ed.mat[c] = dm;
    en.mat[c] = dm;
  }
  {
    oafdtd::Coef<real>* dc = nullptr;
    int rc = upload_vec(&dc, t_coef);
    if (rc) return rc;
    sw.coef = ed.coef = dc;
    sw.n_coef = (int)t_coef.size();
    sw.ade_lo = ade_lo;
    sw.ade_hi = ade_hi;
    real* d = nullptr;
    if (t_beta.empty()) t_beta.push_back((real)0);
    rc = upload_vec(&d, t_beta);
    if (rc) return rc;
    sw.ade_beta = ed.ade_beta = d;
    double* eps = nullptr;
    rc = upload_vec(&eps, t_eps);
    if (rc) return rc;
    en.eps = eps;
    std::vector<real> kp(std::max(P, 1), (real)0), onekp(std::max(P, 1), (real)0);
    for (int q = 0; q < P; ++q) {
      kp[q] = (real)p.ade_kp[q];
      onekp[q] = (real)1 + kp[q];
    }
    rc = upload_vec(&d, kp);
    if (rc) return rc;
    sw.ade_kp = ed.ade_kp = d;
    rc = upload_vec(&d, onekp);
    if (rc) return rc;
    sw.ade_onekp = ed.ade_onekp = d;
    sw.ade_P = ed.ade_P = P;
  }
  for (int c = 0; c < 3; ++c) {
    const int nk = kmax[c] >= kmin[c] ? kmax[c] - kmin[c] + 1 : 0;
    sw.jk0[c] = ed.jk0[c] = kmin[c];
    sw.jnk[c] = ed.jnk[c] = nk;
    real* J = nullptr;
    if (nk > 0) {
      int rc = alloc(&J, (size_t)P * B * nk * Y * X);
      if (rc) return rc;
      keep_state(J, (size_t)P * B * nk * Y * X);
    }
    sw.J[c] = ed.J[c] = J;
  }

  timer.mark("table_mat_J");
  // ---- 1-D metrics
  const int len[3] = {X, Y, Z};
  for (int a = 0; a < 3; ++a) {
    int rc = upload_real(&sw.ip[a], p.inv_primal[a], len[a]);
    if (rc) return rc;
    rc = upload_real(&sw.idd[a], p.inv_dual[a], len[a]);
    if (rc) return rc;
  }

  timer.mark("metrics");
  // ---- CPML
  sw.has_cpml = p.n_corr > 0;
  for (int a = 0; a < 3; ++a) {
    for (int t = 0; t < 3; ++t) sw.pe[a][t] = sw.ph[a][t] = nullptr;
    if (p.pml[a][0] == nullptr) continue;
    for (int t = 0; t < 3; ++t) {
      int rc = upload_real(&sw.pe[a][t], p.pml[a][t], len[a]);
      if (rc) return rc;
      rc = upload_real(&sw.ph[a][t], p.pml[a][3 + t], len[a]);
      if (rc) return rc;
    }
  }
  for (int c = 0; c < 3; ++c)
    for (int s = 0; s < 2; ++s) {
      sw.ecorr[c][s] = oafdtd::CpmlTerm<real>{};
      sw.hcorr[c][s] = oafdtd::CpmlTerm<real>{};
    }
  int last_slot[2][3] = {{-1, -1, -1}, {-1, -1, -1}};
  for (int n = 0; n < p.n_corr; ++n) {
    const oafdtd_correction& k = p.corr[n];
    if (k.kind < 0 || k.kind > 1 || k.c < 0 || k.c > 2 || k.a < 0 || k.a > 2 || k.b < 0 || k.b > 2)
      return fail(OAFDTD_E_INVALID, "bad CPML correction");
    int term = -1;
    for (int t = 0; t < 6; ++t)
      if (kTerms[t][0] == k.c && kTerms[t][1] == k.a && kTerms[t][2] == k.b) term = t;
    const double want = k.kind == 0 ? kTermSign[term < 0 ? 0 : term] : -kTermSign[term < 0 ? 0 : term];
    if (term < 0 || k.sign != want) return fail(OAFDTD_E_INVALID, "CPML correction is not a curl term");
    if (p.pml[k.a][0] == nullptr) return fail(OAFDTD_E_INVALID, "CPML correction on an axis without coefficients");
    const int first_axis = k.c == 0 ? 1 : 0;
    const int slot = k.a == first_axis ? 0 : 1;
    if (slot < last_slot[k.kind][k.c])
      return fail(OAFDTD_E_INVALID, "CPML corrections of a component must come in ascending axis order");
    last_slot[k.kind][k.c] = slot;
    oafdtd::CpmlTerm<real>& term_ref = k.kind == 0 ? sw.ecorr[k.c][slot] : sw.hcorr[k.c][slot];
    int side = term_ref.side[0].psi == nullptr ? 0 : (term_ref.side[1].psi == nullptr ? 1 : 2);
    if (side == 2) return fail(OAFDTD_E_INVALID, "more than two CPML sides on one axis");
    for (int ax = 0; ax < 3; ++ax)
      if (k.lo[ax] < 1 || k.hi[ax] <= k.lo[ax] || k.hi[ax] > len[ax])
        return fail(OAFDTD_E_INVALID, "CPML box out of range");
    // psi spans the slab along the derivative axis and the full storage extent on the others
    long long vol = B;
    for (int ax = 0; ax < 3; ++ax) vol *= (ax == k.a) ? (k.hi[ax] - k.lo[ax]) : len[ax];
    real* psi = nullptr;
    int rc = alloc(&psi, (size_t)vol);
    if (rc) return rc;
    keep_state(psi, (size_t)vol);
    term_ref.axis = k.a;
    term_ref.src = k.b;
    term_ref.sign = (real)k.sign;
    term_ref.side[side].psi = psi;
    for (int ax = 0; ax < 3; ++ax) {
      term_ref.side[side].lo[ax] = k.lo[ax];
      term_ref.side[side].hi[ax] = k.hi[ax];
    }
  }
  sw.dtmu = (real)p.dtmu;
  sw.nx = nx;
  sw.ny = ny;
  sw.nz = nz;
  sw.X = X;
  sw.Y = Y;
  sw.bs = bs;
  sw.B = B;
  sw.tile_z = tile_z;
  if (int rc = alloc(&status, 1)) return rc;
  sw.status = status;
  sw.staged = staged;

  timer.mark("cpml");
  // ---- edge list: injection targets and deferred ADE edges (the surface-impedance edges were
  // checked with their bit set above and have their own pass)
  struct EdgeRec {
    int comp;
    long long flat;
    std::vector<int> inj;
  };
  std::map<std::pair<int, long long>, EdgeRec> edges;
  for (const std::pair<int, long long>& cf : deferred) {
    EdgeRec& r = edges[cf];
    r.comp = cf.first;
    r.flat = cf.second;
  }
  {
    // within one channel a repeated edge keeps only its last entry (NumPy fancy-index +=)
    std::map<std::tuple<int, int, long long>, int64_t> last_in_chan;
    for (int64_t t = 0; t < p.n_inj; ++t) last_in_chan[{p.inj_chan[t], p.inj_comp[t], p.inj_flat[t]}] = t;
    for (int64_t t = 0; t < p.n_inj; ++t) {
      if (last_in_chan[{p.inj_chan[t], p.inj_comp[t], p.inj_flat[t]}] != t) continue;
      EdgeRec& r = edges[{p.inj_comp[t], p.inj_flat[t]}];
      r.comp = p.inj_comp[t];
      r.flat = p.inj_flat[t];
      r.inj.push_back((int)t);
    }
  }
  {
    std::vector<int8_t> comp;
    std::vector<long long> flat, dflat;
    std::vector<int8_t> dcomp;
    std::vector<int> ibeg, iend, dslot, ichan;
    std::vector<double> iamp;
    std::vector<std::pair<int, long long>> def_sorted = deferred;
    std::sort(def_sorted.begin(), def_sorted.end());
    for (auto& kv : edges) {
      EdgeRec& r = kv.second;
      const bool is_def = std::binary_search(def_sorted.begin(), def_sorted.end(), kv.first);
      comp.push_back((int8_t)r.comp);
      flat.push_back(r.flat);
      ibeg.push_back((int)ichan.size());
      for (int t : r.inj) {
        ichan.push_back(p.inj_chan[t]);
        iamp.push_back(p.inj_amp[t]);
      }
      iend.push_back((int)ichan.size());
      if (is_def) {
        dslot.push_back((int)dflat.size());
        dflat.push_back(r.flat);
        dcomp.push_back((int8_t)r.comp);
      } else {
        dslot.push_back(-1);
      }
    }
    ed.n = (int)comp.size();
    int rc;
    int8_t* d8 = nullptr;
    long long* dll = nullptr;
    int* di = nullptr;
    double* dd = nullptr;
    if ((rc = upload_vec(&d8, comp))) return rc;
    ed.comp = d8;
    if ((rc = upload_vec(&dll, flat))) return rc;
    ed.flat = dll;
    if ((rc = upload_vec(&di, ibeg))) return rc;
    ed.inj_beg = di;
    if ((rc = upload_vec(&di, iend))) return rc;
    ed.inj_end = di;
    if ((rc = upload_vec(&di, dslot))) return rc;
    ed.def_slot = di;
    if ((rc = upload_vec(&di, ichan))) return rc;
    ed.i_chan = di;
    if ((rc = upload_vec(&dd, iamp))) return rc;
    ed.i_amp = dd;
    ed.n_def = pr.n_def = (int)dflat.size();
    if ((rc = upload_vec(&dll, dflat))) return rc;
    ed.def_flat = pr.def_flat = dll;
    if ((rc = upload_vec(&d8, dcomp))) return rc;
    ed.def_comp = pr.def_comp = d8;
    real* eold = nullptr;
    if ((rc = alloc(&eold, (size_t)B * std::max<size_t>(dflat.size(), 1)))) return rc;
    keep_state(eold, (size_t)B * std::max<size_t>(dflat.size(), 1));
    ed.eold = pr.eold = eold;
  }
  // surface impedance: one packed record per edge, in the compiled order
  {
    const int ns = (int)p.sibc_n, SP = p.sibc_poles;
    if (bs > 2147483647LL) return fail(OAFDTD_E_INVALID, "storage larger than 2^31 cells per member");
    sb.n = ns;
    sb.P = SP;
    std::vector<oafdtd::SibcEdge<real>> recs((size_t)std::max(ns, 1));
    for (int64_t k = 0; k < p.sibc_n; ++k) {
      oafdtd::SibcEdge<real>& r = recs[k];
      r.flat = (int)p.sibc_flat[k];
      r.comp = (unsigned char)p.sibc_comp[k];
      r.mat = p.sibc_mat[k];
      for (int q = 0; q < 2; ++q) {
        r.sign[q] = (real)p.sibc_hsign[2 * k + q];
        r.hflat[q] = r.sign[q] != (real)0 ? (int)p.sibc_hflat[2 * k + q] : 0;
      }
      r.hcomp0 = (unsigned char)p.sibc_hcomp[2 * k];
      r.hcomp1 = (unsigned char)p.sibc_hcomp[2 * k + 1];
      r.pad = 0;
    }
    std::vector<real> r0(std::max(p.sibc_nmat, 1)), alpha(std::max(p.sibc_nmat * SP, 1)), gp(std::max(SP, 1));
    for (int m = 0; m < p.sibc_nmat; ++m) {
      r0[m] = (real)p.sibc_r0[m];
      for (int q = 0; q < SP; ++q) alpha[m * SP + q] = (real)(p.sibc_rp[m * SP + q] * p.sibc_cp[q]);
    }
    for (int q = 0; q < SP; ++q) gp[q] = (real)p.sibc_gp[q];
    int rc;
    oafdtd::SibcEdge<real>* dre = nullptr;
    real* dr = nullptr;
    if ((rc = upload_vec(&dre, recs))) return rc;
    sb.edge = dre;
    if ((rc = upload_vec(&dr, r0))) return rc;
    sb.r0 = dr;
    if ((rc = upload_vec(&dr, alpha))) return rc;
    sb.alpha = dr;
    if ((rc = upload_vec(&dr, gp))) return rc;
    sb.gp = dr;
    if ((rc = alloc(&dr, (size_t)B * std::max(ns, 1)))) return rc;
    keep_state(dr, (size_t)B * std::max(ns, 1));
    sb.jprev = dr;
    if ((rc = alloc(&dr, (size_t)SP * B * std::max(ns, 1)))) return rc;
    keep_state(dr, (size_t)SP * B * std::max(ns, 1));
    sb.v = dr;
  }
  // sources
  {
    int rc;
    double* dd = nullptr;
    const size_t nw = (size_t)p.n_chan * (size_t)p.max_steps;
    if ((rc = upload(&dd, p.wave, p.n_chan > 0 ? nw : 0))) return rc;
    ed.wave = dd;
    if ((rc = upload(&dd, p.drive, (size_t)B * p.n_chan))) return rc;
    ed.drive = dd;
    ed.n_chan = p.n_chan;
    ed.max_steps = p.max_steps;
  }
  bind(0, 0);
  ed.bs = pr.bs = sb.bs = bs;
  sb.B = B;
  ed.X = X;
  ed.Y = Y;
  ed.B = pr.B = en.B = B;
  if (int rc = alloc(&step_base, 1)) return rc;
  keep_state(step_base, 1);
  ed.step_base = pr.step_base = step_base;

  timer.mark("edges_sibc");
  // ---- probes
  {
    n_probe = p.n_probe;
    n_freq = p.n_freq;
    record_series = p.record_series;
    std::vector<int> kinds(p.probe_kind, p.probe_kind + p.n_probe);
    std::vector<int> comps(p.probe_comp, p.probe_comp + p.n_probe);
    std::vector<long long> off(p.probe_off, p.probe_off + p.n_probe + 1);
    std::vector<int> lists[2];
    for (int q = 0; q < p.n_probe; ++q) {
      if (kinds[q] < 0 || kinds[q] > 1 || comps[q] < 0 || comps[q] > 2 || off[q + 1] < off[q])
        return fail(OAFDTD_E_INVALID, "bad probe");
      lists[kinds[q]].push_back(q);
    }
    const long long total = p.n_probe > 0 ? off[p.n_probe] : 0;
    for (long long e = 0; e < total; ++e)
      if (!in_range(p.probe_flat[e])) return fail(OAFDTD_E_INVALID, "probe point out of range");
    int rc;
    int* di = nullptr;
    long long* dll = nullptr;
    double* dd = nullptr;
    if ((rc = upload_vec(&di, kinds))) return rc;
    pr.kind = di;
    if ((rc = upload_vec(&di, comps))) return rc;
    pr.comp = di;
    if ((rc = upload_vec(&dll, off))) return rc;
    pr.off = dll;
    if ((rc = upload(&dll, reinterpret_cast<const long long*>(p.probe_flat), (size_t)total))) return rc;
    pr.flat = dll;
    if ((rc = upload(&dd, p.probe_w, (size_t)total))) return rc;
    pr.w = dd;
    for (int k = 0; k < 2; ++k) {
      if ((rc = upload_vec(&di, lists[k]))) return rc;
      pr.list[k] = di;
      pr.n_kind[k] = (int)lists[k].size();
    }
    pr.n_probe = p.n_probe;
    pr.n_freq = p.n_freq;
    if ((rc = upload(&dd, p.omega, (size_t)p.n_freq))) return rc;
    pr.omega = dd;
    pr.dt = p.dt;
    double2* acc = nullptr;
    if ((rc = alloc(&acc, (size_t)std::max(p.n_probe, 1) * B * std::max(p.n_freq, 1)))) return rc;
    keep_state(acc, (size_t)std::max(p.n_probe, 1) * B * std::max(p.n_freq, 1));
    pr.acc = acc;
    pr.max_steps = p.max_steps;
    pr.series = nullptr;
    if (p.record_series && p.n_probe > 0) {
      double* ser = nullptr;
      if ((rc = alloc(&ser, (size_t)p.n_probe * B * p.max_steps))) return rc;
      keep_state(ser, (size_t)p.n_probe * B * p.max_steps);
      pr.series = ser;
    }
  }
  timer.mark("probes");
  // ---- energy
  {
    en.X = X;
    en.Y = Y;
    en.Z = Z;
    const double* nodew[3];
    const double* cellw[3];
    for (int a = 0; a < 3; ++a) {
      double* d = nullptr;
      int rc = upload(&d, p.node_w[a], (size_t)len[a]);
      if (rc) return rc;
      nodew[a] = d;
      rc = upload(&d, p.cell_w[a], (size_t)len[a]);
      if (rc) return rc;
      cellw[a] = d;
    }
    for (int cc = 0; cc < 6; ++cc) {
      const int c = cc % 3;
      const bool is_e = cc < 3;
      for (int a = 0; a < 3; ++a) {
        const bool node = is_e ? (a != c) : (a == c);
        en.w[cc][a] = node ? nodew[a] : cellw[a];
      }
    }
    if (sizeof(real) == 4) {  // the float-float weights of the float32 energy sum
      auto split = [](double d) {
        const float hi = (float)d;
        return make_float2(hi, (float)(d - (double)hi));
      };
      const double wscale = std::ldexp(1.0, oafdtd::kEnergyWShift);
      for (int cc = 0; cc < 6; ++cc) {
        const int c = cc % 3;
        const bool is_e = cc < 3;
        const double* hw[3];
        for (int a = 0; a < 3; ++a) hw[a] = (is_e ? (a != c) : (a == c)) ? p.node_w[a] : p.cell_w[a];
        std::vector<float2> wx((size_t)X), wyz((size_t)Z * Y);
        for (int i = 0; i < X; ++i) wx[i] = split(hw[0][i]);
        for (int k = 0; k < Z; ++k)
          for (int j = 0; j < Y; ++j) wyz[(size_t)k * Y + j] = split(hw[1][j] * hw[2][k] * wscale);
        float2* d = nullptr;
        if (int rc = upload_vec(&d, wx)) return rc;
        en.wxf[cc] = d;
        if (int rc = upload_vec(&d, wyz)) return rc;
        en.wyzf[cc] = d;
      }
      std::vector<float2> ef(t_eps.size());
      for (size_t m = 0; m < t_eps.size(); ++m) ef[m] = split(t_eps[m]);
      float2* d = nullptr;
      if (int rc = upload_vec(&d, ef)) return rc;
      en.epsf = d;
    }
    if (int rc = alloc(&energy_partial, (size_t)6 * oafdtd::kEnergyBlocks)) return rc;
    if (int rc = alloc(&energy_out, 6)) return rc;
  }
  timer.mark("energy");
  // ---- sweep regions: per kind, an interior box free of CPML cells (staged sweeps) and the slab
  // boxes around it (slab kernel)
  {
    const int Q = X / 4;
    whole = oafdtd::Span3{0, Q, 1, ny + 2, 1, nz + 2};
    int lo_h[3] = {0, 1, 1};  // the first H cell past the low CPML slabs, per axis
    for (int kind = 0; kind < 2; ++kind) {
      int lo[3] = {0, 1, 1}, hi[3] = {X, ny + 2, nz + 2};
      for (int c = 0; c < 3; ++c)
        for (int t = 0; t < 2; ++t) {
          const oafdtd::CpmlTerm<real>& T = kind == 0 ? sw.ecorr[c][t] : sw.hcorr[c][t];
          for (int sd = 0; sd < 2; ++sd) {
            const oafdtd::CpmlSide<real>& S = T.side[sd];
            if (S.psi == nullptr) continue;
            const int ax = T.axis;
            if (S.lo[ax] <= 1)
              lo[ax] = std::max(lo[ax], S.hi[ax]);
            else
              hi[ax] = std::min(hi[ax], S.lo[ax]);
          }
        }
      // The interior starts on an even quad: its TMA boxes then start at a multiple of 8 cells,
      // 16 bytes for the uint16 index boxes as for the field boxes.
      const int qa = std::min(((lo[0] + 3) / 4 + 1) & ~1, Q), qb = std::max(std::min(hi[0] / 4, Q), qa);
      const int ja = std::min(std::max(lo[1], 1), ny + 2), jb = std::max(std::min(hi[1], ny + 2), ja);
      const int ka = std::min(std::max(lo[2], 1), nz + 2), kb = std::max(std::min(hi[2], nz + 2), ka);
      inner_staged[kind] = oafdtd::Span3{qa, qb, ja, jb, ka, kb};
      // the z-slab planes of the interior's x-y extent hold z corrections only: staged too
      zin_staged[kind][0] = oafdtd::Span3{qa, qb, ja, jb, 1, ka};
      zin_staged[kind][1] = oafdtd::Span3{qa, qb, ja, jb, kb, nz + 2};
      for (int zr = 0; zr < 2; ++zr)
        for (int cc = 0; cc < 2; ++cc) {
          zsd[kind][zr][cc] = -1;
          const oafdtd::CpmlTerm<real>& T = kind == 0 ? sw.ecorr[cc][1] : sw.hcorr[cc][1];
          if (T.axis != 2) continue;
          for (int sd = 0; sd < 2; ++sd) {
            const oafdtd::CpmlSide<real>& S = T.side[sd];
            if (S.psi != nullptr && (S.lo[2] <= 1) == (zr == 0)) zsd[kind][zr][cc] = sd;
          }
        }
      // the slab kernel: the y and x slabs over every plane
      const oafdtd::Span3 boxes[4] = {{0, Q, 1, ja, 1, nz + 2},
                                      {0, Q, jb, ny + 2, 1, nz + 2},
                                      {0, qa, ja, jb, 1, nz + 2},
                                      {qb, Q, ja, jb, 1, nz + 2}};
      int n = 0;
      for (const oafdtd::Span3& bx : boxes)
        if (bx.q1 > bx.q0 && bx.j1 > bx.j0 && bx.k1 > bx.k0) slab_staged[kind][n++] = bx;
      n_slab_staged[kind] = n;
      if (kind == 1)
        for (int ax = 0; ax < 3; ++ax) lo_h[ax] = lo[ax];
    }
    // The fused box: inside both interiors; its first cell on each axis one past the first H
    // cell without corrections and past index 1 (the halo cells the fused sweep recomputes are
    // then plain H cells, no ghosts); its last cell below the wall node n + 1 (no PMC mirror
    // planes inside); the x origin an even quad (16-byte TMA boxes, as the staged sweeps).
    {
      const oafdtd::Span3& e = inner_staged[0];
      const oafdtd::Span3& h = inner_staged[1];
      int q0 = std::max(std::max(e.q0, h.q0), std::max((lo_h[0] + 4) / 4, 2));
      q0 += q0 & 1;
      const int q1 = std::min(std::min(e.q1, h.q1), (nx + 1) / 4);
      const int j0 = std::max(std::max(e.j0, h.j0), std::max(lo_h[1] + 1, 2));
      const int j1 = std::min(std::min(e.j1, h.j1), ny + 1);
      const int k0 = std::max(std::max(e.k0, h.k0), std::max(lo_h[2] + 1, 2));
      const int k1 = std::min(std::min(e.k1, h.k1), nz + 1);
      if (q1 > q0 && j1 > j0 && k1 > k0) {
        fused_box = oafdtd::Span3{q0, q1, j0, j1, k0, k1};
        for (int kind = 0; kind < 2; ++kind) {
          zin_fused[kind][0] = oafdtd::Span3{q0, q1, j0, j1, 1, k0};
          zin_fused[kind][1] = oafdtd::Span3{q0, q1, j0, j1, k1, nz + 2};
          const oafdtd::Span3 boxes[4] = {{0, Q, 1, j0, 1, nz + 2},
                                          {0, Q, j1, ny + 2, 1, nz + 2},
                                          {0, q0, j0, j1, 1, nz + 2},
                                          {q1, Q, j0, j1, 1, nz + 2}};
          int n = 0;
          for (const oafdtd::Span3& bx : boxes)
            if (bx.q1 > bx.q0 && bx.j1 > bx.j0 && bx.k1 > bx.k0) slab_fused[kind][n++] = bx;
          n_slab_fused[kind] = n;
        }
      }
    }
    use_regions(staged);
    std::string why;
    tma_ok = oafdtd::encode_sweep_maps<real>(sw, &maps_p[0], &why);
    if (!tma_ok && staged == 2) {
      staged = 1;
      use_regions(staged);
    }
    // the fused sweep reads the combined table from shared memory (kCoefSmem entries at most)
    if (tma_ok && fused_box.k1 > fused_box.k0 && sw.n_coef <= oafdtd::kCoefSmem) {
      oafdtd::FusedMaps probe{};
      fused_ok = oafdtd::encode_fused_maps<real>(sw, &probe, &why);
    }
  }
  timer.mark("regions_maps");
  // ---- traffic model: algorithmic bytes per time step and kernel class, all batch members.
  // Sweeps: read 3 source components, read-modify-write 3 updated ones (9 values) per grid cell
  // and member; E also the three uint16 indices per cell and J read+write (2 P values) per
  // dispersive edge; psi read+write per correction cell, in the class of the kernel that applies
  // it. The fused sweep: read E and H, write E and H (12 values) per cell and member, the indices
  // and J. Edges: surface-impedance v_p and J_prev read+write, two H samples and the E write per
  // edge. The step's model bytes are those of the separate sweeps (72 + 6 / B bytes per plain
  // cell-update in float32), whatever the variant moves.
  {
    // the Debye edge counts here; the rest on a host thread of its own, with the index arrays
    // and the correction list moved or copied into it
    double n_all = 0.0, n_def = 0.0;
    for (int c = 0; c < 3; ++c) {
      std::vector<long long> nd(kMaxParts, 0);
      parallel_parts((long long)ade_edges[c].size(), [&](long long b0, long long e0, int t) {
        long long n = 0;
        for (long long e = b0; e < e0; ++e) n += ade_edges[c][e].defer ? 1 : 0;
        nd[t] = n;
      });
      long long d = 0;
      for (long long n : nd) d += n;
      n_def += (double)d;
      n_all += (double)((long long)ade_edges[c].size() - d);
    }
    std::vector<oafdtd_correction> corr(p.corr, p.corr + p.n_corr);
    std::array<std::vector<uint16_t>, 3> mats{std::move(host_mat[0]), std::move(host_mat[1]), std::move(host_mat[2])};
    const double sibc_n = (double)p.sibc_n, sibc_poles = (double)p.sibc_poles;
    traffic = std::async(std::launch::async, [this, corr = std::move(corr), mats = std::move(mats), n_all, n_def,
                                              sibc_n, sibc_poles, P, ade_lo, ade_hi]() {
    const std::array<std::vector<uint16_t>, 3>& host_mat = mats;
    const double rb = sizeof(real);
    auto cells_in = [&](const oafdtd::Span3& s) {
      const double x = std::max(0, std::min(4 * s.q1, nx + 1) - std::max(4 * s.q0, 1));
      const double y = std::max(0, std::min(s.j1, ny + 1) - std::max(s.j0, 1));
      const double z = std::max(0, std::min(s.k1, nz + 1) - std::max(s.k0, 1));
      return x * y * z;
    };
    // psi bytes of one kind's corrections inside a box (all of them for the whole domain)
    auto psi_in = [&](int kind, const oafdtd::Span3& z) {
      double out = 0.0;
      for (const oafdtd_correction& k : corr) {
        if (k.kind != kind) continue;
        const double x = std::max(0, std::min(4 * z.q1, (int)k.hi[0]) - std::max(4 * z.q0, (int)k.lo[0]));
        const double y = std::max(0, std::min(z.j1, (int)k.hi[1]) - std::max(z.j0, (int)k.lo[1]));
        const double zz = std::max(0, std::min(z.k1, (int)k.hi[2]) - std::max(z.k0, (int)k.lo[2]));
        out += x * y * zz * (double)B * 2.0 * rb;
      }
      return out;
    };
    // Debye current bytes of the dispersive (not deferred) edges inside a box. One pass over the
    // index arrays counts them per storage row (all three components) for each distinct x range
    // of the boxes asked about; a box then sums its rows.
    const double jv = (double)B * P * 2.0 * rb;
    const oafdtd::Span3* jboxes[6] = {&inner_staged[0], &zin_staged[0][0], &zin_staged[0][1],
                                      &fused_box,       &zin_fused[0][0],  &zin_fused[0][1]};
    std::vector<std::pair<int, int>> xr;  // distinct x ranges [x0, x1)
    for (const oafdtd::Span3* b : jboxes) {
      const std::pair<int, int> r{4 * b->q0, 4 * b->q1};
      if (b->q1 > b->q0 && std::find(xr.begin(), xr.end(), r) == xr.end()) xr.push_back(r);
    }
    const long long R = (long long)Z * Y;
    std::vector<long long> rowcnt(xr.size() * (size_t)R, 0);
    if (ade_hi > ade_lo && !xr.empty())
      parallel_parts(R, [&](long long b0, long long e0, int) {
        for (long long r = b0; r < e0; ++r)
          for (int c = 0; c < 3; ++c) {
            const uint16_t* row = host_mat[c].data() + r * X;
            for (size_t x = 0; x < xr.size(); ++x) {
              long long n = 0;
              for (int i = xr[x].first; i < xr[x].second; ++i) n += row[i] >= ade_lo && row[i] < ade_hi;
              rowcnt[x * (size_t)R + r] += n;
            }
          }
      });
    auto j_in = [&](const oafdtd::Span3& bx) {
      if (ade_hi <= ade_lo || bx.q1 <= bx.q0 || bx.j1 <= bx.j0 || bx.k1 <= bx.k0) return 0.0;
      const size_t x = (size_t)(std::find(xr.begin(), xr.end(), std::pair<int, int>{4 * bx.q0, 4 * bx.q1}) - xr.begin());
      double n_in = 0.0;
      for (int k = bx.k0; k < bx.k1; ++k)
        for (int j = bx.j0; j < bx.j1; ++j) n_in += (double)rowcnt[x * (size_t)R + (size_t)k * Y + j];
      return n_in * jv;
    };
    const oafdtd::Span3 all{0, X / 4, 0, Y, 0, Z};
    const double cells = (double)nx * ny * nz;
    const double j_all = n_all * jv, j_def = n_def * jv;
    const double psi_all[2] = {psi_in(0, all), psi_in(1, all)};
    const double per_h = B * 9.0 * rb, per_e = B * 9.0 * rb + 6.0, per_f = B * 12.0 * rb + 6.0;
    const double edges = sibc_n * B * (2.0 * rb * (1 + sibc_poles) + 3.0 * rb) + j_def;
    // classes: h_sweep, h_slab, ghosts, pre_e, e_sweep, e_slab, edges, probe_e, fused
    {  // variants 1 and 2: staged interior and z-slab boxes, slab boxes around them
      double* st = class_bytes[1];
      const double hc = cells_in(inner_staged[1]) + cells_in(zin_staged[1][0]) + cells_in(zin_staged[1][1]);
      const double ec = cells_in(inner_staged[0]) + cells_in(zin_staged[0][0]) + cells_in(zin_staged[0][1]);
      const double hp = psi_in(1, zin_staged[1][0]) + psi_in(1, zin_staged[1][1]);
      const double ep = psi_in(0, zin_staged[0][0]) + psi_in(0, zin_staged[0][1]);
      const double ej = j_in(inner_staged[0]) + j_in(zin_staged[0][0]) + j_in(zin_staged[0][1]);
      st[0] = hc * per_h + hp;
      st[1] = (cells - hc) * per_h + psi_all[1] - hp;
      st[4] = ec * per_e + ej + ep;
      st[5] = (cells - ec) * per_e + psi_all[0] - ep + (j_all - ej);
      st[6] = edges;
      model_bytes = 0.0;
      for (int k = 0; k < kClasses; ++k) model_bytes += st[k];
    }
    {  // variant 0: the slab kernel alone
      double* sl = class_bytes[0];
      sl[1] = cells * per_h + psi_all[1];
      sl[5] = cells * per_e + psi_all[0] + j_all;
      sl[6] = edges;
    }
    if (fused_box.k1 > fused_box.k0) {  // variant 3: the fused box, z-slab and slab boxes around it
      double* fu = class_bytes[2];
      const double fc = cells_in(fused_box);
      const double fj = j_in(fused_box);
      const double hz = cells_in(zin_fused[1][0]) + cells_in(zin_fused[1][1]);
      const double ez = cells_in(zin_fused[0][0]) + cells_in(zin_fused[0][1]);
      const double hp = psi_in(1, zin_fused[1][0]) + psi_in(1, zin_fused[1][1]);
      const double ep = psi_in(0, zin_fused[0][0]) + psi_in(0, zin_fused[0][1]);
      const double ej = j_in(zin_fused[0][0]) + j_in(zin_fused[0][1]);
      fu[8] = fc * per_f + fj;
      fu[0] = hz * per_h + hp;
      fu[1] = (cells - fc - hz) * per_h + psi_all[1] - hp;
      fu[4] = ez * per_e + ej + ep;
      fu[5] = (cells - fc - ez) * per_e + psi_all[0] - ep + (j_all - fj - ej);
      fu[6] = edges;
    }
    });
  }
  timer.mark("traffic_model");
  // The fused sweep is the default where it applies and the device has room for the second
  // field buffers; otherwise the staged sweeps run in place.
  if (fused_ok && staged == 2) {
    size_t free_b = 0, total_b = 0;
    OA_CUDA(cudaMemGetInfo(&free_b, &total_b));
    if ((double)free_b > 1.05 * 6.0 * (double)bs * B * sizeof(real))
      if (int rc = set_variant(3)) return rc;
  }
  OA_CUDA(cudaStreamSynchronize(stream));
  timer.mark("device_sync");
  return OAFDTD_OK;
}

// ---------------------------------------------------------------------------- step
// The staged sweep and the slab kernel of one kind. Profiling (ev set) runs them one after the
// other between the class events ev[slot], ev[slot + 1], ev[slot + 2]; otherwise the slab kernel
// is forked onto the side stream and joined back.
template <typename real>
int Engine<real>::sweep_pair(int kind, cudaEvent_t* ev, int slot, unsigned rec, const oafdtd::SweepMaps& mp,
                             int pre_e_off) {
  const char* names[2][2] = {{"e_sweep: ", "e_slab: "}, {"h_sweep: ", "h_slab: "}};
  const bool fork = ev == nullptr && sw.staged;
  cudaError_t err;
  if (fork) {
    OA_CUDA(cudaEventRecord(fork_ev, stream));
    OA_CUDA(cudaStreamWaitEvent(side, fork_ev, 0));
    err = oafdtd::launch_slab<real>(sw, kind, side);
    if (err != cudaSuccess) return fail(OAFDTD_E_CUDA, std::string(names[kind][1]) + cudaGetErrorString(err));
    OA_CUDA(cudaEventRecord(join_ev, side));
    err = oafdtd::launch_staged_sweep<real>(sw, mp, stream, kind == 1);
    if (err != cudaSuccess) return fail(OAFDTD_E_CUDA, std::string(names[kind][0]) + cudaGetErrorString(err));
    if (pre_e_off >= 0) {  // the fused step's pre_e, after the (shorter) staged sweep, beside the slab kernel
      err = oafdtd::launch_pre_e<real>(pr, pre_e_off, stream);
      if (err != cudaSuccess) return fail(OAFDTD_E_CUDA, std::string("pre_e: ") + cudaGetErrorString(err));
    }
    OA_CUDA(cudaStreamWaitEvent(stream, join_ev, 0));
    return OAFDTD_OK;
  }
  if (ev) OA_CUDA(cudaEventRecordWithFlags(ev[slot], stream, rec));
  if (sw.staged) {
    err = oafdtd::launch_staged_sweep<real>(sw, mp, stream, kind == 1);
    if (err != cudaSuccess) return fail(OAFDTD_E_CUDA, std::string(names[kind][0]) + cudaGetErrorString(err));
  }
  if (ev) OA_CUDA(cudaEventRecordWithFlags(ev[slot + 1], stream, rec));
  err = oafdtd::launch_slab<real>(sw, kind, stream);
  if (err != cudaSuccess) return fail(OAFDTD_E_CUDA, std::string(names[kind][1]) + cudaGetErrorString(err));
  if (ev) OA_CUDA(cudaEventRecordWithFlags(ev[slot + 2], stream, rec));
  return OAFDTD_OK;
}

// One time step (parts 3) or one half of it (1: H, 2: E), from the current buffers. Profiling
// records the class events of the step: ev[9] at its start, ev[0..8] after the fused sweep,
// h_sweep, h_slab, ghosts, pre_e, e_sweep, e_slab, edges and probe_e. In the fused variant the
// H part outside the fused box runs beside the fused sweep, on the side stream, and the buffers
// swap after the step (after each half for the halves, which run the separate sweeps).
template <typename real>
int Engine<real>::launch_step(int off, cudaEvent_t* ev, bool capturing, int parts) {
  cudaError_t err;
  // inside a stream capture an event record becomes a graph node only with the external flag
  const unsigned rec = capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
  const int p = cur[0];
  const bool fused = staged == 3 && parts == 3;
  // In a fused step E^n stays in the current buffers for the whole step, so pre_e (the H probes
  // at (n + 1/2) dt, E^n of the deferred Debye edges) can wait until the E z-slab sweep is
  // launched and run beside the E slab kernel; the edge pass, which uses what it saves, comes
  // after both. In place (the other variants, the halves) it must precede the E sweeps.
  const bool late_pre_e = fused && ev == nullptr;
  // In a fused step without PMC mirrors, the E work whose stencil reads no H of the fused box (the
  // slab and z-slab boxes below it on some axis) starts on the side stream as soon as the H work
  // outside the box is done, beside the rest of the H phase; the rest follows the fused sweep.
  const bool early_e = late_pre_e && pmc_mask == 0;
  use_regions(fused ? 3 : (staged == 3 ? 2 : staged));
  bind(p, p);
  const oafdtd::SweepMaps& mp = maps_p[p];
  if (ev) OA_CUDA(cudaEventRecordWithFlags(ev[9], stream, rec));
  if (fused) {
    if (ev) {
      err = oafdtd::launch_fused_sweep<real>(sw, fmaps[p], stream);
      if (err != cudaSuccess) return fail(OAFDTD_E_CUDA, std::string("fused: ") + cudaGetErrorString(err));
      if (int rc = sweep_pair(1, ev, 0, rec, mp)) return rc;
    } else {
      // The H cells outside the fused box read only the current buffers: the H z-slab sweep and
      // the H slab kernel run beside the fused sweep, on the side stream, launched after it so
      // its one wave of blocks is placed first (the side kernels take the SMs it leaves and its
      // tail). Launched before it, or all three on one stream, the step took 0.886 and 0.891 ms
      // against 0.871 ms (400x400x120, 128 planes per block).
      OA_CUDA(cudaEventRecord(fork_ev, stream));
      err = oafdtd::launch_fused_sweep<real>(sw, fmaps[p], stream);
      if (err != cudaSuccess) return fail(OAFDTD_E_CUDA, std::string("fused: ") + cudaGetErrorString(err));
      OA_CUDA(cudaStreamWaitEvent(side, fork_ev, 0));
      err = oafdtd::launch_staged_sweep<real>(sw, mp, side, true);
      if (err == cudaSuccess) err = oafdtd::launch_slab<real>(sw, 1, side);
      if (err != cudaSuccess) return fail(OAFDTD_E_CUDA, std::string("h_sweep: ") + cudaGetErrorString(err));
      OA_CUDA(cudaEventRecord(join_ev, side));
      if (early_e) {  // the E work that needs only the H just done, on the side stream at once
        const oafdtd::SweepArgs<real> lo = e_part(true);
        err = oafdtd::launch_slab<real>(lo, 0, side);
        if (err == cudaSuccess) err = oafdtd::launch_staged_sweep<real>(lo, mp, side, false);
        if (err != cudaSuccess) return fail(OAFDTD_E_CUDA, std::string("early E: ") + cudaGetErrorString(err));
        OA_CUDA(cudaEventRecord(ejoin_ev, side));
      }
      OA_CUDA(cudaStreamWaitEvent(stream, join_ev, 0));
    }
  } else if (parts & 1) {
    if (ev) OA_CUDA(cudaEventRecordWithFlags(ev[0], stream, rec));
    if (int rc = sweep_pair(1, ev, 0, rec, mp)) return rc;
  }
  if (parts & 1) {
    if (pmc_mask) {
      err = oafdtd::launch_ghosts<real>(sw.Ho, pmc_mask, nx, ny, nz, X, Y, B, stream);
      if (err != cudaSuccess) return fail(OAFDTD_E_CUDA, std::string("ghosts: ") + cudaGetErrorString(err));
    }
    if (ev) OA_CUDA(cudaEventRecordWithFlags(ev[3], stream, rec));
    if (!late_pre_e) {
      err = oafdtd::launch_pre_e<real>(pr, off, stream);
      if (err != cudaSuccess) return fail(OAFDTD_E_CUDA, std::string("pre_e: ") + cudaGetErrorString(err));
    }
  }
  if (parts & 2) {
    if (early_e) {  // the rest of the E work on the main stream, then pre_e, then both joined
      const oafdtd::SweepArgs<real> hi = e_part(false);
      err = oafdtd::launch_slab<real>(hi, 0, stream);
      if (err == cudaSuccess) err = oafdtd::launch_staged_sweep<real>(hi, mp, stream, false);
      if (err == cudaSuccess) err = oafdtd::launch_pre_e<real>(pr, off, stream);
      if (err != cudaSuccess) return fail(OAFDTD_E_CUDA, std::string("late E: ") + cudaGetErrorString(err));
      OA_CUDA(cudaStreamWaitEvent(stream, ejoin_ev, 0));
    } else if (int rc = sweep_pair(0, ev, 4, rec, mp, late_pre_e ? off : -1)) {
      return rc;
    }
    err = oafdtd::launch_sibc<real>(sb, stream);
    if (err == cudaSuccess) err = oafdtd::launch_edges<real>(ed, off, stream);
    if (err != cudaSuccess) return fail(OAFDTD_E_CUDA, std::string("edges: ") + cudaGetErrorString(err));
    if (ev) OA_CUDA(cudaEventRecordWithFlags(ev[7], stream, rec));
    err = oafdtd::launch_probe_e<real>(pr, off, stream);
    if (err != cudaSuccess) return fail(OAFDTD_E_CUDA, std::string("probe_e: ") + cudaGetErrorString(err));
    if (ev) OA_CUDA(cudaEventRecordWithFlags(ev[8], stream, rec));
  }
  if (staged == 3) {  // the other buffers now hold the newer field(s)
    if (parts & 1) cur[1] ^= 1;
    if (parts & 2) cur[0] ^= 1;
  }
  return OAFDTD_OK;
}

template <typename real>
int Engine<real>::capture() {
  if (graph_exec) {
    cudaGraphExecDestroy(graph_exec);
    graph_exec = nullptr;
  }
  graph_ready = false;
  graph_kernels = 0;
  cudaGraph_t graph = nullptr;
  // a capture launches nothing: the buffer state it walks through is put back afterwards (a whole
  // chunk is an even number of steps, so a replay leaves the buffers where it found them)
  const int cur0[2] = {cur[0], cur[1]};
  graph_parity = cur[0];
  OA_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
  int rc = OAFDTD_OK;
  for (int o = 0; o < oafdtd::kChunk && rc == OAFDTD_OK; ++o)
    rc = launch_step(o, profiling ? &events[(size_t)o * (kClasses + 1)] : nullptr, true);
  if (rc == OAFDTD_OK) {
    cudaError_t err = oafdtd::launch_bump(step_base, oafdtd::kChunk, stream);
    if (err != cudaSuccess) rc = fail(OAFDTD_E_CUDA, cudaGetErrorString(err));
  }
  cur[0] = cur0[0];
  cur[1] = cur0[1];
  cudaError_t err = cudaStreamEndCapture(stream, &graph);
  if (rc != OAFDTD_OK) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (err != cudaSuccess) return fail(OAFDTD_E_CUDA, std::string("graph capture: ") + cudaGetErrorString(err));
  {
    size_t n = 0;
    err = cudaGraphGetNodes(graph, nullptr, &n);
    std::vector<cudaGraphNode_t> nodes(n);
    if (err == cudaSuccess && n) err = cudaGraphGetNodes(graph, nodes.data(), &n);
    int64_t kernels = 0;
    for (size_t q = 0; q < n && err == cudaSuccess; ++q) {
      cudaGraphNodeType t;
      err = cudaGraphNodeGetType(nodes[q], &t);
      if (err == cudaSuccess && t == cudaGraphNodeTypeKernel) ++kernels;
    }
    if (err != cudaSuccess) {
      cudaGraphDestroy(graph);
      return fail(OAFDTD_E_CUDA, std::string("graph nodes: ") + cudaGetErrorString(err));
    }
    graph_kernels = kernels;
  }
  err = cudaGraphInstantiate(&graph_exec, graph, 0);
  cudaGraphDestroy(graph);
  if (err != cudaSuccess) {
    graph_kernels = 0;
    return fail(OAFDTD_E_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(err));
  }
  graph_ready = true;
  return OAFDTD_OK;
}

template <typename real>
int Engine<real>::step(int64_t n) {
  if (int rc = enqueue(n)) return rc;
  return wait();
}

template <typename real>
int Engine<real>::wait() {
  OA_CUDA(cudaSetDevice(device));
  OA_CUDA(cudaStreamSynchronize(stream));
  OA_CUDA(cudaGetLastError());
  return check_status();
}

// Queues n steps on the engine's stream (captured 64-step graphs for whole chunks) and returns;
// wait() synchronises. Profiling reads its events chunk by chunk, so it synchronises per chunk.
template <typename real>
int Engine<real>::enqueue(int64_t n) {
  if (n < 0) return fail(OAFDTD_E_INVALID, "negative step count");
  if (half_pending) return fail(OAFDTD_E_INVALID, "an H half is pending: finish the step with the E half");
  if (steps + n > max_steps) return fail(OAFDTD_E_RANGE, "step count exceeds max_steps (wave table length)");
  OA_CUDA(cudaSetDevice(device));
  if (graph_dirty) {
    graph_ready = false;
    graph_kernels = 0;
    graph_dirty = false;
  }
  if (profiling && events.empty()) {
    events.resize((size_t)oafdtd::kChunk * (kClasses + 1));
    for (auto& e : events) OA_CUDA(cudaEventCreate(&e));
    graph_ready = false;
  }
  sw.tile_z = tile_z;
  if (profiling) {
    for (double& v : prof_ms) v = 0.0;
    prof_steps = 0;
  }
  int64_t done = 0;
  while (done < n) {
    const int64_t start = steps;
    const int take = (int)std::min<int64_t>(n - done, oafdtd::kChunk - start % oafdtd::kChunk);
    if (use_graph && take == oafdtd::kChunk) {
      if (!graph_ready || (staged == 3 && graph_parity != cur[0])) {
        int rc = capture();
        if (rc) return rc;
      }
      OA_CUDA(cudaGraphLaunch(graph_exec, stream));
    } else {
      for (int o = 0; o < take; ++o) {
        int rc = launch_step(o, profiling ? &events[(size_t)o * (kClasses + 1)] : nullptr);
        if (rc) return rc;
      }
      cudaError_t err = oafdtd::launch_bump(step_base, take, stream);
      if (err != cudaSuccess) return fail(OAFDTD_E_CUDA, cudaGetErrorString(err));
    }
    if (profiling) {
      OA_CUDA(cudaStreamSynchronize(stream));
      // class k < 8: ev[k] to ev[k + 1]; the fused sweep: ev[9] to ev[0]; the step: ev[9] to ev[8]
      for (int o = 0; o < take; ++o) {
        cudaEvent_t* ev = &events[(size_t)o * (kClasses + 1)];
        float ms = 0.f;
        for (int k = 0; k < 8; ++k) {
          OA_CUDA(cudaEventElapsedTime(&ms, ev[k], ev[k + 1]));
          prof_ms[k] += ms;
        }
        OA_CUDA(cudaEventElapsedTime(&ms, ev[9], ev[0]));
        prof_ms[8] += ms;
        OA_CUDA(cudaEventElapsedTime(&ms, ev[9], ev[8]));
        prof_ms[kClasses] += ms;
      }
      prof_steps += take;
    }
    steps += take;
    done += take;
  }
  return OAFDTD_OK;
}

template <typename real>
int Engine<real>::check_status() {
  int word = 0;
  OA_CUDA(cudaMemcpy(&word, status, sizeof(word), cudaMemcpyDeviceToHost));
  if (word & oafdtd::kStatusWaitTimeout)
    return fail(OAFDTD_E_TIMEOUT, "a staged sweep gave up waiting for its plane copies (bounded mbarrier wait)");
  return OAFDTD_OK;
}

template <typename real>
int Engine<real>::step_timed(int64_t n, double* ms) {
  OA_CUDA(cudaSetDevice(device));
  if (!t_start) OA_CUDA(cudaEventCreate(&t_start));
  if (!t_stop) OA_CUDA(cudaEventCreate(&t_stop));
  OA_CUDA(cudaEventRecord(t_start, stream));
  int rc = step(n);
  if (rc) return rc;
  OA_CUDA(cudaEventRecord(t_stop, stream));
  OA_CUDA(cudaEventSynchronize(t_stop));
  float f = 0.f;
  OA_CUDA(cudaEventElapsedTime(&f, t_start, t_stop));
  *ms = f;
  return OAFDTD_OK;
}

template <typename real>
int Engine<real>::kernel_times(double* out, int n) {
  for (int k = 0; k < std::min(n, kClasses + 1); ++k) out[k] = prof_steps ? prof_ms[k] / prof_steps : 0.0;
  return OAFDTD_OK;
}

template <typename real>
int Engine<real>::energy(double* out) {
  OA_CUDA(cudaSetDevice(device));
  for (int cc = 0; cc < 6; ++cc) en.F[cc] = field(cc);
  cudaError_t err = oafdtd::launch_energy<real>(en, energy_partial, oafdtd::kEnergyBlocks, energy_out, stream);
  if (err != cudaSuccess) return fail(OAFDTD_E_CUDA, cudaGetErrorString(err));
  double parts[6];
  OA_CUDA(cudaMemcpyAsync(parts, energy_out, sizeof(parts), cudaMemcpyDeviceToHost, stream));
  OA_CUDA(cudaStreamSynchronize(stream));
  double total = 0.0;
  for (int c = 0; c < 3; ++c) {
    total += 0.5 * parts[c];
    total += 0.5 * kMu0 * parts[3 + c];
  }
  *out = total;
  return OAFDTD_OK;
}

template <typename real>
int Engine<real>::dft(double* out) {
  OA_CUDA(cudaSetDevice(device));
  const size_t count = (size_t)n_probe * B * n_freq;
  if (count)
    OA_CUDA(cudaMemcpyAsync(out, pr.acc, count * sizeof(double2), cudaMemcpyDeviceToHost, stream));
  OA_CUDA(cudaStreamSynchronize(stream));
  return OAFDTD_OK;
}

template <typename real>
int Engine<real>::series(double* out) {
  if (!record_series) return fail(OAFDTD_E_INVALID, "the engine was created without record_series");
  OA_CUDA(cudaSetDevice(device));
  for (int q = 0; q < n_probe; ++q)
    for (int b = 0; b < B; ++b)
      if (steps)
        OA_CUDA(cudaMemcpyAsync(out + ((size_t)q * B + b) * steps,
                                pr.series + ((size_t)q * B + b) * max_steps, steps * sizeof(double),
                                cudaMemcpyDeviceToHost, stream));
  OA_CUDA(cudaStreamSynchronize(stream));
  return OAFDTD_OK;
}

template <typename real>
int Engine<real>::fields(int comp, double* out) {
  if (comp < 0 || comp > 5) return fail(OAFDTD_E_INVALID, "component must be 0..5");
  OA_CUDA(cudaSetDevice(device));
  const real* src = field(comp);
  const size_t count = (size_t)bs * B;
  std::vector<real> tmp(count);
  OA_CUDA(cudaMemcpyAsync(tmp.data(), src, count * sizeof(real), cudaMemcpyDeviceToHost, stream));
  OA_CUDA(cudaStreamSynchronize(stream));
  for (size_t k = 0; k < count; ++k) out[k] = (double)tmp[k];
  return OAFDTD_OK;
}

// One half of a time step, eagerly launched (a z-slab decomposition exchanges boundary planes
// between the halves): 0 the H half, 1 the E half, which also advances the step counter.
template <typename real>
int Engine<real>::step_half(int which) {
  OA_CUDA(cudaSetDevice(device));
  if (which != 0 && which != 1) return fail(OAFDTD_E_INVALID, "half must be 0 (H) or 1 (E)");
  if (which == 0) {
    if (half_pending) return fail(OAFDTD_E_INVALID, "an H half is already pending");
    if (steps + 1 > max_steps) return fail(OAFDTD_E_RANGE, "step count exceeds max_steps (wave table length)");
    sw.tile_z = tile_z;
    if (int rc = launch_step(0, nullptr, false, 1)) return rc;
    half_pending = true;
  } else {
    if (!half_pending) return fail(OAFDTD_E_INVALID, "an E half needs its H half first");
    if (int rc = launch_step(0, nullptr, false, 2)) return rc;
    cudaError_t err = oafdtd::launch_bump(step_base, 1, stream);
    if (err != cudaSuccess) return fail(OAFDTD_E_CUDA, cudaGetErrorString(err));
    half_pending = false;
    steps += 1;
  }
  OA_CUDA(cudaStreamSynchronize(stream));
  OA_CUDA(cudaGetLastError());
  return check_status();
}

// One storage plane k of a component, all batch members, (B, Y, X): read into out, or written
// from in.
template <typename real>
int Engine<real>::plane(int comp, int k, double* out, const double* in) {
  if (comp < 0 || comp > 5) return fail(OAFDTD_E_INVALID, "component must be 0..5");
  if (k < 0 || k >= Z) return fail(OAFDTD_E_INVALID, "plane out of range");
  OA_CUDA(cudaSetDevice(device));
  real* f = field(comp);
  const size_t per = (size_t)X * Y;
  std::vector<real> tmp(per * B);
  if (in) {  // written to both buffers: the plane is the same state in either
    for (size_t q = 0; q < tmp.size(); ++q) tmp[q] = (real)in[q];
    for (int buf = 0; buf < (two_buffers ? 2 : 1); ++buf)
      for (int b = 0; b < B; ++b)
        OA_CUDA(cudaMemcpyAsync(fbuf[buf][comp] + (size_t)b * bs + (size_t)k * per, tmp.data() + b * per,
                                per * sizeof(real), cudaMemcpyHostToDevice, stream));
    OA_CUDA(cudaStreamSynchronize(stream));
  } else {
    for (int b = 0; b < B; ++b)
      OA_CUDA(cudaMemcpyAsync(tmp.data() + b * per, f + (size_t)b * bs + (size_t)k * per, per * sizeof(real),
                              cudaMemcpyDeviceToHost, stream));
    OA_CUDA(cudaStreamSynchronize(stream));
    for (size_t q = 0; q < tmp.size(); ++q) out[q] = (double)tmp[q];
  }
  return OAFDTD_OK;
}

// The same plane in the engine's own precision, device to device (dst or src is device memory
// of (B, Y, X) elements, on this GPU or a peer): one copy per batch member on the engine's
// stream, finished before the call returns.
template <typename real>
int Engine<real>::plane_device(int comp, int k, void* dst, const void* src) {
  if (comp < 0 || comp > 5) return fail(OAFDTD_E_INVALID, "component must be 0..5");
  if (k < 0 || k >= Z) return fail(OAFDTD_E_INVALID, "plane out of range");
  OA_CUDA(cudaSetDevice(device));
  const size_t per = (size_t)X * Y;
  for (int b = 0; b < B; ++b) {
    if (src) {  // written to both buffers, as oafdtd_set_plane
      for (int buf = 0; buf < (two_buffers ? 2 : 1); ++buf)
        OA_CUDA(cudaMemcpyAsync(fbuf[buf][comp] + (size_t)b * bs + (size_t)k * per,
                                static_cast<const real*>(src) + b * per, per * sizeof(real), cudaMemcpyDefault,
                                stream));
    } else {
      OA_CUDA(cudaMemcpyAsync(static_cast<real*>(dst) + b * per, field(comp) + (size_t)b * bs + (size_t)k * per,
                              per * sizeof(real), cudaMemcpyDefault, stream));
    }
  }
  OA_CUDA(cudaStreamSynchronize(stream));
  return OAFDTD_OK;
}

// Snapshot layout: a 32-byte header (magic, format version, total bytes, step count), the six
// current field arrays (E0..E2, H0..H2), then every other state buffer in registration order.
// out == in == nullptr: report the size only. A restore writes the fields into both buffers.
constexpr uint64_t kSnapshotMagic = 0x3130504E53444641ull;  // "AFDSNP01" read little-endian
constexpr uint64_t kSnapshotVersion = 2;

template <typename real>
int Engine<real>::snapshot(void* out, int64_t* bytes, const void* in) {
  const size_t fbytes = (size_t)bs * B * sizeof(real);
  uint64_t total = 32 + 6 * (uint64_t)fbytes;
  for (const auto& sb_ : state_bufs) total += sb_.second;
  if (bytes) *bytes = (int64_t)total;
  if (!out && !in) return OAFDTD_OK;
  if (half_pending) return fail(OAFDTD_E_INVALID, "an H half is pending");
  OA_CUDA(cudaSetDevice(device));
  if (out) {
    unsigned char* o = static_cast<unsigned char*>(out);
    const uint64_t head[4] = {kSnapshotMagic, kSnapshotVersion, total, (uint64_t)steps};
    std::memcpy(o, head, sizeof(head));
    size_t at = 32;
    for (int comp = 0; comp < 6; ++comp, at += fbytes)
      OA_CUDA(cudaMemcpyAsync(o + at, field(comp), fbytes, cudaMemcpyDeviceToHost, stream));
    for (const auto& sb_ : state_bufs) {
      OA_CUDA(cudaMemcpyAsync(o + at, sb_.first, sb_.second, cudaMemcpyDeviceToHost, stream));
      at += sb_.second;
    }
    OA_CUDA(cudaStreamSynchronize(stream));
    return OAFDTD_OK;
  }
  const unsigned char* i = static_cast<const unsigned char*>(in);
  uint64_t head[4];
  std::memcpy(head, i, sizeof(head));
  if (head[0] != kSnapshotMagic || head[1] != kSnapshotVersion) return fail(OAFDTD_E_INVALID, "not a snapshot of this format");
  if (head[2] != total) return fail(OAFDTD_E_INVALID, "the snapshot was taken of another problem or configuration");
  if ((int64_t)head[3] > max_steps) return fail(OAFDTD_E_RANGE, "the snapshot's step count exceeds max_steps");
  size_t at = 32;
  for (int comp = 0; comp < 6; ++comp, at += fbytes)
    for (int buf = 0; buf < (two_buffers ? 2 : 1); ++buf)
      OA_CUDA(cudaMemcpyAsync(fbuf[buf][comp], i + at, fbytes, cudaMemcpyHostToDevice, stream));
  for (const auto& sb_ : state_bufs) {
    OA_CUDA(cudaMemcpyAsync(sb_.first, i + at, sb_.second, cudaMemcpyHostToDevice, stream));
    at += sb_.second;
  }
  OA_CUDA(cudaStreamSynchronize(stream));
  steps = (int64_t)head[3];
  return OAFDTD_OK;
}

template <typename real>
int Engine<real>::set_field(int comp, const double* in) {
  if (comp < 0 || comp > 5) return fail(OAFDTD_E_INVALID, "component must be 0..5");
  OA_CUDA(cudaSetDevice(device));
  const size_t count = (size_t)bs * B;
  std::vector<real> tmp(count);
  for (size_t k = 0; k < count; ++k) tmp[k] = (real)in[k];
  for (int buf = 0; buf < (two_buffers ? 2 : 1); ++buf)  // the same state in both buffers
    OA_CUDA(cudaMemcpyAsync(fbuf[buf][comp], tmp.data(), count * sizeof(real), cudaMemcpyHostToDevice, stream));
  OA_CUDA(cudaStreamSynchronize(stream));
  return OAFDTD_OK;
}

template <typename real>
int Engine<real>::sync_buffers() {
  if (!two_buffers) return OAFDTD_OK;
  OA_CUDA(cudaSetDevice(device));
  for (int comp = 0; comp < 6; ++comp) {
    const int c = cur[comp < 3 ? 0 : 1];
    OA_CUDA(cudaMemcpyAsync(fbuf[1 - c][comp], fbuf[c][comp], (size_t)bs * B * sizeof(real), cudaMemcpyDeviceToDevice,
                            stream));
  }
  return OAFDTD_OK;
}

template <typename real>
int Engine<real>::encode_maps() {
  std::string why;
  const int n = two_buffers ? 2 : 1;
  for (int p = 0; p < n; ++p) {
    bind(p, p);
    sw.staged = staged == 3 ? 2 : staged;
    if (tma_ok && !oafdtd::encode_sweep_maps<real>(sw, &maps_p[p], &why)) return fail(OAFDTD_E_CUDA, why);
    if (staged == 3 && !oafdtd::encode_fused_maps<real>(sw, &fmaps[p], &why)) return fail(OAFDTD_E_CUDA, why);
  }
  bind(cur[0], cur[0]);
  return OAFDTD_OK;
}

// Variant 3 allocates the second field buffers (once) and copies the current fields into them:
// cells no sweep writes (ghosts, the padding of the rows) must hold the same values in both.
template <typename real>
int Engine<real>::set_variant(int v) {
  if (v < 0 || v > 3) return fail(OAFDTD_E_INVALID, "variant must be 0..3");
  if (half_pending) return fail(OAFDTD_E_INVALID, "an H half is pending: finish the step with the E half");
  if (v >= 2 && !tma_ok)
    return fail(OAFDTD_E_INVALID, "variants 2 and 3 need TMA descriptors, which the driver did not encode");
  if (v == 3 && !fused_ok)
    return fail(OAFDTD_E_INVALID, "variant 3 needs a fused box (an interior free of CPML cells) and its descriptors");
  OA_CUDA(cudaSetDevice(device));
  if (v == 3 && !two_buffers) {
    for (int comp = 0; comp < 6; ++comp)
      if (int rc = alloc(&fbuf[1][comp], (size_t)bs * B)) return rc;
    two_buffers = true;
  }
  // leaving the fused variant with the newer fields in buffer 1: stay there, in place
  if (v == 3 && staged != 3)
    if (int rc = sync_buffers()) return rc;
  staged = v;
  if (int rc = encode_maps()) return rc;
  OA_CUDA(cudaStreamSynchronize(stream));
  return OAFDTD_OK;
}

// ---------------------------------------------------------------------------- batched sweeps
// Several engines of one precision and one sweep variant stepped as one: every kernel class of
// the step is a single launch over the blocks of all engines (a BatchGrid maps each block to its
// engine and to its block in that engine's own grid), with the engines' arguments in device
// arrays, one set per field-buffer parity. The launches run in the order and on the streams of
// Engine::launch_step, the same kernel bodies on the same arguments, so every engine's fields
// come out bit for bit as when it steps alone. Kernel boundaries order the half steps of every
// engine at once; nothing waits on the device. Whole 64-step chunks replay one captured graph.
struct BatchBase {
  virtual ~BatchBase() = default;
  virtual int enqueue(int64_t n) = 0;
  virtual int wait() = 0;
  int64_t graph_kernels = 0;
};

template <typename real>
struct Batch final : BatchBase {
  struct Launch {
    oafdtd::BatchGrid g{};
    int blocks = 0;
    int key = 0;  // kernel variant of the engines in this launch
  };
  std::vector<Engine<real>*> eng;
  int device = 0, variant = 0;
  cudaStream_t stream = nullptr, side = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr, done_ev = nullptr;
  std::vector<cudaEvent_t> in_ev;
  std::vector<void*> allocs;
  oafdtd::SweepArgs<real>* d_sw[2] = {};
  oafdtd::SweepMaps* d_mp[2] = {};
  oafdtd::FusedMaps* d_fm[2] = {};
  oafdtd::ProbeArgs<real>* d_pr[2] = {};
  oafdtd::SibcArgs<real>* d_sb[2] = {};
  oafdtd::EdgeArgs<real>* d_ed[2] = {};
  oafdtd::SlabLaunch* d_slab[2] = {};  // per kind (the same for both parities)
  long long** d_step_base = nullptr;
  std::vector<oafdtd::SweepArgs<real>> h_sw[2];
  std::vector<Launch> fused, h_inner, h_z, e_inner, e_z, slab_h, slab_e, pre_e, probe_e, edges, sibc;
  bool tma = false;
  cudaGraphExec_t graph[2] = {};

  ~Batch() override {
    for (cudaGraphExec_t g : graph)
      if (g) cudaGraphExecDestroy(g);
    for (void* q : allocs) cudaFree(q);
    for (cudaEvent_t e : in_ev) cudaEventDestroy(e);
    for (cudaEvent_t e : {fork_ev, join_ev, done_ev})
      if (e) cudaEventDestroy(e);
    if (side) cudaStreamDestroy(side);
    if (stream) cudaStreamDestroy(stream);
  }

  template <typename T>
  int upload(T** out, const T* host, size_t count) {
    *out = nullptr;
    void* q = nullptr;
    OA_CUDA(cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T)));
    allocs.push_back(q);
    if (count) OA_CUDA(cudaMemcpy(q, host, count * sizeof(T), cudaMemcpyHostToDevice));
    *out = static_cast<T*>(q);
    return OAFDTD_OK;
  }

  // One launch per kernel variant over the engines' grids (x, y, z blocks; 1-D: x only).
  int plan(const std::vector<dim3>& grids, const std::vector<int>& keys, std::vector<Launch>* out) {
    out->clear();
    const int n = (int)eng.size();
    std::vector<int> done(n, 0);
    for (int i = 0; i < n; ++i) {
      const long long bi = (long long)grids[i].x * grids[i].y * grids[i].z;
      if (done[i] || bi == 0) continue;
      const int key = keys[i];
      // every block of the launch: (engine, x, y, z), x fastest within the engine's grid
      std::vector<int4> blk;
      for (int k = i; k < n; ++k) {
        const dim3 g = grids[k];
        const long long bk = (long long)g.x * g.y * g.z;
        if (done[k] || bk == 0 || keys[k] != key) continue;
        done[k] = 1;
        if ((long long)blk.size() + bk > 2147483647LL) return fail(OAFDTD_E_INVALID, "a batched launch exceeds 2^31 blocks");
        for (unsigned z = 0; z < g.z; ++z)
          for (unsigned y = 0; y < g.y; ++y)
            for (unsigned x = 0; x < g.x; ++x) blk.push_back(make_int4(k, (int)x, (int)y, (int)z));
      }
      Launch L;
      L.blocks = (int)blk.size();
      L.key = key;
      int4* d_blk;
      if (int rc = upload(&d_blk, blk.data(), blk.size())) return rc;
      L.g = oafdtd::BatchGrid{d_blk};
      out->push_back(L);
    }
    return OAFDTD_OK;
  }

  int build(const std::vector<Engine<real>*>& engines) {
    eng = engines;
    const int n = (int)eng.size();
    Engine<real>& e0 = *eng[0];
    device = e0.device;
    variant = e0.staged;
    for (Engine<real>* e : eng) {
      if (e->device != device) return fail(OAFDTD_E_INVALID, "the engines of a batch share one device");
      if (e->staged != variant) return fail(OAFDTD_E_INVALID, "the engines of a batch run one sweep variant");
      if (e->half_pending) return fail(OAFDTD_E_INVALID, "an engine has an H half pending");
      if (e->profiling) return fail(OAFDTD_E_INVALID, "an engine of a batch is in profiling mode");
      if (e->steps != e0.steps || e->cur[0] != e0.cur[0] || e->cur[1] != e0.cur[1])
        return fail(OAFDTD_E_INVALID, "the engines of a batch start at the same step and buffers");
    }
    OA_CUDA(cudaSetDevice(device));
    for (Engine<real>* e : eng) OA_CUDA(cudaStreamSynchronize(e->stream));
    OA_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    OA_CUDA(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
    for (cudaEvent_t* ev : {&fork_ev, &join_ev, &done_ev}) OA_CUDA(cudaEventCreateWithFlags(ev, cudaEventDisableTiming));
    in_ev.assign(n, nullptr);
    for (cudaEvent_t& ev : in_ev) OA_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    tma = variant >= 2;
    const int rv = variant;
    // the engines' arguments of a step starting in buffer p (in place: p = 0 only)
    const int parities = variant == 3 ? 2 : 1;
    std::vector<oafdtd::SweepMaps> mp(n);
    std::vector<oafdtd::FusedMaps> fm(n);
    std::vector<oafdtd::ProbeArgs<real>> pr(n);
    std::vector<oafdtd::SibcArgs<real>> sb(n);
    std::vector<oafdtd::EdgeArgs<real>> ed(n);
    for (int p = 0; p < parities; ++p) {
      h_sw[p].resize(n);
      for (int i = 0; i < n; ++i) {
        Engine<real>& e = *eng[i];
        e.sw.tile_z = e.tile_z;
        e.use_regions(rv);
        e.bind(p, p);
        h_sw[p][i] = e.sw;
        mp[i] = e.maps_p[p];
        fm[i] = e.fmaps[p];
        pr[i] = e.pr;
        sb[i] = e.sb;
        ed[i] = e.ed;
      }
      if (int rc = upload(&d_sw[p], h_sw[p].data(), n)) return rc;
      if (int rc = upload(&d_mp[p], mp.data(), n)) return rc;
      if (int rc = upload(&d_fm[p], fm.data(), n)) return rc;
      if (int rc = upload(&d_pr[p], pr.data(), n)) return rc;
      if (int rc = upload(&d_sb[p], sb.data(), n)) return rc;
      if (int rc = upload(&d_ed[p], ed.data(), n)) return rc;
    }
    for (Engine<real>* e : eng) e->bind(e->cur[0], e->cur[1]);
    // launch geometry, from the parity-0 arguments (the boxes do not depend on the buffers)
    const std::vector<oafdtd::SweepArgs<real>>& a = h_sw[0];
    std::vector<dim3> g_fused(n), g_hi(n), g_hz(n), g_ei(n), g_ez(n), g_sh(n), g_se(n), g_pre(n), g_probe(n),
        g_edge(n), g_sibc(n);
    std::vector<int> k_pole(n), k_zero(n, 0), k_sibc(n);
    std::vector<oafdtd::SlabLaunch> slabs[2];
    slabs[0].resize(n);
    slabs[1].resize(n);
    for (int i = 0; i < n; ++i) {
      cudaError_t err = cudaSuccess;
      if (variant == 3 && (err = oafdtd::fused_grid(a[i], &g_fused[i])) != cudaSuccess)
        return fail(OAFDTD_E_INVALID, "fused sweep geometry of a batched engine");
      if (variant != 0) {
        if ((err = oafdtd::staged_grids(a[i], 1, &g_hi[i], &g_hz[i])) != cudaSuccess ||
            (err = oafdtd::staged_grids(a[i], 0, &g_ei[i], &g_ez[i])) != cudaSuccess)
          return fail(OAFDTD_E_INVALID, "staged sweep geometry of a batched engine");
      } else {
        g_hi[i] = g_hz[i] = g_ei[i] = g_ez[i] = dim3(0, 0, 0);
      }
      if (variant != 3) g_fused[i] = dim3(0, 0, 0);
      for (int kind = 0; kind < 2; ++kind) {
        long long blocks = 0;
        if (oafdtd::slab_plan(a[i], kind, &slabs[kind][i], &blocks) != cudaSuccess)
          return fail(OAFDTD_E_INVALID, "slab geometry of a batched engine");
        (kind == 0 ? g_se : g_sh)[i] = dim3((unsigned)blocks, 1, 1);
      }
      const Engine<real>& e = *eng[i];
      g_pre[i] = dim3((unsigned)oafdtd::pre_e_blocks(e.pr), 1, 1);
      g_probe[i] = dim3((unsigned)oafdtd::probe_e_blocks(e.pr), 1, 1);
      g_edge[i] = dim3((unsigned)oafdtd::edge_blocks(e.ed), 1, 1);
      g_sibc[i] = dim3((unsigned)oafdtd::sibc_blocks(e.sb), 1, 1);
      k_pole[i] = a[i].ade_P > 1 ? 1 : 0;
      k_sibc[i] = oafdtd::sibc_variant(e.sb);
    }
    for (int kind = 0; kind < 2; ++kind)
      if (int rc = upload(&d_slab[kind], slabs[kind].data(), n)) return rc;
    std::vector<long long*> bases(n);
    for (int i = 0; i < n; ++i) bases[i] = eng[i]->step_base;
    if (int rc = upload(&d_step_base, bases.data(), n)) return rc;
    const std::pair<std::vector<dim3>*, std::pair<std::vector<int>*, std::vector<Launch>*>> plans[] = {
        {&g_fused, {&k_pole, &fused}},  {&g_hi, {&k_zero, &h_inner}}, {&g_hz, {&k_zero, &h_z}},
        {&g_ei, {&k_pole, &e_inner}},   {&g_ez, {&k_pole, &e_z}},     {&g_sh, {&k_zero, &slab_h}},
        {&g_se, {&k_pole, &slab_e}},    {&g_pre, {&k_zero, &pre_e}},  {&g_probe, {&k_zero, &probe_e}},
        {&g_edge, {&k_zero, &edges}},   {&g_sibc, {&k_sibc, &sibc}},
    };
    for (const auto& q : plans)
      if (int rc = plan(*q.first, *q.second.first, q.second.second)) return rc;
    return OAFDTD_OK;
  }

  int sweep_launches(const std::vector<Launch>& ls, bool h, bool z, int p, cudaStream_t s) {
    for (const Launch& L : ls) {
      const cudaError_t err =
          oafdtd::launch_staged_batch<real>(d_sw[p], d_mp[p], L.g, L.blocks, h, tma, z, L.key != 0, s);
      if (err != cudaSuccess) return fail(OAFDTD_E_CUDA, std::string("batched sweep: ") + cudaGetErrorString(err));
    }
    return OAFDTD_OK;
  }
  int slab_launches(int kind, int p, cudaStream_t s) {
    for (const Launch& L : kind == 0 ? slab_e : slab_h) {
      const cudaError_t err =
          oafdtd::launch_slab_batch<real>(d_sw[p], d_slab[kind], L.g, L.blocks, kind, L.key != 0, s);
      if (err != cudaSuccess) return fail(OAFDTD_E_CUDA, std::string("batched slab: ") + cudaGetErrorString(err));
    }
    return OAFDTD_OK;
  }
  // the staged sweep of one kind with its slab kernel beside it (Engine::sweep_pair)
  int pair(int kind, int p) {
    const bool h = kind == 1;
    if (variant != 0) {
      OA_CUDA(cudaEventRecord(fork_ev, stream));
      OA_CUDA(cudaStreamWaitEvent(side, fork_ev, 0));
      if (int rc = slab_launches(kind, p, side)) return rc;
      OA_CUDA(cudaEventRecord(join_ev, side));
      if (int rc = sweep_launches(h ? h_inner : e_inner, h, false, p, stream)) return rc;
      if (int rc = sweep_launches(h ? h_z : e_z, h, true, p, stream)) return rc;
      OA_CUDA(cudaStreamWaitEvent(stream, join_ev, 0));
      return OAFDTD_OK;
    }
    return slab_launches(kind, p, stream);
  }

  // One time step of every engine, from buffers p (Engine::launch_step with parts 3).
  int launch_step(int off, int p) {
    cudaError_t err = cudaSuccess;
    if (variant == 3) {  // the fused sweeps first, the H work outside their boxes beside them
      OA_CUDA(cudaEventRecord(fork_ev, stream));
      for (const Launch& L : fused)
        if ((err = oafdtd::launch_fused_batch<real>(d_sw[p], d_fm[p], L.g, L.blocks, L.key != 0, stream)) != cudaSuccess)
          return fail(OAFDTD_E_CUDA, std::string("batched fused sweep: ") + cudaGetErrorString(err));
      OA_CUDA(cudaStreamWaitEvent(side, fork_ev, 0));
      if (int rc = sweep_launches(h_inner, true, false, p, side)) return rc;
      if (int rc = sweep_launches(h_z, true, true, p, side)) return rc;
      if (int rc = slab_launches(1, p, side)) return rc;
      OA_CUDA(cudaEventRecord(join_ev, side));
      OA_CUDA(cudaStreamWaitEvent(stream, join_ev, 0));
    } else if (int rc = pair(1, p)) {
      return rc;
    }
    for (size_t i = 0; i < eng.size(); ++i) {
      const Engine<real>& e = *eng[i];
      if (!e.pmc_mask) continue;
      if ((err = oafdtd::launch_ghosts<real>(h_sw[p][i].Ho, e.pmc_mask, e.nx, e.ny, e.nz, e.X, e.Y, e.B, stream)) !=
          cudaSuccess)
        return fail(OAFDTD_E_CUDA, std::string("ghosts: ") + cudaGetErrorString(err));
    }
    for (const Launch& L : pre_e)
      if ((err = oafdtd::launch_pre_e_batch<real>(d_pr[p], L.g, L.blocks, off, stream)) != cudaSuccess)
        return fail(OAFDTD_E_CUDA, std::string("batched pre_e: ") + cudaGetErrorString(err));
    if (int rc = pair(0, p)) return rc;
    for (const Launch& L : sibc)
      if ((err = oafdtd::launch_sibc_batch<real>(d_sb[p], L.g, L.blocks, L.key, stream)) != cudaSuccess)
        return fail(OAFDTD_E_CUDA, std::string("batched sibc: ") + cudaGetErrorString(err));
    for (const Launch& L : edges)
      if ((err = oafdtd::launch_edges_batch<real>(d_ed[p], L.g, L.blocks, off, stream)) != cudaSuccess)
        return fail(OAFDTD_E_CUDA, std::string("batched edges: ") + cudaGetErrorString(err));
    for (const Launch& L : probe_e)
      if ((err = oafdtd::launch_probe_e_batch<real>(d_pr[p], L.g, L.blocks, off, stream)) != cudaSuccess)
        return fail(OAFDTD_E_CUDA, std::string("batched probe_e: ") + cudaGetErrorString(err));
    return OAFDTD_OK;
  }

  int capture(int p) {
    cudaGraph_t g = nullptr;
    OA_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    int rc = OAFDTD_OK;
    int q = p;
    for (int o = 0; o < oafdtd::kChunk && rc == OAFDTD_OK; ++o) {
      rc = launch_step(o, q);
      if (variant == 3) q ^= 1;
    }
    if (rc == OAFDTD_OK) {
      const cudaError_t err = oafdtd::launch_bump_batch(d_step_base, (int)eng.size(), oafdtd::kChunk, stream);
      if (err != cudaSuccess) rc = fail(OAFDTD_E_CUDA, cudaGetErrorString(err));
    }
    const cudaError_t err = cudaStreamEndCapture(stream, &g);
    if (rc != OAFDTD_OK) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (err != cudaSuccess) return fail(OAFDTD_E_CUDA, std::string("batch capture: ") + cudaGetErrorString(err));
    size_t nodes = 0;
    int64_t kernels = 0;
    if (cudaGraphGetNodes(g, nullptr, &nodes) == cudaSuccess && nodes) {
      std::vector<cudaGraphNode_t> v(nodes);
      if (cudaGraphGetNodes(g, v.data(), &nodes) == cudaSuccess)
        for (cudaGraphNode_t nd : v) {
          cudaGraphNodeType t;
          if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++kernels;
        }
    }
    const cudaError_t ierr = cudaGraphInstantiate(&graph[p], g, 0);
    cudaGraphDestroy(g);
    if (ierr != cudaSuccess) return fail(OAFDTD_E_CUDA, std::string("batch instantiate: ") + cudaGetErrorString(ierr));
    graph_kernels = kernels;
    return OAFDTD_OK;
  }

  int enqueue(int64_t n) override {
    if (n < 0) return fail(OAFDTD_E_INVALID, "negative step count");
    Engine<real>& e0 = *eng[0];
    for (Engine<real>* e : eng) {
      if (e->steps != e0.steps || e->cur[0] != e0.cur[0] || e->half_pending)
        return fail(OAFDTD_E_INVALID, "an engine of the batch was stepped on its own");
      if (e->steps + n > e->max_steps) return fail(OAFDTD_E_RANGE, "step count exceeds max_steps (wave table length)");
    }
    OA_CUDA(cudaSetDevice(device));
    for (size_t i = 0; i < eng.size(); ++i) {
      OA_CUDA(cudaEventRecord(in_ev[i], eng[i]->stream));
      OA_CUDA(cudaStreamWaitEvent(stream, in_ev[i], 0));
    }
    int64_t done = 0;
    while (done < n) {
      const int64_t start = e0.steps;
      const int take = (int)std::min<int64_t>(n - done, oafdtd::kChunk - start % oafdtd::kChunk);
      const int p = variant == 3 ? e0.cur[0] : 0;
      if (e0.use_graph && take == oafdtd::kChunk) {
        if (!graph[p])
          if (int rc = capture(p)) return rc;
        OA_CUDA(cudaGraphLaunch(graph[p], stream));
      } else {
        int q = p;
        for (int o = 0; o < take; ++o) {
          if (int rc = launch_step(o, q)) return rc;
          if (variant == 3) q ^= 1;
        }
        const cudaError_t err = oafdtd::launch_bump_batch(d_step_base, (int)eng.size(), take, stream);
        if (err != cudaSuccess) return fail(OAFDTD_E_CUDA, cudaGetErrorString(err));
      }
      for (Engine<real>* e : eng) {
        e->steps += take;
        if (variant == 3 && (take & 1)) {
          e->cur[0] ^= 1;
          e->cur[1] ^= 1;
        }
      }
      done += take;
    }
    // later work on an engine's own stream follows the batch
    OA_CUDA(cudaEventRecord(done_ev, stream));
    for (Engine<real>* e : eng) OA_CUDA(cudaStreamWaitEvent(e->stream, done_ev, 0));
    return OAFDTD_OK;
  }

  int wait() override {
    OA_CUDA(cudaSetDevice(device));
    OA_CUDA(cudaStreamSynchronize(stream));
    OA_CUDA(cudaGetLastError());
    for (Engine<real>* e : eng)
      if (int rc = e->check_status()) return rc;
    return OAFDTD_OK;
  }
};

}  // namespace

namespace oafdtd {
void set_last_error(const std::string& msg) { g_last_error = msg; }
}  // namespace oafdtd

struct oafdtd_engine {
  std::unique_ptr<EngineBase> impl;
};

struct oafdtd_batch {
  std::unique_ptr<BatchBase> impl;
};

extern "C" {

int32_t oafdtd_abi_version(void) { return OAFDTD_ABI_VERSION; }

const char* oafdtd_last_error(void) { return g_last_error.c_str(); }

int32_t oafdtd_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

int oafdtd_set_device(int32_t device) {
  const int n = oafdtd_device_count();
  if (device < 0 || device >= n) return fail(OAFDTD_E_NODEVICE, "device index out of range");
  OA_CUDA(cudaSetDevice(device));
  return OAFDTD_OK;
}

int oafdtd_device_info(char* name, int32_t name_len, int32_t* cc_major, int32_t* cc_minor,
                       int64_t* free_bytes, int64_t* total_bytes, int32_t* runtime_version) {
  if (oafdtd_device_count() == 0) return fail(OAFDTD_E_NODEVICE, "no CUDA device is visible");
  int dev = 0;
  OA_CUDA(cudaGetDevice(&dev));
  cudaDeviceProp prop;
  OA_CUDA(cudaGetDeviceProperties(&prop, dev));
  if (name && name_len > 0) {
    std::strncpy(name, prop.name, (size_t)name_len - 1);
    name[name_len - 1] = 0;
  }
  if (cc_major) *cc_major = prop.major;
  if (cc_minor) *cc_minor = prop.minor;
  size_t fr = 0, tot = 0;
  OA_CUDA(cudaMemGetInfo(&fr, &tot));
  if (free_bytes) *free_bytes = (int64_t)fr;
  if (total_bytes) *total_bytes = (int64_t)tot;
  int rv = 0;
  OA_CUDA(cudaRuntimeGetVersion(&rv));
  if (runtime_version) *runtime_version = rv;
  return OAFDTD_OK;
}

int oafdtd_create(const oafdtd_problem* problem, oafdtd_engine** out) {
  if (out == nullptr || problem == nullptr) return fail(OAFDTD_E_INVALID, "null argument");
  *out = nullptr;
  if (problem->abi_version != OAFDTD_ABI_VERSION) return fail(OAFDTD_E_INVALID, "ABI version mismatch");
  if (oafdtd_device_count() == 0) return fail(OAFDTD_E_NODEVICE, "no CUDA device is visible");
  std::unique_ptr<oafdtd_engine> h(new (std::nothrow) oafdtd_engine);
  if (!h) return fail(OAFDTD_E_OOM, "host allocation failed");
  int rc;
  try {
    if (problem->real_bytes == 4) {
      auto* e = new Engine<float>();
      h->impl.reset(e);
      rc = e->build(*problem);
    } else if (problem->real_bytes == 8) {
      auto* e = new Engine<double>();
      h->impl.reset(e);
      rc = e->build(*problem);
    } else {
      return fail(OAFDTD_E_INVALID, "real_bytes must be 4 or 8");
    }
  } catch (const std::bad_alloc&) {
    return fail(OAFDTD_E_OOM, "host allocation failed while preparing the problem");
  }
  if (rc != OAFDTD_OK) return rc;
  *out = h.release();
  return OAFDTD_OK;
}

int oafdtd_destroy(oafdtd_engine* engine) {
  delete engine;
  return OAFDTD_OK;
}

int oafdtd_step(oafdtd_engine* engine, int64_t n) {
  if (!engine) return fail(OAFDTD_E_INVALID, "null engine");
  return engine->impl->step(n);
}

int oafdtd_step_timed(oafdtd_engine* engine, int64_t n, double* device_ms) {
  if (!engine || !device_ms) return fail(OAFDTD_E_INVALID, "null argument");
  return engine->impl->step_timed(n, device_ms);
}

int oafdtd_step_count(const oafdtd_engine* engine, int64_t* out) {
  if (!engine || !out) return fail(OAFDTD_E_INVALID, "null argument");
  *out = engine->impl->steps;
  return OAFDTD_OK;
}

int oafdtd_energy(oafdtd_engine* engine, double* out) {
  if (!engine || !out) return fail(OAFDTD_E_INVALID, "null argument");
  return engine->impl->energy(out);
}

int oafdtd_dft(oafdtd_engine* engine, double* out) {
  if (!engine || !out) return fail(OAFDTD_E_INVALID, "null argument");
  return engine->impl->dft(out);
}

int oafdtd_series(oafdtd_engine* engine, double* out) {
  if (!engine || !out) return fail(OAFDTD_E_INVALID, "null argument");
  return engine->impl->series(out);
}

int oafdtd_fields(oafdtd_engine* engine, int32_t comp, double* out) {
  if (!engine || !out) return fail(OAFDTD_E_INVALID, "null argument");
  return engine->impl->fields(comp, out);
}

int oafdtd_snapshot_bytes(oafdtd_engine* engine, int64_t* out) {
  if (!engine || !out) return fail(OAFDTD_E_INVALID, "null argument");
  return engine->impl->snapshot(nullptr, out, nullptr);
}

int oafdtd_snapshot(oafdtd_engine* engine, void* out) {
  if (!engine || !out) return fail(OAFDTD_E_INVALID, "null argument");
  return engine->impl->snapshot(out, nullptr, nullptr);
}

int oafdtd_restore(oafdtd_engine* engine, const void* in) {
  if (!engine || !in) return fail(OAFDTD_E_INVALID, "null argument");
  return engine->impl->snapshot(nullptr, nullptr, in);
}

int oafdtd_step_async(oafdtd_engine* engine, int64_t n) {
  if (!engine) return fail(OAFDTD_E_INVALID, "null engine");
  return engine->impl->enqueue(n);
}

int oafdtd_wait(oafdtd_engine* engine) {
  if (!engine) return fail(OAFDTD_E_INVALID, "null engine");
  return engine->impl->wait();
}

int oafdtd_step_half(oafdtd_engine* engine, int32_t which) {
  if (!engine) return fail(OAFDTD_E_INVALID, "null engine");
  return engine->impl->step_half(which);
}

int oafdtd_plane(oafdtd_engine* engine, int32_t comp, int32_t k, double* out) {
  if (!engine || !out) return fail(OAFDTD_E_INVALID, "null argument");
  return engine->impl->plane(comp, k, out, nullptr);
}

int oafdtd_set_plane(oafdtd_engine* engine, int32_t comp, int32_t k, const double* in) {
  if (!engine || !in) return fail(OAFDTD_E_INVALID, "null argument");
  return engine->impl->plane(comp, k, nullptr, in);
}

int oafdtd_plane_device(oafdtd_engine* engine, int32_t comp, int32_t k, void* dst) {
  if (!engine || !dst) return fail(OAFDTD_E_INVALID, "null argument");
  return engine->impl->plane_device(comp, k, dst, nullptr);
}

int oafdtd_set_plane_device(oafdtd_engine* engine, int32_t comp, int32_t k, const void* src) {
  if (!engine || !src) return fail(OAFDTD_E_INVALID, "null argument");
  return engine->impl->plane_device(comp, k, nullptr, src);
}

int oafdtd_set_field(oafdtd_engine* engine, int32_t comp, const double* in) {
  if (!engine || !in) return fail(OAFDTD_E_INVALID, "null argument");
  return engine->impl->set_field(comp, in);
}

int oafdtd_peak_bytes(const oafdtd_engine* engine, int64_t* out) {
  if (!engine || !out) return fail(OAFDTD_E_INVALID, "null argument");
  *out = engine->impl->bytes;
  return OAFDTD_OK;
}

int oafdtd_set_graph(oafdtd_engine* engine, int32_t use_graph) {
  if (!engine) return fail(OAFDTD_E_INVALID, "null engine");
  engine->impl->use_graph = use_graph ? 1 : 0;
  return OAFDTD_OK;
}

int oafdtd_set_tuning(oafdtd_engine* engine, int32_t tile_z, int32_t variant) {
  if (!engine) return fail(OAFDTD_E_INVALID, "null engine");
  if (tile_z < 0 || tile_z > 4096) return fail(OAFDTD_E_INVALID, "tile_z must be 0..4096 planes");
  if (variant < -1 || variant > 3) return fail(OAFDTD_E_INVALID, "variant must be -1, 0, 1, 2 or 3");
  if (variant >= 0 && variant != engine->impl->staged)
    if (int rc = engine->impl->set_variant(variant)) return rc;
  if (tile_z) engine->impl->tile_z = tile_z;
  engine->impl->graph_dirty = true;  // a new launch shape needs a new graph
  return OAFDTD_OK;
}

int oafdtd_get_tuning(const oafdtd_engine* engine, int32_t* tile_z, int32_t* variant) {
  if (!engine || !tile_z || !variant) return fail(OAFDTD_E_INVALID, "null argument");
  *tile_z = engine->impl->tile_z;
  *variant = engine->impl->staged;
  return OAFDTD_OK;
}

int oafdtd_batch_create(oafdtd_engine* const* engines, int32_t n, oafdtd_batch** out) {
  if (!engines || !out || n < 1) return fail(OAFDTD_E_INVALID, "null argument or empty batch");
  *out = nullptr;
  std::vector<Engine<float>*> f32;
  std::vector<Engine<double>*> f64;
  for (int i = 0; i < n; ++i) {
    if (!engines[i]) return fail(OAFDTD_E_INVALID, "null engine in the batch");
    EngineBase* e = engines[i]->impl.get();
    if (auto* ef = dynamic_cast<Engine<float>*>(e)) f32.push_back(ef);
    else if (auto* ed = dynamic_cast<Engine<double>*>(e)) f64.push_back(ed);
  }
  if (!f32.empty() && !f64.empty()) return fail(OAFDTD_E_INVALID, "the engines of a batch share one precision");
  std::unique_ptr<oafdtd_batch> b(new (std::nothrow) oafdtd_batch);
  if (!b) return fail(OAFDTD_E_OOM, "host allocation");
  if (!f32.empty()) {
    auto* impl = new Batch<float>();
    b->impl.reset(impl);
    if (int rc = impl->build(f32)) return rc;
  } else {
    auto* impl = new Batch<double>();
    b->impl.reset(impl);
    if (int rc = impl->build(f64)) return rc;
  }
  *out = b.release();
  return OAFDTD_OK;
}

int oafdtd_batch_step_async(oafdtd_batch* batch, int64_t n) {
  if (!batch) return fail(OAFDTD_E_INVALID, "null batch");
  return batch->impl->enqueue(n);
}

int oafdtd_batch_wait(oafdtd_batch* batch) {
  if (!batch) return fail(OAFDTD_E_INVALID, "null batch");
  return batch->impl->wait();
}

int oafdtd_batch_graph_kernels(const oafdtd_batch* batch, int64_t* out) {
  if (!batch || !out) return fail(OAFDTD_E_INVALID, "null argument");
  *out = batch->impl->graph_kernels;
  return OAFDTD_OK;
}

int oafdtd_batch_destroy(oafdtd_batch* batch) {
  delete batch;
  return OAFDTD_OK;
}

int oafdtd_graph_kernels(oafdtd_engine* engine, int64_t* out) {
  if (!engine || !out) return fail(OAFDTD_E_INVALID, "null argument");
  *out = engine->impl->graph_kernels;
  return OAFDTD_OK;
}

int oafdtd_kernel_bytes(oafdtd_engine* engine, double* out, int32_t n) {
  if (!engine || !out || n < 0) return fail(OAFDTD_E_INVALID, "null argument");
  EngineBase& e = *engine->impl;
  e.traffic_ready();
  const double* cls = e.class_bytes[e.staged == 3 ? 2 : (e.staged ? 1 : 0)];
  double total = 0.0;
  for (int k = 0; k < EngineBase::kClasses; ++k) {
    if (k < n) out[k] = cls[k];
    total += cls[k];
  }
  if (n > EngineBase::kClasses) out[EngineBase::kClasses] = total;
  return OAFDTD_OK;
}

int oafdtd_set_profiling(oafdtd_engine* engine, int32_t on) {
  if (!engine) return fail(OAFDTD_E_INVALID, "null engine");
  engine->impl->profiling = on ? 1 : 0;
  engine->impl->graph_dirty = true;  // event records live inside the captured graph
  return OAFDTD_OK;
}

int oafdtd_kernel_times(oafdtd_engine* engine, double* out_ms, int32_t n) {
  if (!engine || !out_ms) return fail(OAFDTD_E_INVALID, "null argument");
  return engine->impl->kernel_times(out_ms, n);
}

int oafdtd_model_bytes(const oafdtd_engine* engine, double* out) {
  if (!engine || !out) return fail(OAFDTD_E_INVALID, "null argument");
  engine->impl->traffic_ready();
  *out = engine->impl->model_bytes;
  return OAFDTD_OK;
}

}  // extern "C"
