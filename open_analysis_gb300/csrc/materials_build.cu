// Native model compiler: the volume stages of compile_model on the host, multi-threaded.
//
// Replaces the NumPy stages of the reference's compile_model (packages/oa-fdtd/src/oa_fdtd/
// model.py:501-768) that touch every cell and every edge:
//   * per-cell materials (_cell_materials, model.py:272-296): here one uint16 region id per cell
//     (0 = vacuum, r + 1 = region r, later regions win), not (2 + poles) float64 volumes;
//   * the area-weighted mean of the four cells around each E edge (_edge_average,
//     model.py:300-321), in the same summation order, plus the static Debye term folded into eps
//     (model.py:534-537) and the lumped-port loading added to sigma (model.py:610-647);
//   * the averaged-material table (model.py:688-722): keys (eps, sigma) rounded to 12 decimals
//     (NumPy's round: multiply by 1e12, round half to even, divide), their sorted unique set,
//     uint16 index 0 = PEC, i + 1 = table entry i;
//   * the Debye edge lists (_compile_ade, model.py:331-367): the dispersive non-PEC edges in C
//     order with their averaged pole strengths.
// Every floating-point operation is the one NumPy performs, in the same order, with contraction
// of multiply-add into FMA disabled for host code (-ffp-contract=off), so the arrays equal the
// NumPy compiler's bit for bit. Work is split by z planes over std::thread workers.

#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <thread>
#include <unordered_map>
#include <utility>
#include <vector>

#include "../../include/oafdtd.h"
#include "oafdtd_internal.cuh"

namespace {

struct Key {
  double eps, sig;
  bool operator<(const Key& o) const { return eps < o.eps || (eps == o.eps && sig < o.sig); }
  bool operator==(const Key& o) const { return eps == o.eps && sig == o.sig; }
};

double round12(double x) {
  // NumPy's np.round(x, 12) for float64: (x * 1e12) rounded half to even, divided by 1e12
  return std::nearbyint(x * 1e12) / 1e12;
}

struct Desc {
  int n[3];
  std::vector<double> w[3];        // storage cell weights, length n + 2
  std::vector<uint16_t> region;    // (nz + 2, ny + 2, nx + 2) region ids
  int n_regions = 0, n_poles = 0;
  std::vector<double> reg_eps, reg_sig, reg_del;  // per id (0 = vacuum), reg_del (id, pole)
  std::vector<double> static_fac;
  double dt = 0.0, eps0 = 0.0;
  std::vector<double> taus;
  const uint8_t* pec[3] = {nullptr, nullptr, nullptr};
  std::vector<std::vector<std::pair<int64_t, double>>> loads;  // per component, in order
};

// Averaged (eps, sigma, strengths) of one edge; returns eps with the static Debye term and sigma
// with the port loads applied by the caller.
struct EdgeVals {
  double eps, sig;
  double del[8];
};

constexpr int kMaxPoles = 8;

}  // namespace

struct oafdtd_materials {
  Desc d;
  std::vector<Key> table;
  int pitch = 0;
  std::vector<uint16_t> idx[3];    // storage arrays (nz + 2, ny + 2, pitch)
  // Debye lists per worker and component, in worker (plane) order: [w * 3 + c]; fetch writes them
  // straight into the caller's buffers
  std::vector<std::vector<int64_t>> ade_flat;
  std::vector<std::vector<double>> ade_del;  // (edge, pole) per worker
  int64_t ade_n[3] = {0, 0, 0};
  int threads = 1;
};

namespace {

// Lattice (nz + 1, ny + 1, nx + 1) of component c, transverse axes p < q.
void axes(int c, int& p, int& q) {
  p = c == 0 ? 1 : 0;
  q = c == 2 ? 1 : 2;
}

inline void edge_values(const Desc& d, int c, int lx, int ly, int lz, EdgeVals& v) {
  int p, q;
  axes(c, p, q);
  const int l[3] = {lx, ly, lz};
  const int sx = d.n[0] + 2, sy = d.n[1] + 2;
  // NumPy's accumulators start at 0.0 and add the four products in this order
  double acc_e = 0.0, acc_s = 0.0, wsum = 0.0;
  double acc_d[kMaxPoles];
  for (int pi = 0; pi < d.n_poles; ++pi) acc_d[pi] = 0.0;
  for (int dp = 0; dp < 2; ++dp)
    for (int dq = 0; dq < 2; ++dq) {
      int cell[3];
      cell[c] = l[c] + 1;
      cell[p] = l[p] + 1 - dp;
      cell[q] = l[q] + 1 - dq;
      const double weight = d.w[p][l[p] + 1 - dp] * d.w[q][l[q] + 1 - dq];
      const int id = d.region[((int64_t)cell[2] * sy + cell[1]) * sx + cell[0]];
      acc_e += weight * d.reg_eps[id];
      acc_s += weight * d.reg_sig[id];
      wsum += weight;
      for (int pi = 0; pi < d.n_poles; ++pi) acc_d[pi] += weight * d.reg_del[id * d.n_poles + pi];
    }
  v.eps = acc_e / wsum;
  v.sig = acc_s / wsum;
  for (int pi = 0; pi < d.n_poles; ++pi) v.del[pi] = acc_d[pi] / wsum;
  for (int pi = 0; pi < d.n_poles; ++pi) v.eps += v.del[pi] * d.static_fac[pi];
}

template <typename F>
void parallel_planes(int nplanes, int threads, F&& fn) {
  const int t = std::max(1, std::min(threads, nplanes));
  std::vector<std::thread> pool;
  for (int w = 0; w < t; ++w)
    pool.emplace_back([&, w] {
      const int a = (int)((int64_t)nplanes * w / t), b = (int)((int64_t)nplanes * (w + 1) / t);
      fn(w, a, b);
    });
  for (auto& th : pool) th.join();
}

// The port loads of one lattice edge, applied in order (sigma += load).
inline double loaded_sig(const Desc& d, int c, int64_t lat, double sig) {
  const auto& ld = d.loads[c];
  if (ld.empty()) return sig;
  auto it = std::lower_bound(ld.begin(), ld.end(), std::make_pair(lat, -INFINITY),
                             [](const std::pair<int64_t, double>& a, const std::pair<int64_t, double>& b) {
                               return a.first < b.first;
                             });
  for (; it != ld.end() && it->first == lat; ++it) sig += it->second;
  return sig;
}

struct KeyHash {
  size_t operator()(const Key& k) const {
    uint64_t a, b;
    std::memcpy(&a, &k.eps, 8);
    std::memcpy(&b, &k.sig, 8);
    return (size_t)(a * 0x9E3779B97F4A7C15ull ^ (b + 0x632BE59BD9B4E019ull + (a << 6) + (a >> 2)));
  }
};

// One pass over every edge: each worker numbers the keys it meets (its own small dictionary) and
// writes those local numbers into the index arrays, and collects its Debye edges; then the local
// dictionaries merge into the sorted global table and each worker renumbers its own planes.
int build(oafdtd_materials& m, int threads) {
  Desc& d = m.d;
  const int nx = d.n[0], ny = d.n[1], nz = d.n[2];
  const int lx = nx + 1, ly = ny + 1, lz = nz + 1;
  m.pitch = (nx + 2 + 31) / 32 * 32;
  const int64_t plane = (int64_t)(ny + 2) * m.pitch;
  for (int c = 0; c < 3; ++c) m.idx[c].assign((size_t)(nz + 2) * plane, 0);
  std::vector<std::vector<Key>> local(threads);
  std::vector<std::vector<int64_t>> flat((size_t)threads * 3);
  std::vector<std::vector<double>> dels((size_t)threads * 3);
  std::vector<int> overflow(threads, 0);
  parallel_planes(lz, threads, [&](int w, int k0, int k1) {
    std::unordered_map<Key, uint16_t, KeyHash> ids;
    std::vector<Key>& keys = local[w];
    EdgeVals v;
    for (int c = 0; c < 3; ++c) {
      Key last{NAN, NAN};
      uint16_t last_id = 0;
      for (int k = k0; k < k1; ++k)
        for (int j = 0; j < ly; ++j)
          for (int i = 0; i < lx; ++i) {
            const int64_t lat = ((int64_t)k * ly + j) * lx + i;
            if (d.pec[c][lat]) continue;
            edge_values(d, c, i, j, k, v);
            const Key key{round12(v.eps), round12(loaded_sig(d, c, lat, v.sig))};
            if (!(key == last)) {
              last = key;
              auto it = ids.find(key);
              if (it == ids.end()) {
                if (keys.size() >= 65534) {
                  overflow[w] = 1;
                  return;
                }
                keys.push_back(key);
                it = ids.emplace(key, (uint16_t)keys.size()).first;
              }
              last_id = it->second;
            }
            const int64_t st = (int64_t)(k + 1) * plane + (int64_t)(j + 1) * m.pitch + (i + 1);
            m.idx[c][st] = last_id;
            if (d.n_poles > 0) {
              double strength = 0.0;
              for (int pi = 0; pi < d.n_poles; ++pi) strength += v.del[pi];
              if (strength > 1e-12) {
                flat[(size_t)w * 3 + c].push_back(st);
                for (int pi = 0; pi < d.n_poles; ++pi) dels[(size_t)w * 3 + c].push_back(v.del[pi]);
              }
            }
          }
    }
  });
  for (int w = 0; w < threads; ++w) {
    if (overflow[w]) {
      oafdtd::set_last_error("oafdtd_materials_build: more than 65534 averaged materials exceed the uint16 table");
      return OAFDTD_E_TABLE;
    }
    m.table.insert(m.table.end(), local[w].begin(), local[w].end());
  }
  std::sort(m.table.begin(), m.table.end());
  m.table.erase(std::unique(m.table.begin(), m.table.end()), m.table.end());
  if (m.table.size() + 1 > 65535) {
    oafdtd::set_last_error("oafdtd_materials_build: " + std::to_string(m.table.size()) +
                           " averaged materials exceed the uint16 table");
    return OAFDTD_E_TABLE;
  }
  // renumber: local number -> 1 + position in the sorted table, over each worker's own planes
  parallel_planes(lz, threads, [&](int w, int k0, int k1) {
    std::vector<uint16_t> lut(local[w].size() + 1, 0);
    for (size_t t = 0; t < local[w].size(); ++t)
      lut[t + 1] = (uint16_t)(std::lower_bound(m.table.begin(), m.table.end(), local[w][t]) - m.table.begin() + 1);
    for (int c = 0; c < 3; ++c)
      for (int k = k0; k < k1; ++k) {
        uint16_t* row = m.idx[c].data() + (int64_t)(k + 1) * plane;
        for (int64_t e = 0; e < plane; ++e) row[e] = lut[row[e]];
      }
  });
  // Debye lists stay with their workers (worker order = plane order = C order)
  m.threads = threads;
  m.ade_flat = std::move(flat);
  m.ade_del = std::move(dels);
  for (int c = 0; c < 3; ++c)
    for (int w = 0; w < threads; ++w) m.ade_n[c] += (int64_t)m.ade_flat[(size_t)w * 3 + c].size();
  return OAFDTD_OK;
}

}  // namespace

extern "C" {

int oafdtd_materials_build(const oafdtd_material_desc* in, oafdtd_materials** out) {
  if (!in || !out) return OAFDTD_E_INVALID;
  *out = nullptr;
  if (in->nx < 1 || in->ny < 1 || in->nz < 1 || in->n_regions < 0 || in->n_poles < 0 || in->n_poles > kMaxPoles ||
      in->n_regions > 65534 || in->n_loads < 0) {
    oafdtd::set_last_error("oafdtd_materials_build: bad sizes (at most 8 poles and 65534 regions)");
    return OAFDTD_E_INVALID;
  }
  for (int a = 0; a < 3; ++a)
    if (!in->cell_w[a] || !in->centres[a] || !in->pec[a]) {
      oafdtd::set_last_error("oafdtd_materials_build: missing weights, centres or PEC mask");
      return OAFDTD_E_INVALID;
    }
  auto* m = new oafdtd_materials();
  Desc& d = m->d;
  d.n[0] = in->nx, d.n[1] = in->ny, d.n[2] = in->nz;
  for (int a = 0; a < 3; ++a) {
    d.w[a].assign(in->cell_w[a], in->cell_w[a] + d.n[a] + 2);
    d.pec[a] = in->pec[a];
  }
  d.n_regions = in->n_regions;
  d.n_poles = in->n_poles;
  d.reg_eps.assign(1, 1.0);
  d.reg_sig.assign(1, 0.0);
  d.reg_del.assign((size_t)d.n_poles, 0.0);
  for (int r = 0; r < in->n_regions; ++r) {
    d.reg_eps.push_back(in->reg_eps[r]);
    d.reg_sig.push_back(in->reg_sig[r]);
    for (int pi = 0; pi < d.n_poles; ++pi) d.reg_del.push_back(in->reg_strength[(size_t)r * d.n_poles + pi]);
  }
  d.static_fac.assign(in->static_fac, in->static_fac + d.n_poles);
  d.dt = in->dt;
  d.eps0 = in->eps0;
  if (d.n_poles > 0 && !in->taus) {
    delete m;
    oafdtd::set_last_error("oafdtd_materials_build: Debye poles without relaxation times");
    return OAFDTD_E_INVALID;
  }
  if (d.n_poles > 0) d.taus.assign(in->taus, in->taus + d.n_poles);
  // region ids: cells whose centre lies in the closed box; later regions overwrite earlier ones
  const int sx = d.n[0] + 2, sy = d.n[1] + 2, sz = d.n[2] + 2;
  d.region.assign((size_t)sx * sy * sz, 0);
  for (int r = 0; r < in->n_regions; ++r) {
    int lo[3], hi[3];
    bool empty = false;
    for (int a = 0; a < 3; ++a) {
      lo[a] = d.n[a], hi[a] = -1;
      for (int i = 0; i < d.n[a]; ++i) {
        const double x = in->centres[a][i];
        if (x >= in->reg_lo[3 * r + a] && x <= in->reg_hi[3 * r + a]) lo[a] = std::min(lo[a], i), hi[a] = std::max(hi[a], i);
      }
      if (hi[a] < lo[a]) empty = true;
    }
    if (empty) continue;
    for (int k = lo[2]; k <= hi[2]; ++k)
      for (int j = lo[1]; j <= hi[1]; ++j)
        for (int i = lo[0]; i <= hi[0]; ++i) d.region[((size_t)(k + 1) * sy + (j + 1)) * sx + (i + 1)] = (uint16_t)(r + 1);
  }
  d.loads.assign(3, {});
  const int64_t lattice = (int64_t)(d.n[0] + 1) * (d.n[1] + 1) * (d.n[2] + 1);
  for (int64_t e = 0; e < in->n_loads; ++e) {
    const int c = in->load_comp[e];
    const int64_t lat = in->load_lattice[e];
    if (c < 0 || c > 2 || lat < 0 || lat >= lattice) {
      delete m;
      oafdtd::set_last_error("oafdtd_materials_build: port load outside the lattice");
      return OAFDTD_E_INVALID;
    }
    d.loads[c].emplace_back(lat, in->load_sig[e]);
  }
  // stable: loads of one edge keep their order
  for (auto& ld : d.loads)
    std::stable_sort(ld.begin(), ld.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
  int threads = in->threads > 0 ? in->threads : (int)std::thread::hardware_concurrency();
  threads = std::max(1, std::min(threads, 64));
  const int rc = build(*m, threads);
  if (rc != OAFDTD_OK) {
    delete m;
    return rc;
  }
  *out = m;
  return OAFDTD_OK;
}

int oafdtd_materials_sizes(const oafdtd_materials* m, int32_t* n_mat, int64_t* ade_n) {
  if (!m || !n_mat || !ade_n) return OAFDTD_E_INVALID;
  *n_mat = (int32_t)m->table.size() + 1;
  for (int c = 0; c < 3; ++c) ade_n[c] = m->ade_n[c] < 0 ? -m->ade_n[c] - 1 : m->ade_n[c];
  return OAFDTD_OK;
}

int oafdtd_materials_fetch(oafdtd_materials* m, uint16_t* idx0, uint16_t* idx1, uint16_t* idx2, double* eps_tab,
                           double* sig_tab, int64_t* flat0, int64_t* flat1, int64_t* flat2, double* beta0,
                           double* beta1, double* beta2, double* cbe0, double* cbe1, double* cbe2) {
  if (!m || !idx0 || !idx1 || !idx2 || !eps_tab || !sig_tab) return OAFDTD_E_INVALID;
  uint16_t* idx[3] = {idx0, idx1, idx2};
  int64_t* flat[3] = {flat0, flat1, flat2};
  double* beta[3] = {beta0, beta1, beta2};
  double* cbe[3] = {cbe0, cbe1, cbe2};
  for (int c = 0; c < 3; ++c) {
    if (m->ade_n[c] < 0) {
      oafdtd::set_last_error("oafdtd_materials_fetch: the lists were fetched already");
      return OAFDTD_E_INVALID;
    }
    if (m->ade_n[c] > 0 && (!flat[c] || !beta[c] || !cbe[c])) return OAFDTD_E_INVALID;
  }
  const Desc& d = m->d;
  const int P = d.n_poles, T = m->threads;
  // the tables, and cb of every entry in the operation order of the NumPy update_coefficients:
  // ep = eps * eps0; loss = sigma * dt / (2 ep); cb = dt / ep / (1 + loss); the PEC entry 0
  const size_t n_mat = m->table.size() + 1;
  std::vector<double> cb(n_mat, 0.0);
  eps_tab[0] = 0.0, sig_tab[0] = 0.0;
  for (size_t t = 0; t < m->table.size(); ++t) {
    const double eps = m->table[t].eps, sig = m->table[t].sig;
    eps_tab[t + 1] = eps, sig_tab[t + 1] = sig;
    if (eps > 0) {
      const double ep = eps * d.eps0;
      const double loss = sig * d.dt / (2.0 * ep);
      cb[t + 1] = d.dt / ep / (1.0 + loss);
    }
  }
  std::vector<double> denom(P);
  for (int pi = 0; pi < P; ++pi) denom[pi] = d.taus[pi] + 0.5 * d.dt;
  for (int c = 0; c < 3; ++c) std::memcpy(idx[c], m->idx[c].data(), m->idx[c].size() * sizeof(uint16_t));
  // one component at a time: each worker's segment goes to its own offset (the copies run side by
  // side), then that component's lists are released, so the lists and their copies never all
  // coexist
  for (int c = 0; c < 3; ++c) {
    if (m->ade_n[c] == 0) continue;
    std::vector<std::thread> pool;
    for (int w = 0; w < T; ++w)
      pool.emplace_back([&, w, c] {
        int64_t at = 0;
        for (int v = 0; v < w; ++v) at += (int64_t)m->ade_flat[(size_t)v * 3 + c].size();
        const auto& f = m->ade_flat[(size_t)w * 3 + c];
        const auto& dl = m->ade_del[(size_t)w * 3 + c];
        std::memcpy(flat[c] + at, f.data(), f.size() * sizeof(int64_t));
        const uint16_t* ic = idx[c];
        for (size_t e = 0; e < f.size(); ++e) {
          cbe[c][at + e] = cb[ic[f[e]]];
          for (int pi = 0; pi < P; ++pi)
            beta[c][(size_t)pi * m->ade_n[c] + at + e] = d.eps0 * dl[e * P + pi] / denom[pi];
        }
      });
    for (auto& th : pool) th.join();
    for (int w = 0; w < T; ++w) {
      std::vector<int64_t>().swap(m->ade_flat[(size_t)w * 3 + c]);
      std::vector<double>().swap(m->ade_del[(size_t)w * 3 + c]);
    }
    m->ade_n[c] = -m->ade_n[c] - 1;  // fetched: the lists are gone
  }
  return OAFDTD_OK;
}

int oafdtd_materials_free(oafdtd_materials* m) {
  delete m;
  return OAFDTD_OK;
}

}  // extern "C"
