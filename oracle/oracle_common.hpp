// Oracle (test infrastructure only): CPU FP64 restatement of the Graph-Cut
// RANSAC hot path of danini/graph-cut-ransac. Nothing in the product links or
// calls this code; tests, smoke() and the CPU-baseline leg of bench.py use it
// as the checker.
//
// This header: containers, the counter-based random generator, samplers and
// the grid neighbourhood graph.
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>
#include <unordered_map>
#include <queue>
#include <vector>

namespace oracle {

// Row-major view of an N x cols double matrix; stands in for cv::Mat.
struct Mat {
  const double* d = nullptr;
  int64_t rows = 0;
  int cols = 0;
  const double* row(int64_t i) const { return d + i * cols; }
};

using Model = std::array<double, 9>;  // 3x3 row-major

// src/pygcransac/include/scoring_function.h:47-72 — comparisons use value only.
struct Score {
  size_t inlier_number = 0;
  double value = 0.0;
};
inline bool operator<(const Score& a, const Score& b) { return a.value < b.value; }

// Settings, defaults from src/pygcransac/include/settings.h:65-86.
struct Settings {
  bool do_final_iterated_least_squares = true;
  bool do_local_optimization = true;
  size_t max_local_optimization_number = 10;
  size_t max_graph_cut_number = 10;
  size_t max_least_squares_iterations = 10;
  size_t min_iteration_number_before_lo = 20;
  size_t min_iteration_number = 20;
  size_t max_iteration_number = std::numeric_limits<size_t>::max();
  size_t max_unsuccessful_model_generations = 100;
  double spatial_coherence_weight = 0.14;
  double threshold = 2.0;
  double confidence = 0.95;
  // SPRT preemptive verification (the drivers' use_sprt and
  // min_inlier_ratio_for_sprt arguments)
  bool use_sprt = false;
  double sprt_min_inlier_ratio = 0.01;
  bool use_space_partitioning = false;
};

struct Statistics {
  size_t iteration_number = 0;
  size_t graph_cut_number = 0;
  size_t local_optimization_number = 0;
  size_t neighbor_number = 0;
  bool irls_applied = false;
  double score = 0.0;
  std::vector<size_t> inliers;
};

// ---------------------------------------------------------------------------
// Counter-based generator: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel
// random numbers: as easy as 1, 2, 3", SC'11). The reference seeds std::mt19937
// from std::random_device (src/pygcransac/include/uniform_random_generator.h:51-54),
// so its streams cannot be reproduced; the engine and this oracle share the
// following definition instead: the d-th 32-bit draw of call c of stream s under
// seed k is word (d & 3) of Philox(counter = {d >> 2, c_lo, c_hi, s}, key = {k_lo, k_hi}).
inline void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
    const uint32_t n1 = (uint32_t)p1;
    const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
    const uint32_t n3 = (uint32_t)p0;
    c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

inline uint32_t draw_u32(uint64_t seed, uint32_t stream, uint64_t call, uint32_t draw) {
  uint32_t c[4] = {draw >> 2, (uint32_t)call, (uint32_t)(call >> 32), stream};
  philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  return c[draw & 3];
}

// Stream ids shared with the device samplers.
enum : uint32_t {
  STREAM_MAIN = 1,
  STREAM_LO = 2,
  STREAM_SPRT = 3,
  STREAM_NAPSAC_LOCAL = 3,
  STREAM_NAPSAC_CENTER = 4,
  STREAM_NAPSAC_GLOBAL = 5,
  STREAM_AR = 6,
};

// Restates utils::UniformRandomGenerator (uniform_random_generator.h:44-124):
// inclusive integer range, unique sets by rejection. One generateUniqueRandomSet
// call consumes one call index of the stream.
struct Generator {
  uint64_t seed = 0;
  uint32_t stream = 0;
  uint64_t calls = 0;
  uint64_t lo = 0, hi = 0;
  Generator() = default;
  Generator(uint64_t s, uint32_t st) : seed(s), stream(st) {}
  void reset(uint64_t lo_, uint64_t hi_) { lo = lo_; hi = hi_; }
  uint64_t next(uint64_t call, uint32_t& d) const {
    const uint64_t range = hi - lo + 1;
    return lo + (((uint64_t)draw_u32(seed, stream, call, d++) * range) >> 32);
  }
  // generateUniqueRandomSet(sample, k) (:75-88)
  void unique_set(size_t* s, size_t k) {
    const uint64_t call = calls++;
    uint32_t d = 0;
    for (size_t i = 0; i < k; ++i) {
      s[i] = next(call, d);
      for (int j = (int)i - 1; j >= 0; --j)
        if (s[i] == s[j]) { --i; break; }
      if (d > (1u << 24)) return;  // guard: only reachable for an empty range
    }
  }
  // generateUniqueRandomSet(sample, k, max) (:90-103)
  void unique_set_max(size_t* s, size_t k, size_t max) {
    reset(0, max);
    unique_set(s, k);
  }
  // generateUniqueRandomSet(sample, k, max, to_skip) (:105-123)
  void unique_set_skip(size_t* s, size_t k, size_t max, size_t skip) {
    reset(0, max);
    const uint64_t call = calls++;
    uint32_t d = 0;
    for (size_t i = 0; i < k; ++i) {
      s[i] = next(call, d);
      if (s[i] == skip) { --i; continue; }
      for (int j = (int)i - 1; j >= 0; --j)
        if (s[i] == s[j]) { --i; break; }
      if (d > (1u << 24)) return;
    }
  }
};

// ---------------------------------------------------------------------------
// Samplers (src/pygcransac/include/samplers/sampler.h:44-87 interface).
struct Sampler {
  virtual ~Sampler() {}
  virtual bool sample(const std::vector<size_t>& pool, size_t* subset, size_t k) = 0;
};

// A recorded sample sequence in place of the main sampler: call c returns
// row c of the tape ([calls][k] point indices). A call past the end of the
// tape, or a row holding an index outside [0, n) (a failed call of the
// recording sampler is written as -1), is an unsuccessful sampler call. The
// reference's hook for this is the Sampler* argument of GCRANSAC::run
// (GCRANSAC.h:69-76, samplers/sampler.h:44-87).
struct TapeSampler : Sampler {
  const int32_t* tape;
  int64_t calls;
  size_t n;
  int64_t next = 0;
  TapeSampler(const int32_t* t, int64_t c, size_t n_) : tape(t), calls(c), n(n_) {}
  bool sample(const std::vector<size_t>& pool, size_t* subset, size_t k) override {
    (void)pool;
    const int64_t c = next++;
    if (c >= calls) return false;
    const int32_t* row = tape + (size_t)c * k;
    for (size_t q = 0; q < k; ++q) {
      if (row[q] < 0 || (size_t)row[q] >= n) return false;
      subset[q] = (size_t)row[q];
    }
    return true;
  }
};

// samplers/uniform_sampler.h:97-115
struct UniformSampler : Sampler {
  Generator gen;
  UniformSampler(uint64_t seed, uint32_t stream) : gen(seed, stream) {}
  bool sample(const std::vector<size_t>& pool, size_t* subset, size_t k) override {
    if (k > pool.size()) return false;
    gen.unique_set_max(subset, k, pool.size() - 1);
    for (size_t i = 0; i < k; ++i) subset[i] = pool[subset[i]];
    return true;
  }
};

// samplers/importance_sampler.h:51-136: m independent draws (repeats
// allowed) from the multinomial of the point probabilities. The table is
// std::discrete_distribution's (p_i / sum p, running sums in row order, the
// last entry 1); a draw takes a 53-bit uniform u from stream words 2q and
// 2q + 1 of the call (in place of mt19937) and the first entry not below u.
// One call index per sample.
struct ImportanceSampler : Sampler {
  uint64_t seed;
  uint32_t stream;
  uint64_t calls = 0;
  std::vector<double> cdf;
  ImportanceSampler(uint64_t s, uint32_t st, const double* p, size_t n) : seed(s), stream(st), cdf(n) {
    double sum = 0.0;
    for (size_t i = 0; i < n; ++i) sum += p[i];
    double acc = 0.0;
    for (size_t i = 0; i < n; ++i) {
      acc += p[i] / sum;
      cdf[i] = acc;
    }
    if (n) cdf[n - 1] = 1.0;
  }
  bool sample(const std::vector<size_t>& pool, size_t* subset, size_t k) override {
    (void)pool;
    const uint64_t call = calls++;
    for (size_t q = 0; q < k; ++q) {
      const uint32_t w0 = draw_u32(seed, stream, call, (uint32_t)(2 * q));
      const uint32_t w1 = draw_u32(seed, stream, call, (uint32_t)(2 * q + 1));
      const double u = ((double)(w0 >> 5) * 67108864.0 + (double)(w1 >> 6)) * (1.0 / 9007199254740992.0);
      size_t i = (size_t)(std::lower_bound(cdf.begin(), cdf.end(), u) - cdf.begin());
      subset[q] = i < cdf.size() ? i : cdf.size() - 1;
    }
    return true;
  }
};

// samplers/adaptive_reordering_sampler.h:46-166 with the driver's division
// by the largest probability (gcransac_python.cpp:1731-1736): a max-heap of
// (probability, index); a sample pops the m largest entries and the update
// that follows every sample pushes each sampled point back with
// |a / (a + b + appearances)| + jitter clamped to [0, 0.999]. The jitter,
// rand() in the reference, is 0.01 u / (2^32 - 1) - 0.005 with u draw q of
// the call on stream STREAM_AR; probabilities that are not positive start at
// 1e-12 (the reference divides by zero there). std::priority_queue has the
// reference's tie order (larger index first among equal probabilities).
struct ARSampler : Sampler {
  uint64_t seed;
  uint32_t stream;
  uint64_t calls = 0;
  std::vector<double> a, b;
  std::vector<size_t> cnt;
  std::priority_queue<std::pair<double, size_t>> q;
  ARSampler(uint64_t s, uint32_t st, const double* probs, size_t n, double variance)
      : seed(s), stream(st), a(n), b(n), cnt(n, 0) {
    double mx = 0.0;
    for (size_t i = 0; i < n; ++i) mx = probs[i] > mx ? probs[i] : mx;
    for (size_t i = 0; i < n; ++i) {
      double p = probs[i] / mx;
      if (p == 1.0) p -= 1e-6;
      if (!(p > 1e-12)) p = 1e-12;
      a[i] = p * p * (1.0 - p) / variance - p;
      b[i] = a[i] * (1.0 - p) / p;
      q.emplace(p, i);
    }
  }
  bool sample(const std::vector<size_t>& pool, size_t* subset, size_t k) override {
    (void)pool;
    const uint64_t call = calls++;
    for (size_t i = 0; i < k; ++i) {
      subset[i] = q.top().second;
      q.pop();
    }
    for (size_t i = 0; i < k; ++i) {
      const size_t idx = subset[i];
      ++cnt[idx];
      const double r = std::fabs(a[idx] / (a[idx] + b[idx] + (double)cnt[idx]));
      const double u = (double)draw_u32(seed, stream, call, (uint32_t)i);
      double v = r + 0.01 * (u / 4294967295.0) - 0.005;
      v = v < 0.999 ? v : 0.999;
      v = v > 0.0 ? v : 0.0;
      q.emplace(v, idx);
    }
    return true;
  }
};

// samplers/prosac_sampler.h:51-237
struct ProsacSampler : Sampler {
  size_t sample_size, point_number, convergence, kth = 1, largest, subset_size;
  std::vector<size_t> growth;
  Generator gen;
  ProsacSampler(uint64_t seed, uint32_t stream, size_t m, size_t n, size_t conv = 100000)
      : sample_size(m), point_number(n), convergence(conv), gen(seed, stream) {
    // initialize() (:129-174)
    growth.assign(point_number, 0);
    double T_n = (double)convergence;
    for (size_t i = 0; i < sample_size; ++i) T_n *= (double)(sample_size - i) / (double)(point_number - i);
    size_t T_n_prime = 1;
    for (size_t i = 0; i < point_number; ++i) {
      if (i + 1 <= sample_size) { growth[i] = T_n_prime; continue; }
      const double Tn_plus1 = (double)(i + 1) * T_n / (double)(i + 1 - sample_size);
      growth[i] = T_n_prime + (unsigned int)std::ceil(Tn_plus1 - T_n);
      T_n = Tn_plus1;
      T_n_prime = growth[i];
    }
    largest = sample_size;
    subset_size = sample_size;
    gen.reset(0, subset_size - 1);
  }
  void increment() {  // incrementIterationNumber (:65-87)
    ++kth;
    if (kth > convergence) gen.reset(0, point_number - 1);
    else if (kth > growth[subset_size - 1]) {
      ++subset_size;
      if (subset_size > point_number) subset_size = point_number;
      if (largest < subset_size) largest = subset_size;
      gen.reset(0, subset_size - 2);
    }
  }
  void set_sample_number(size_t k) {  // setSampleNumber (:177-197)
    kth = k;
    if (kth > convergence) gen.reset(0, point_number - 1);
    else
      while (kth > growth[subset_size - 1] && subset_size != point_number) {
        ++subset_size;
        if (subset_size > point_number) subset_size = point_number;
        if (largest < subset_size) largest = subset_size;
        gen.reset(0, subset_size - 2);
      }
  }
  bool sample(const std::vector<size_t>&, size_t* subset, size_t k) override {
    if (k != sample_size) { increment(); return false; }
    if (kth > convergence) { gen.unique_set(subset, k); return true; }
    gen.unique_set(subset, sample_size - 1);
    subset[sample_size - 1] = subset_size - 1;
    increment();
    return true;
  }
};

// ---------------------------------------------------------------------------
// neighborhood/grid_neighborhood_graph.h:132-301. Cells are keyed by
// sum_d idx_d * n^d with idx_d = floor(coord_d / cell_size_d); a point's
// neighbours are all points of its cell (itself included) in index order.
struct Grid {
  std::vector<std::vector<size_t>> cells;  // point lists, first-occurrence order
  std::vector<int64_t> cell_of_point;      // index into cells
  std::vector<uint64_t> keys;              // key of each cell
  std::vector<std::array<uint64_t, 4>> idx;  // cell indices along the four axes
  std::vector<size_t> key_order;           // cells by ascending key
  double cs[4] = {0, 0, 0, 0};
  size_t nd = 0;
  size_t neighbor_number = 0;
  Grid() = default;
  Grid(const Mat& pts, const double cell_sizes[4], size_t n_div) {
    std::unordered_map<uint64_t, size_t> index;
    cell_of_point.assign(pts.rows, -1);
    nd = n_div;
    for (int dd = 0; dd < 4; ++dd) cs[dd] = cell_sizes[dd];
    for (int64_t r = 0; r < pts.rows; ++r) {
      const double* p = pts.row(r);
      uint64_t key = 0, off = 1;
      std::array<uint64_t, 4> ci;
      for (int dd = 0; dd < 4; ++dd) {
        const uint64_t id = (uint64_t)(int64_t)std::floor(p[dd] / cell_sizes[dd]);
        ci[dd] = id;
        key += off * id;
        off *= (uint64_t)n_div;
      }
      auto it = index.find(key);
      size_t c;
      if (it == index.end()) {
        c = cells.size();
        index.emplace(key, c);
        cells.emplace_back();
        keys.push_back(key);
        idx.push_back(ci);
      } else c = it->second;
      cells[c].push_back((size_t)r);
      cell_of_point[r] = (int64_t)c;
    }
    for (auto& c : cells) neighbor_number += c.size() * (c.size() - 1) / 2;
    key_order.resize(cells.size());
    for (size_t c = 0; c < cells.size(); ++c) key_order[c] = c;
    std::sort(key_order.begin(), key_order.end(), [&](size_t a, size_t b) { return keys[a] < keys[b]; });
  }
  const std::vector<size_t>& neighbors(size_t i) const {
    return radius_mode ? radius_nb[i] : cells[cell_of_point[i]];
  }
  bool empty() const { return cells.empty() && radius_nb.empty(); }

  // FlannNeighborhoodGraph (neighborhood/flann_neighborhood_graph.h:100-139)
  // with an exact ball search in place of the approximate k-d tree: the
  // neighbours of i are the j != i whose squared 4-D distance
  // ((a^2 + b^2) + c^2) + d^2 is at most radius^2, in index order.
  bool radius_mode = false;
  std::vector<std::vector<size_t>> radius_nb;
  static Grid radius_graph(const Mat& pts, double radius) {
    Grid g;
    g.radius_mode = true;
    g.radius_nb.assign(pts.rows, {});
    const double r2 = radius * radius;
    for (int64_t i = 0; i < pts.rows; ++i) {
      const double* p = pts.row(i);
      for (int64_t j = 0; j < pts.rows; ++j) {
        if (j == i) continue;
        const double* q = pts.row(j);
        const double a = q[0] - p[0], b = q[1] - p[1], c = q[2] - p[2], d = q[3] - p[3];
        const double d2 = ((a * a + b * b) + c * c) + d * d;
        if (d2 <= r2) g.radius_nb[i].push_back((size_t)j);
      }
      g.neighbor_number += g.radius_nb[i].size();
    }
    g.neighbor_number /= 2;
    return g;
  }
};

// samplers/progressive_napsac_sampler.h:50-326 with layers {16, 8, 4, 2} and
// sampler_length 0.5 as set by the drivers (src/pygcransac/src/gcransac_python.cpp:4333-4343).
struct ProgressiveNapsacSampler : Sampler {
  size_t sample_size, point_number, layer_number, kth = 0, max_iters;
  std::vector<Grid> layers;
  std::vector<size_t> current_layer, hits, subset_size;
  std::vector<size_t> growth;
  ProsacSampler one_point, global;
  Generator gen;
  ProgressiveNapsacSampler(uint64_t seed, const Mat& pts, const std::vector<size_t>& layer_data, size_t m,
                           const double sizes[4], double sampler_length)
      : sample_size(m), point_number(pts.rows), layer_number(layer_data.size()),
        current_layer(pts.rows, 0), hits(pts.rows, 0), subset_size(pts.rows, m),
        one_point(seed, STREAM_NAPSAC_CENTER, 1, pts.rows, pts.rows),
        global(seed, STREAM_NAPSAC_GLOBAL, m, pts.rows, pts.rows),
        gen(seed, STREAM_NAPSAC_LOCAL) {
    gen.reset(0, point_number);
    max_iters = (size_t)(sampler_length * (double)pts.rows);
    for (size_t l = 0; l < layer_number; ++l) {
      double cs[4];
      for (int dd = 0; dd < 4; ++dd) cs[dd] = sizes[dd] / (double)layer_data[l];
      layers.emplace_back(pts, cs, layer_data[l]);
    }
    growth.assign(point_number, 0);
    const size_t local = sample_size - 1;
    double T_n = (double)max_iters;
    for (size_t i = 0; i < local; ++i) T_n *= (double)(local - i) / (double)(point_number - i);
    unsigned int T_n_prime = 1;
    for (size_t i = 0; i < point_number; ++i) {
      if (i + 1 <= local) { growth[i] = T_n_prime; continue; }
      const double Tn_plus1 = (double)(i + 1) * T_n / (double)(i + 1 - local);
      growth[i] = T_n_prime + (size_t)std::ceil(Tn_plus1 - T_n);
      T_n = Tn_plus1;
      T_n_prime = (unsigned int)growth[i];
    }
  }
  bool sample(const std::vector<size_t>& pool, size_t* subset, size_t k) override {
    ++kth;
    if (k != sample_size) return false;
    if (k > pool.size()) return false;
    if (kth > max_iters) {
      global.set_sample_number(kth);
      return global.sample(pool, subset, k);
    }
    if (!one_point.sample(pool, subset, 1)) return false;
    const size_t initial = subset[0];
    size_t& h = ++hits[initial];
    size_t& ss = subset_size[initial];
    while (h > growth[ss - 1] && ss < point_number) ss = std::min(ss + 1, point_number);
    size_t& layer = current_layer[initial];
    bool last = false;
    for (;;) {
      if (layer >= layer_number) { last = true; break; }
      if (layers[layer].neighbors(initial).size() < ss) { ++layer; continue; }
      break;
    }
    if (!last) {
      const std::vector<size_t>& nb = layers[layer].neighbors(initial);
      subset[sample_size - 1] = initial;
      subset[sample_size - 2] = nb[ss - 1];
      gen.unique_set_skip(subset, k - 2, ss - 2, initial);
      for (size_t i = 0; i < k - 2; ++i) {
        subset[i] = nb[subset[i]];
        ++hits[subset[i]];
      }
      ++hits[subset[k - 2]];
    } else {
      global.set_sample_number(kth);
      const bool ok = global.sample(pool, subset, k);
      subset[sample_size - 1] = initial;
      return ok;
    }
    return true;
  }
};

// GCRANSAC::getIterationNumber (src/pygcransac/include/GCRANSAC.h:156-172)
inline size_t iteration_number_for(size_t inliers, size_t points, size_t m, double log_prob) {
  const double q = std::pow((double)inliers / (double)points, (double)m);
  const double l2 = std::log(1 - q);
  if (std::abs(l2) < std::numeric_limits<double>::epsilon()) return std::numeric_limits<size_t>::max();
  const double iter = log_prob / l2;
  return (size_t)iter + 1;
}

inline double det3(const Model& m) {
  return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
         m[2] * (m[3] * m[7] - m[4] * m[6]);
}

inline bool inverse3(const double* m, double* out) {
  const double c00 = m[4] * m[8] - m[5] * m[7];
  const double c01 = m[5] * m[6] - m[3] * m[8];
  const double c02 = m[3] * m[7] - m[4] * m[6];
  const double det = m[0] * c00 + m[1] * c01 + m[2] * c02;
  if (det == 0) return false;
  const double id = 1.0 / det;
  out[0] = c00 * id;
  out[1] = (m[2] * m[7] - m[1] * m[8]) * id;
  out[2] = (m[1] * m[5] - m[2] * m[4]) * id;
  out[3] = c01 * id;
  out[4] = (m[0] * m[8] - m[2] * m[6]) * id;
  out[5] = (m[2] * m[3] - m[0] * m[5]) * id;
  out[6] = c02 * id;
  out[7] = (m[1] * m[6] - m[0] * m[7]) * id;
  out[8] = (m[0] * m[4] - m[1] * m[3]) * id;
  return true;
}

inline void matmul3(const double* a, const double* b, double* c) {
  double t[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) t[i * 3 + j] = a[i * 3] * b[j] + a[i * 3 + 1] * b[3 + j] + a[i * 3 + 2] * b[6 + j];
  std::memcpy(c, t, sizeof t);
}

}  // namespace oracle
