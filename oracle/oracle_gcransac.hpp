// Oracle (test infrastructure only): graph-cut labelling, MSAC / MAGSAC++
// scoring and the GC-RANSAC loop, restated from
// src/pygcransac/include/GCRANSAC.h and scoring_function.h of the reference.
#pragma once

#include "oracle_common.hpp"

namespace oracle {

// ---------------------------------------------------------------------------
// s-t min cut for the labelling step. The reference builds an
// Energy<double,double,double> (src/pygcransac/include/energy.h:203-253) and
// runs Boykov-Kolmogorov max-flow (maxflow.cpp:471-607); a node is an inlier
// iff what_segment() is SINK (GCRANSAC.h:1014-1017), i.e. iff the node can
// still reach the sink in the residual graph of a maximum flow. That set is the
// same for every maximum flow, so this oracle uses Dinic's algorithm followed
// by a reverse residual search from the sink. Residuals at or below kResidualEps
// count as saturated (the engine uses the same rule).
constexpr double kResidualEps = 1e-12;

struct FlowGraph {
  struct Arc { int to; int rev; double cap; };
  int n, S, T;
  std::vector<std::vector<Arc>> adj;
  explicit FlowGraph(int n_) : n(n_), S(n_), T(n_ + 1), adj(n_ + 2) {}
  void add_arc_pair(int u, int v, double c_uv, double c_vu) {
    adj[u].push_back({v, (int)adj[v].size(), c_uv});
    adj[v].push_back({u, (int)adj[u].size() - 1, c_vu});
  }
  std::vector<int> level, it;
  bool bfs() {
    level.assign(n + 2, -1);
    std::vector<int> q;
    q.reserve(n + 2);
    q.push_back(S);
    level[S] = 0;
    for (size_t h = 0; h < q.size(); ++h) {
      const int u = q[h];
      for (const Arc& a : adj[u])
        if (a.cap > 0 && level[a.to] < 0) { level[a.to] = level[u] + 1; q.push_back(a.to); }
    }
    return level[T] >= 0;
  }
  double dfs(int u, double f) {
    if (u == T) return f;
    for (int& i = it[u]; i < (int)adj[u].size(); ++i) {
      Arc& a = adj[u][i];
      if (a.cap > 0 && level[a.to] == level[u] + 1) {
        const double d = dfs(a.to, std::min(f, a.cap));
        if (d > 0) {
          a.cap -= d;
          adj[a.to][a.rev].cap += d;
          return d;
        }
      }
    }
    return 0;
  }
  void maxflow() {
    for (int rounds = 0; rounds < 1000000 && bfs(); ++rounds) {
      it.assign(n + 2, 0);
      while (dfs(S, std::numeric_limits<double>::infinity()) > 0) {}
    }
  }
  // Nodes that reach T through arcs of residual capacity > kResidualEps.
  std::vector<char> sink_side() {
    std::vector<char> mark(n + 2, 0);
    std::vector<int> q{T};
    mark[T] = 1;
    for (size_t h = 0; h < q.size(); ++h) {
      const int v = q[h];
      for (const Arc& a : adj[v]) {
        // a: v -> u; residual of u -> v is the sister arc
        const int u = a.to;
        if (mark[u]) continue;
        if (adj[u][a.rev].cap > kResidualEps) { mark[u] = 1; q.push_back(u); }
      }
    }
    return mark;
  }
};

// ---------------------------------------------------------------------------
// MSACScoringFunction::getScore (scoring_function.h:137-233). The early-exit
// test at :182 compares (N - i) + sum r^2 against -best and cannot fire for a
// non-negative best score, so it is omitted.
template <class Est>
struct MSACScoring {
  double sq_trunc = 0;
  void initialize(double sq, size_t) { sq_trunc = sq; }
  Score get(const Mat& pts, const Model& m, const Est& est, std::vector<size_t>* inliers) const {
    Score s;
    if (inliers) inliers->clear();
    for (int64_t i = 0; i < pts.rows; ++i) {
      const double r2 = est.squared_residual(pts.row(i), m);
      if (r2 < sq_trunc) {
        if (inliers) inliers->push_back((size_t)i);
        ++s.inlier_number;
        s.value -= r2;
      }
    }
    if (s.inlier_number == 0) return Score();
    s.value = (s.value + (double)s.inlier_number * sq_trunc) / sq_trunc;
    return s;
  }
  // getScore over index sets (scoring_function.h:186-218): the listed points
  // in order
  Score get_subset(const Mat& pts, const Model& m, const Est& est, const std::vector<size_t>& idx,
                   std::vector<size_t>* inliers) const {
    Score s;
    if (inliers) inliers->clear();
    for (size_t i : idx) {
      const double r2 = est.squared_residual(pts.row(i), m);
      if (r2 < sq_trunc) {
        if (inliers) inliers->push_back(i);
        ++s.inlier_number;
        s.value -= r2;
      }
    }
    if (s.inlier_number == 0) return Score();
    s.value = (s.value + (double)s.inlier_number * sq_trunc) / sq_trunc;
    return s;
  }
};

// MAGSACScoringFunction::getScore (scoring_function.h:237-348). The weight
// table stored_gamma_values[x] (gamma_values.cpp:2012) holds the upper
// incomplete gamma function Gamma(1.5, x / 1000) for x = 0..36000; it is
// regenerated here from that definition (checked against the reference table
// text by the tests).
struct MagsacTable {
  std::vector<double> g;
  MagsacTable();
};
const MagsacTable& magsac_table();

template <class Est>
struct MAGSACScoring {
  double threshold = 0;  // settings.threshold (not the 1.5x truncated one)
  void initialize(double, size_t) {}
  // MAGSAC++ scores every point even when index sets are given
  // (scoring_function.h:253-304)
  template <class Idx>
  Score get_subset(const Mat& pts, const Model& m, const Est& est, const Idx&, std::vector<size_t>* inliers) const {
    return get(pts, m, est, inliers);
  }
  Score get(const Mat& pts, const Model& m, const Est& est, std::vector<size_t>* inliers) const {
    constexpr double k = 3.64;
    constexpr double C = 0.25;
    constexpr double gamma_k = 0.0036572608340910764;
    const double two_ad_dof = std::pow(2.0, 1.5);
    const double C_times_two_ad_dof = C * two_ad_dof;
    const double gamma_value = std::tgamma(1.5);
    const double gamma_difference = gamma_value - gamma_k;
    const double squared_sigma_max_2 = threshold * threshold * 2.0;
    const double one_over_sigma = C_times_two_ad_dof / threshold;
    const double weight_zero = one_over_sigma * gamma_difference;
    (void)k;
    const std::vector<double>& table = magsac_table().g;
    Score s;
    if (inliers) inliers->clear();
    for (int64_t i = 0; i < pts.rows; ++i) {
      const double r = std::sqrt(est.squared_residual(pts.row(i), m));
      if (r > threshold) continue;
      double w;
      if (r < std::numeric_limits<double>::epsilon()) w = weight_zero;
      else {
        size_t x = (size_t)std::round(1e4 * (r * r) / squared_sigma_max_2);
        if (36000 < x) x = 36000;
        w = one_over_sigma * (table[x] - gamma_k);
      }
      s.value += w / weight_zero;
      if (r > threshold) continue;
      ++s.inlier_number;
      if (inliers) inliers->push_back((size_t)i);
    }
    return s;
  }
};

// ---------------------------------------------------------------------------
// SpacePartitioningRANSAC::runHomography (inlier_selectors/
// space_partitioning_ransac.h:341-505): a cell with fewer than four points is
// always kept; otherwise its four source-image corners are mapped by H and
// the cell is kept when one lands in the cell's destination indices or when
// the threshold-grown box of the mapped corners 00 and 11 overlaps the
// destination cell. Cells are visited by ascending key (the reference visits
// them in std::unordered_map order, which is library-specific). A mapped
// coordinate outside the int range (or NaN) converts to INT_MIN.
inline int sp_trunc_int(double v) {
  if (!(v > -2147483649.0 && v < 2147483648.0)) return std::numeric_limits<int>::min();
  return (int)v;
}

inline void sp_select(const Grid& g, const Model& H, double thr, std::vector<size_t>& sel, size_t& point_number) {
  sel.clear();
  point_number = 0;
  if (std::fabs(det3(H)) < 1e-3) return;
  const double cs1 = g.cs[0], cs2 = g.cs[1], cs3 = g.cs[2], cs4 = g.cs[3];
  const uint64_t n = (uint64_t)g.nd;
  auto proj = [&](uint64_t hx, uint64_t vy, double& x, double& y) {
    const double X1 = (double)hx * cs1, Y1 = (double)vy * cs2;
    double x2p = X1 * H[0] + Y1 * H[1] + H[2], y2p = X1 * H[3] + Y1 * H[4] + H[5],
           h2p = X1 * H[6] + Y1 * H[7] + H[8];
    x2p /= h2p;
    y2p /= h2p;
    x = x2p;
    y = y2p;
  };
  const int steps[8] = {0, 0, 0, 1, 1, 0, 1, 1};
  for (size_t c : g.key_order) {
    const std::vector<size_t>& points = g.cells[c];
    if (points.size() < 4) {
      sel.push_back(c);
      point_number += points.size();
      continue;
    }
    const std::array<uint64_t, 4>& ci = g.idx[c];
    bool overlaps = false;
    double c00x = 0, c00y = 0, c11x = 0, c11y = 0;
    for (int st = 0; st < 8; st += 2) {
      const uint64_t hx = ci[0] + (uint64_t)steps[st];
      if (hx >= n) continue;
      const uint64_t vy = ci[1] + (uint64_t)steps[st + 1];
      if (vy >= n) continue;
      double x, y;
      proj(hx, vy, x, y);
      if (st == 0) { c00x = x; c00y = y; }
      if (st == 6) { c11x = x; c11y = y; }
      const int ix = sp_trunc_int(x / cs3), iy = sp_trunc_int(y / cs4);
      if ((uint64_t)(int64_t)ix == ci[2] && (uint64_t)(int64_t)iy == ci[3]) {
        sel.push_back(c);
        point_number += points.size();
        overlaps = true;
        break;
      }
    }
    if (!overlaps) {
      const uint64_t hx11 = ci[0] + 1, vy11 = ci[1] + 1;
      if (vy11 >= n || hx11 >= n) proj(hx11, vy11, c11x, c11y);
      const double l1x = c00x - thr, l1y = c00y - thr, r1x = c11x + thr, r1y = c11y + thr;
      const double l2x = cs3 * (double)ci[2], l2y = cs4 * (double)ci[3];
      const double r2x = l2x + cs3, r2y = l2y + cs4;
      if ((l1x <= r2x && l2x <= r1x) || (r1y <= l2y && r2y <= l1y)) {
        sel.push_back(c);
        point_number += points.size();
      }
    }
  }
}

// ---------------------------------------------------------------------------
// SPRTPreemptiveVerfication (preemption/preemption_sprt.h:50-380). Two inputs
// of the reference are not reproducible and are replaced: the point order is a
// Fisher-Yates permutation with the reference's loop structure whose draws
// come from Philox stream 3 instead of rand(), and t_M is 1/m (the reference
// gets 1/m whenever its first-sample estimate returns a model, because the
// timer it divides by is not restarted; otherwise it uses a wall-clock time).
struct Sprt {
  std::vector<size_t> pool;
  size_t cursor = 0;
  double epsilon = 0, delta = 0, A = 0;
  size_t last_update = 0;
  double t_M = 1, m_S = 1, amp = 1.0;

  void init(size_t N, size_t m, size_t max_solutions, double min_ratio, uint64_t seed) {
    pool.resize(N);
    for (size_t i = 0; i < N; ++i) pool[i] = i;
    size_t max = N;
    for (size_t i = 0; i < N; ++i) {
      const size_t idx = draw_u32(seed, STREAM_SPRT, 0, (uint32_t)i) % max;
      const size_t t = pool[idx];
      --max;
      pool[idx] = pool[max];
      pool[max] = t;
    }
    cursor = 0;
    t_M = 1.0 / (double)m;
    m_S = (double)max_solutions;
    delta = min_ratio / 10.0;
    epsilon = min_ratio;
    A = threshold_A(epsilon, delta);
    last_update = 0;
  }
  // estimateThresholdA (preemption_sprt.h:361-379)
  double threshold_A(double eps, double del) const {
    const double C = (1 - del) * std::log((1 - del) / (1 - eps)) + del * (std::log(del / eps));
    const double K = (t_M * C) / m_S + 1;
    double An_1 = K, An = K;
    for (unsigned i = 0; i < 10; ++i) {
      An = K + std::log(An_1);
      if (std::fabs(An - An_1) < 1.5e-8) break;
      An_1 = An;
    }
    return An;
  }
  // verifyModel (preemption_sprt.h:232-347). Without index sets the points
  // are taken from the pool, continuing at the cursor; with index sets (space
  // partitioning) the listed points are walked in order and the cursor stays.
  // Writes the tested inliers in walk order; returns whether the model passed.
  template <class Est>
  bool verify(const Mat& pts, const Model& model, const Est& est, double threshold, size_t iteration,
              const Score& best, std::vector<size_t>& inliers, Score& score,
              const std::vector<size_t>* index_set = nullptr) {
    inliers.clear();
    const size_t N = (size_t)pts.rows;
    const double sq = threshold * threshold;
    const double eps = epsilon, del = delta, a = A;
    double lambda = 1, lambda_new;
    score = Score();
    bool valid = true;
    if (index_set) {
      for (size_t idx : *index_set) {
        const double r2 = est.squared_residual(pts.row(idx), model);
        if (r2 < sq) {
          lambda_new = lambda * (del / eps);
          ++score.inlier_number;
          score.value += 1.0 - r2 / sq;
          inliers.push_back(idx);
        } else {
          lambda_new = lambda * ((1 - del) / (1 - eps));
        }
        if (lambda_new > a * amp) {
          valid = false;
          break;
        }
        lambda = lambda_new;
      }
    }
    for (size_t t = 0; t < N && !index_set; ++t) {
      const size_t idx = pool[cursor];
      const double r2 = est.squared_residual(pts.row(idx), model);
      if (r2 < sq) {
        lambda_new = lambda * (del / eps);
        ++score.inlier_number;
        score.value += 1.0 - r2 / sq;
        inliers.push_back(idx);
      } else {
        lambda_new = lambda * ((1 - del) / (1 - eps));
      }
      if (++cursor >= N) cursor = 0;
      if (lambda_new > a * amp) {
        valid = false;
        break;
      }
      lambda = lambda_new;
    }
    if (valid) {
      if (score.value > best.value) {
        epsilon = (double)score.inlier_number / N;
        A = threshold_A(epsilon, del);
        last_update = iteration;
      }
    } else {
      const double de = (double)score.inlier_number / N;
      if (de > 0 && std::fabs(del - de) / del > 0.05) {
        delta = de;
        A = threshold_A(eps, de);
        last_update = iteration;
      }
    }
    return valid;
  }
};

// ---------------------------------------------------------------------------
// GCRANSAC<Estimator, GridNeighborhoodGraph<4>, Scoring>::run, restated from
// GCRANSAC.h:200-627 together with graphCutLocalOptimization (779-910),
// labeling (912-1021) and iteratedLeastSquaresFitting (629-758).
template <class Est, class Scoring>
struct GCRansac {
  Settings settings;
  Statistics statistics;
  Scoring scoring;
  double truncated_threshold = 0, squared_truncated_threshold = 0, log_probability = 0;
  const Grid* graph = nullptr;
  size_t models_scored = 0;  // main-loop models + LO trials + IRLS fits
  uint64_t sprt_seed = 0;    // seed of the SPRT point permutation
  Sampler* main_sampler = nullptr;
  Sampler* lo_sampler = nullptr;

  // labeling (GCRANSAC.h:912-1021)
  void labeling(const Mat& pts, const Model& model, const Est& est, double lambda, double thr,
                std::vector<size_t>& inliers) {
    const int64_t N = pts.rows;
    const double sq = thr * thr * 9 / 4;
    const double oml = 1.0 - lambda;
    std::vector<double> d(N), tr(N, 0.0);
    for (int64_t i = 0; i < N; ++i) {
      const double r2 = est.squared_residual(pts.row(i), model);
      d[i] = std::min(std::max(r2 / sq, 0.0), 1.0);
      const double e = 1 - d[i];
      // add_term1(i, E0, E1) = add_tweights(i, E1, E0): tr_cap = E1 - E0
      if (r2 <= sq) tr[i] = 0 - oml * e;
      else tr[i] = oml * (1 - e) - 0;
    }
    FlowGraph g((int)N);
    if (lambda > 0 && graph) {
      // Each unordered pair of a cell once, smaller index first
      // (the used_edges de-duplication of GCRANSAC.h:963-989).
      for (int64_t i = 0; i < N; ++i) {
        for (size_t j : graph->neighbors((size_t)i)) {
          if ((int64_t)j <= i) continue;
          const double e00 = 0.5 * (d[i] + d[j]);
          // add_term2(i, j, e00*l, l, l, 0): tweights(i, 0, e00*l), edge(i, j, l - e00*l, l)
          const double A = e00 * lambda;
          tr[i] = tr[i] - A;
          g.add_arc_pair((int)i, (int)j, lambda - A, lambda);
        }
      }
    }
    for (int64_t i = 0; i < N; ++i) {
      if (tr[i] > 0) g.add_arc_pair(g.S, (int)i, tr[i], 0.0);
      else if (tr[i] < 0) g.add_arc_pair((int)i, g.T, -tr[i], 0.0);
    }
    g.maxflow();
    const std::vector<char> sink = g.sink_side();
    inliers.clear();
    for (int64_t i = 0; i < N; ++i)
      if (sink[i]) inliers.push_back((size_t)i);
  }

  bool gc_local_optimization(const Mat& pts, std::vector<size_t>& best_inliers_io, Model& best_model_io,
                             Score& best_score_io, const Est& est, size_t trials) {
    const size_t inlier_limit = est.inlier_limit();
    Score max_score = best_score_io;
    Model best_model = best_model_io;
    std::vector<Model> models;
    std::vector<size_t> best_inliers, inliers, tmp;
    ++statistics.local_optimization_number;
    std::vector<size_t> sample(inlier_limit);
    while (++statistics.graph_cut_number < settings.max_graph_cut_number) {
      bool updated = false;
      inliers.clear();
      labeling(pts, best_model, est, settings.spatial_coherence_weight, settings.threshold, inliers);
      const size_t ss = std::min(inlier_limit, inliers.size());
      for (size_t trial = 0; trial < trials; ++trial) {
        models.clear();
        if (ss < inliers.size()) {
          lo_sampler->sample(inliers, sample.data(), ss);
          if (!est.estimate_nonminimal(pts, sample.data(), ss, models, nullptr)) continue;
        } else if (est.sample_size_rt() < inliers.size()) {
          if (!est.estimate_nonminimal(pts, inliers.data(), inliers.size(), models, nullptr)) break;
        } else
          break;
        for (Model& m : models) {
          tmp.clear();
          ++models_scored;
          const Score s = scoring.get(pts, m, est, &tmp);
          if (max_score < s) {
            updated = true;
            max_score = s;
            best_model = m;
            best_inliers.swap(tmp);
            tmp.clear();
          }
        }
      }
      if (!updated) break;
    }
    if (best_score_io < max_score) {
      best_score_io = max_score;
      best_model_io = best_model;
      best_inliers_io.swap(best_inliers);
      return true;
    }
    return false;
  }

  bool irls(const Mat& pts, const Est& est, std::vector<size_t>& inliers, Model& model) {
    const size_t m = est.sample_size_rt();
    if (inliers.size() <= m) return false;
    size_t iterations = 0;
    std::vector<size_t> tmp;
    std::vector<double> weights(pts.rows, 0.0);
    Score best_score;
    while (++iterations < settings.max_least_squares_iterations) {
      std::vector<Model> models;
      for (size_t k = 0; k < inliers.size(); ++k) {
        const size_t p = inliers[k];
        const double r2 = est.squared_residual(pts.row(p), model);
        const double w = std::max(0.0, 1.0 - r2 / squared_truncated_threshold);
        weights[p] = w * w;
      }
      est.estimate_nonminimal(pts, inliers.data(), inliers.size(), models, weights.data());
      for (size_t p : inliers) weights[p] = 0;
      if (models.empty()) break;
      if (models.size() == 1) {
        tmp.clear();
        ++models_scored;
        const Score s = scoring.get(pts, models[0], est, &tmp);
        if (tmp.size() < m) break;
        if (s.inlier_number <= inliers.size()) break;
        model = models[0];
        inliers.swap(tmp);
      } else {
        bool updated = false;
        for (Model& mm : models) {
          tmp.clear();
          ++models_scored;
          const Score s = scoring.get(pts, mm, est, &tmp);
          if (tmp.size() < m) continue;
          if (s.inlier_number <= inliers.size()) continue;
          if (s.inlier_number >= best_score.inlier_number) {
            updated = true;
            best_score = s;
            model = mm;
            inliers.swap(tmp);
          }
        }
        if (!updated) break;
      }
    }
    return iterations > 1;
  }

  // Returns true when a model was found.
  bool run(const Mat& pts, const Est& est, Sampler* main_s, Sampler* lo_s, const Grid* g, Model& out) {
    statistics = Statistics();
    models_scored = 0;
    main_sampler = main_s;
    lo_sampler = lo_s;
    graph = g;
    statistics.neighbor_number = g ? g->neighbor_number : 0;
    const size_t m = est.sample_size_rt();
    log_probability = std::log(1.0 - settings.confidence);
    size_t max_iteration = iteration_number_for(1, pts.rows, m, log_probability);
    std::vector<size_t> sample(m);
    const size_t N = (size_t)pts.rows;
    size_t off = 0;
    Model best_model{};
    Score current_score, best_score;
    std::vector<std::vector<size_t>> cont(2);
    truncated_threshold = 1.5 * settings.threshold;
    squared_truncated_threshold = truncated_threshold * truncated_threshold;
    scoring.initialize(squared_truncated_threshold, N);
    std::vector<size_t> pool(N);
    for (size_t i = 0; i < N; ++i) pool[i] = i;
    std::vector<Model> models;
    Sprt sprt;
    if (settings.use_sprt) sprt.init(N, m, Est::max_solutions(), settings.sprt_min_inlier_ratio, sprt_seed);
    const bool use_sp = settings.use_space_partitioning && Est::space_partitioning && graph != nullptr;
    std::vector<size_t> sp_cells, sp_points;
    while (settings.min_iteration_number > statistics.iteration_number ||
           statistics.iteration_number < std::min(max_iteration, settings.max_iteration_number)) {
      bool do_lo = false;
      ++statistics.iteration_number;
      models.clear();
      int unsuccessful = -1;
      while (++unsuccessful < (int)settings.max_unsuccessful_model_generations) {
        if (!main_sampler->sample(pool, sample.data(), m)) continue;
        if (!est.is_valid_sample(pts, sample.data())) continue;
        if (est.estimate_minimal(pts, sample.data(), models)) break;
      }
      statistics.iteration_number += unsuccessful;
      for (Model& model : models) {
        ++models_scored;
        const std::vector<size_t>* sel_pts = nullptr;
        if (use_sp) {
          // GCRANSAC.h:343-366: reject when the selected cells hold fewer
          // points than the best model has inliers
          size_t sel_n = 0;
          sp_select(*graph, model, truncated_threshold, sp_cells, sel_n);
          if (sel_n < best_score.inlier_number) continue;
          sp_points.clear();
          for (size_t c : sp_cells)
            for (size_t p : graph->cells[c]) sp_points.push_back(p);
          sel_pts = &sp_points;
        }
        if (settings.use_sprt) {
          // SPRT provides the score (GCRANSAC.h:370-431)
          if (!sprt.verify(pts, model, est, truncated_threshold, statistics.iteration_number, best_score, cont[off],
                           current_score, sel_pts))
            continue;
        } else if (sel_pts) {
          current_score = scoring.get_subset(pts, model, est, *sel_pts, &cont[off]);
        } else {
          current_score = scoring.get(pts, model, est, &cont[off]);
        }
        bool updated_model = false;
        if (best_score < current_score &&
            est.is_valid_model(model, pts, cont[off], sample.data(), truncated_threshold, updated_model)) {
          if (updated_model) current_score = scoring.get(pts, model, est, &cont[off]);
          off = (off + 1) % 2;
          best_model = model;
          best_score = current_score;
          do_lo = statistics.iteration_number > settings.min_iteration_number_before_lo &&
                  best_score.inlier_number > m;
          max_iteration = iteration_number_for(best_score.inlier_number, N, m, log_probability);
        }
      }
      if (settings.do_local_optimization && do_lo) {
        ++statistics.local_optimization_number;
        gc_local_optimization(pts, cont[off], best_model, best_score, est, settings.max_local_optimization_number);
        max_iteration = iteration_number_for(best_score.inlier_number, N, m, log_probability);
      }
    }
    if (best_score.inlier_number <= m) return false;
    if (settings.do_local_optimization && statistics.local_optimization_number == 0) {
      ++statistics.local_optimization_number;
      gc_local_optimization(pts, cont[off], best_model, best_score, est, settings.max_local_optimization_number);
    }
    if (cont[off].size() != best_score.inlier_number) off = (off + 1) % 2;
    if (cont[off].size() != best_score.inlier_number) best_score = scoring.get(pts, best_model, est, &cont[off]);
    bool irls_applied = false;
    if (settings.do_final_iterated_least_squares) {
      Model model = best_model;
      const bool ok = irls(pts, est, cont[off], model);
      if (ok) {
        const size_t idx = (off + 1) % 2;
        cont[idx].clear();
        current_score = scoring.get(pts, model, est, &cont[idx]);
        if (best_score < current_score) {
          irls_applied = true;
          best_model = model;
          off = idx;
        }
      }
    }
    if (!irls_applied) {
      models.clear();
      est.estimate_nonminimal(pts, cont[off].data(), best_score.inlier_number, models, nullptr);
      for (Model& model : models) {
        const size_t idx = (off + 1) % 2;
        cont[idx].clear();
        current_score = scoring.get(pts, model, est, &cont[idx]);
        if (best_score < current_score) {
          best_model = model;
          off = idx;
        }
      }
    }
    statistics.irls_applied = irls_applied;
    statistics.inliers.swap(cont[off]);
    statistics.score = best_score.value;
    out = best_model;
    return true;
  }
};

}  // namespace oracle
