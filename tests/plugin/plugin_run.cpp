// Test driver of the C++ plugin surface (include/gcransac/GCRANSAC.h): reads
// one pair and its configuration, runs gcransac::GCRANSAC<...>::run with the
// library's plugin types, writes the model, the inliers and the statistics.
//   plugin_run IN OUT
// IN  (little-endian): int32 kind, sampler, scoring, sprt, space_partitioning,
//     divisions (0: the radius graph, radius cell[0]); int64 n; double
//     threshold, confidence, lambda; int64
//     max_iterations, min_iterations; int32 lo_number; uint64 seed; double
//     sprt_ratio, cell[4], sizes[4]; double points[n][4], pixels[n][4],
//     K1[9], K2[9]; double sampler_variance, probabilities[n] (read by samplers
//     3 and 4)
// OUT int32 has_model; double model[9]; int64 iterations, graph_cuts,
//     local_optimisations; double score; int64 inlier count, inliers[]
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "gcransac/GCRANSAC.h"

using namespace gcransac;

struct Input {
  int32_t kind, sampler, scoring, sprt, sp, divisions;
  int64_t n;
  double threshold, confidence, lambda;
  int64_t max_it, min_it;
  int32_t lo;
  uint64_t seed;
  double sprt_ratio, cell[4], sizes[4];
  std::vector<double> points, pixels;
  double K1[9], K2[9];
  double variance;
  std::vector<double> probs;
};

template <class T>
static void rd(FILE* f, T* v, size_t k = 1) {
  if (fread(v, sizeof(T), k, f) != k) {
    fprintf(stderr, "short input\n");
    exit(2);
  }
}

template <class Graph>
Graph make_graph(const Input& in, const MatView* pixels);
template <>
neighborhood::GridNeighborhoodGraph<4> make_graph(const Input& in, const MatView* pixels) {
  return neighborhood::GridNeighborhoodGraph<4>(pixels, {in.cell[0], in.cell[1], in.cell[2], in.cell[3]},
                                                (size_t)in.divisions);
}
template <>
neighborhood::FlannNeighborhoodGraph make_graph(const Input& in, const MatView* pixels) {
  return neighborhood::FlannNeighborhoodGraph(pixels, in.cell[0]);
}

template <class Est, template <class> class Scoring, bool SPRT, bool SP, class Graph>
static int run_case(const Input& in, const Est& est, FILE* out) {
  using Pre = typename std::conditional<SPRT, preemption::SPRTPreemptiveVerfication<Est>,
                                        preemption::EmptyPreemptiveVerfication<Est>>::type;
  using Sel = typename std::conditional<SP, inlier_selector::SpacePartitioningRANSAC<Est, Graph>,
                                        inlier_selector::EmptyInlierSelector<Est, Graph>>::type;
  const MatView points(in.points.data(), (int)in.n, 4), pixels(in.pixels.data(), (int)in.n, 4);
  Graph graph = make_graph<Graph>(in, &pixels);
  sampler::UniformSampler uniform(&pixels), lo_sampler(&pixels);
  sampler::ProsacSampler prosac(&pixels, Est::sampleSize());
  std::vector<double> sizes(in.sizes, in.sizes + 4);
  sampler::ProgressiveNapsacSampler<4>* pnapsac = nullptr;
  if (in.sampler == GCR_SAMPLER_PNAPSAC)
    pnapsac = new sampler::ProgressiveNapsacSampler<4>(&pixels, {16, 8, 4, 2}, Est::sampleSize(), sizes, 0.5);
  sampler::ImportanceSampler importance(&pixels, in.probs, Est::sampleSize());
  sampler::AdaptiveReorderingSampler* ar = nullptr;
  if (in.sampler == GCR_SAMPLER_AR)
    ar = new sampler::AdaptiveReorderingSampler(&pixels, in.probs, Est::sampleSize(), in.variance);
  sampler::Sampler<MatView, size_t>* main_sampler =
      in.sampler == GCR_SAMPLER_UNIFORM      ? (sampler::Sampler<MatView, size_t>*)&uniform
      : in.sampler == GCR_SAMPLER_PROSAC     ? (sampler::Sampler<MatView, size_t>*)&prosac
      : in.sampler == GCR_SAMPLER_IMPORTANCE ? (sampler::Sampler<MatView, size_t>*)&importance
      : in.sampler == GCR_SAMPLER_AR         ? (sampler::Sampler<MatView, size_t>*)ar
                                             : (sampler::Sampler<MatView, size_t>*)pnapsac;
  GCRANSAC<Est, Graph, Scoring<Est>, Pre, Sel> g;
  g.settings.threshold = in.threshold;
  g.settings.confidence = in.confidence;
  g.settings.spatial_coherence_weight = in.lambda;
  g.settings.max_iteration_number = (size_t)in.max_it;
  g.settings.min_iteration_number = (size_t)in.min_it;
  g.settings.max_local_optimization_number = (size_t)in.lo;
  g.seed = in.seed;
  Model model;
  Pre pre = [&]() {
    if constexpr (SPRT) return Pre(points, est, in.sprt_ratio);
    else return Pre();
  }();
  Sel sel(&graph);
  g.run(points, est, main_sampler, &lo_sampler, &graph, model, pre, sel);
  const auto& st = g.getRansacStatistics();
  const int32_t has = model.descriptor.rows() == 3;
  fwrite(&has, 4, 1, out);
  fwrite(model.descriptor.v, 8, 9, out);
  const int64_t it = (int64_t)st.iteration_number, gc = (int64_t)st.graph_cut_number,
                lo = (int64_t)st.local_optimization_number, ni = (int64_t)st.inliers.size();
  fwrite(&it, 8, 1, out);
  fwrite(&gc, 8, 1, out);
  fwrite(&lo, 8, 1, out);
  fwrite(&st.score, 8, 1, out);
  fwrite(&ni, 8, 1, out);
  for (size_t i : st.inliers) {
    const int64_t v = (int64_t)i;
    fwrite(&v, 8, 1, out);
  }
  delete pnapsac;
  delete ar;
  return 0;
}

template <class Est, bool SP, class Graph>
static int dispatch_graph(const Input& in, const Est& est, FILE* out) {
  if (in.scoring == GCR_SCORING_MAGSAC) {
    if (in.sprt) return run_case<Est, MAGSACScoringFunction, true, SP, Graph>(in, est, out);
    return run_case<Est, MAGSACScoringFunction, false, SP, Graph>(in, est, out);
  }
  if (in.sprt) return run_case<Est, MSACScoringFunction, true, SP, Graph>(in, est, out);
  return run_case<Est, MSACScoringFunction, false, SP, Graph>(in, est, out);
}

template <class Est, bool SP>
static int dispatch(const Input& in, const Est& est, FILE* out) {
  if (in.divisions == 0) {
    if constexpr (SP) return 2;  // space partitioning needs the grid
    else return dispatch_graph<Est, false, neighborhood::FlannNeighborhoodGraph>(in, est, out);
  }
  return dispatch_graph<Est, SP, neighborhood::GridNeighborhoodGraph<4>>(in, est, out);
}

int main(int argc, char** argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: plugin_run IN OUT\n");
    return 2;
  }
  FILE* f = fopen(argv[1], "rb");
  if (!f) return 2;
  Input in;
  rd(f, &in.kind); rd(f, &in.sampler); rd(f, &in.scoring); rd(f, &in.sprt); rd(f, &in.sp); rd(f, &in.divisions);
  rd(f, &in.n); rd(f, &in.threshold); rd(f, &in.confidence); rd(f, &in.lambda); rd(f, &in.max_it);
  rd(f, &in.min_it); rd(f, &in.lo); rd(f, &in.seed); rd(f, &in.sprt_ratio); rd(f, in.cell, 4); rd(f, in.sizes, 4);
  in.points.resize((size_t)in.n * 4);
  in.pixels.resize((size_t)in.n * 4);
  rd(f, in.points.data(), in.points.size());
  rd(f, in.pixels.data(), in.pixels.size());
  rd(f, in.K1, 9);
  rd(f, in.K2, 9);
  rd(f, &in.variance);
  in.probs.resize((size_t)in.n);
  rd(f, in.probs.data(), in.probs.size());
  fclose(f);
  FILE* out = fopen(argv[2], "wb");
  if (!out) return 2;
  int rc = 2;
  try {
    if (in.kind == GCR_HOMOGRAPHY) {
      utils::DefaultHomographyEstimator est;
      rc = in.sp ? dispatch<utils::DefaultHomographyEstimator, true>(in, est, out)
                 : dispatch<utils::DefaultHomographyEstimator, false>(in, est, out);
    } else if (in.kind == GCR_FUNDAMENTAL) {
      utils::DefaultFundamentalMatrixEstimator est;
      rc = dispatch<utils::DefaultFundamentalMatrixEstimator, false>(in, est, out);
    } else {
      utils::DefaultEssentialMatrixEstimator est(in.K1, in.K2);
      rc = dispatch<utils::DefaultEssentialMatrixEstimator, false>(in, est, out);
    }
  } catch (const std::exception& e) {
    fprintf(stderr, "run failed: %s\n", e.what());
    rc = 3;
  }
  fclose(out);
  return rc;
}
