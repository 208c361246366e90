// Oracle (test infrastructure only): homography estimator restated from
// src/pygcransac/include/estimators/homography_estimator.h:58-382 and
// src/pygcransac/include/estimators/solver_homography_four_point.h:109-286.
#pragma once

#include "oracle_common.hpp"
#include "oracle_linalg.hpp"

namespace oracle {

struct HomographyEstimator {
  static constexpr size_t sample_size() { return 4; }
  static constexpr bool space_partitioning = true;  // SpacePartitioningRANSAC applies
  static constexpr size_t max_solutions() { return 1; }  // maximumMinimalSolutions
  size_t sample_size_rt() const { return 4; }
  static constexpr size_t non_minimal_sample_size() { return 4; }
  size_t inlier_limit() const { return 7 * sample_size(); }

  // squaredResidual (homography_estimator.h:181-199)
  double squared_residual(const double* p, const Model& h) const {
    const double x1 = p[0], y1 = p[1], x2 = p[2], y2 = p[3];
    const double t1 = h[0] * x1 + h[1] * y1 + h[2];
    const double t2 = h[3] * x1 + h[4] * y1 + h[5];
    const double t3 = h[6] * x1 + h[7] * y1 + h[8];
    const double d1 = x2 - (t1 / t3);
    const double d2 = y2 - (t2 / t3);
    return d1 * d1 + d2 * d2;
  }

  // HomographyFourPointSolver::estimateMinimalModel (:109-190) on rows
  // idx(i); weight of row i is weights[idx(i)].
  static bool minimal_solve(const double* const rows[4], const double* w4, Model& out) {
    double a[8][9];
    for (int i = 0; i < 4; ++i) {
      const double* p = rows[i];
      const double x1 = p[0], y1 = p[1], x2 = p[2], y2 = p[3];
      const double w = w4 ? w4[i] : 1.0;
      const double mwx1 = -w * x1, mwy1 = -w * y1, wx2 = w * x2, wy2 = w * y2;
      double* r0 = a[2 * i];
      double* r1 = a[2 * i + 1];
      r0[0] = mwx1; r0[1] = mwy1; r0[2] = -w; r0[3] = 0; r0[4] = 0; r0[5] = 0;
      r0[6] = wx2 * x1; r0[7] = wx2 * y1; r0[8] = -wx2;
      r1[0] = 0; r1[1] = 0; r1[2] = 0; r1[3] = mwx1; r1[4] = mwy1; r1[5] = -w;
      r1[6] = wy2 * x1; r1[7] = wy2 * y1; r1[8] = -wy2;
    }
    double h[8];
    gauss_elimination<8>(a, h);
    for (int i = 0; i < 8; ++i)
      if (std::isnan(h[i])) return false;
    out = {h[0], h[1], h[2], h[3], h[4], h[5], h[6], h[7], 1.0};
    return true;
  }

  bool estimate_minimal(const Mat& pts, const size_t* s, std::vector<Model>& models) const {
    const double* rows[4] = {pts.row(s[0]), pts.row(s[1]), pts.row(s[2]), pts.row(s[3])};
    Model h;
    if (!minimal_solve(rows, nullptr, h)) return false;
    models.push_back(h);
    return true;
  }

  // estimateModelNonminimal (:136-173): Hartley normalisation (:213-310), then
  // HomographyFourPointSolver::estimateModel on the packed normalised rows with
  // sample == nullptr, so packed row i is weighted by weights[i] (the weight of
  // point index i, not of the i-th sample point), then denormalisation.
  bool estimate_nonminimal(const Mat& pts, const size_t* s, size_t n, std::vector<Model>& models,
                           const double* weights) const {
    if (n < non_minimal_sample_size()) return false;
    double ms[2] = {0, 0}, md[2] = {0, 0};
    for (size_t i = 0; i < n; ++i) {
      const double* p = pts.row(s[i]);
      ms[0] += p[0]; ms[1] += p[1]; md[0] += p[2]; md[1] += p[3];
    }
    ms[0] /= n; ms[1] /= n; md[0] /= n; md[1] /= n;
    double ads = 0, add = 0;
    for (size_t i = 0; i < n; ++i) {
      const double* p = pts.row(s[i]);
      const double dx1 = ms[0] - p[0], dy1 = ms[1] - p[1], dx2 = md[0] - p[2], dy2 = md[1] - p[3];
      ads += std::sqrt(dx1 * dx1 + dy1 * dy1);
      add += std::sqrt(dx2 * dx2 + dy2 * dy2);
    }
    ads /= n; add /= n;
    const double rs = M_SQRT2 / ads, rd = M_SQRT2 / add;
    std::vector<double> np(n * 4);
    for (size_t i = 0; i < n; ++i) {
      const double* p = pts.row(s[i]);
      np[i * 4 + 0] = (p[0] - ms[0]) * rs;
      np[i * 4 + 1] = (p[1] - ms[1]) * rs;
      np[i * 4 + 2] = (p[2] - md[0]) * rd;
      np[i * 4 + 3] = (p[3] - md[1]) * rd;
    }
    const double Ts[9] = {rs, 0, -rs * ms[0], 0, rs, -rs * ms[1], 0, 0, 1};
    const double Td[9] = {rd, 0, -rd * md[0], 0, rd, -rd * md[1], 0, 0, 1};
    Model hn;
    if (n == 4) {
      const double* rows[4] = {&np[0], &np[4], &np[8], &np[12]};
      double w4[4];
      if (weights) for (int i = 0; i < 4; ++i) w4[i] = weights[i];
      if (!minimal_solve(rows, weights ? w4 : nullptr, hn)) return false;
    } else {
      const int m = (int)(2 * n);
      std::vector<double> A((size_t)m * 8), b(m);
      for (size_t i = 0; i < n; ++i) {
        const double x1 = np[i * 4], y1 = np[i * 4 + 1], x2 = np[i * 4 + 2], y2 = np[i * 4 + 3];
        const double w = weights ? weights[i] : 1.0;
        const double mwx1 = -w * x1, mwy1 = -w * y1, wx2 = w * x2, wy2 = w * y2;
        double* r0 = &A[(2 * i) * 8];
        double* r1 = &A[(2 * i + 1) * 8];
        r0[0] = mwx1; r0[1] = mwy1; r0[2] = -w; r0[3] = 0; r0[4] = 0; r0[5] = 0; r0[6] = wx2 * x1; r0[7] = wx2 * y1;
        b[2 * i] = -wx2;
        r1[0] = 0; r1[1] = 0; r1[2] = 0; r1[3] = mwx1; r1[4] = mwy1; r1[5] = -w; r1[6] = wy2 * x1; r1[7] = wy2 * y1;
        b[2 * i + 1] = -wy2;
      }
      double h[8];
      lstsq_colpiv_qr(A, b, m, 8, h);  // never fails, like the reference's solver
      hn = {h[0], h[1], h[2], h[3], h[4], h[5], h[6], h[7], 1.0};
    }
    double Tdi[9];
    inverse3(Td, Tdi);
    double t[9];
    matmul3(Tdi, hn.data(), t);
    Model out;
    matmul3(t, Ts, out.data());
    models.push_back(out);
    return true;
  }

  // isValidModel (:326-342)
  bool is_valid_model(Model& m, const Mat&, const std::vector<size_t>&, const size_t*, double, bool&) const {
    return std::abs(det3(m)) >= 1e-2;
  }

  // isValidSample (:346-381): all four points on the same side of the lines
  // through two of them, in both images.
  bool is_valid_sample(const Mat& pts, const size_t* s) const {
    const double *a = pts.row(s[0]), *b = pts.row(s[1]), *c = pts.row(s[2]), *d = pts.row(s[3]);
    auto cross = [](double r[3], const double* u, const double* v) {
      r[0] = u[1] - v[1];
      r[1] = v[0] - u[0];
      r[2] = u[0] * v[1] - u[1] * v[0];
    };
    double p[3], q[3];
    cross(p, a, b);
    cross(q, a + 2, b + 2);
    if ((p[0] * c[0] + p[1] * c[1] + p[2]) * (q[0] * c[2] + q[1] * c[3] + q[2]) < 0) return false;
    if ((p[0] * d[0] + p[1] * d[1] + p[2]) * (q[0] * d[2] + q[1] * d[3] + q[2]) < 0) return false;
    cross(p, c, d);
    cross(q, c + 2, d + 2);
    if ((p[0] * a[0] + p[1] * a[1] + p[2]) * (q[0] * a[2] + q[1] * a[3] + q[2]) < 0) return false;
    if ((p[0] * b[0] + p[1] * b[1] + p[2]) * (q[0] * b[2] + q[1] * b[3] + q[2]) < 0) return false;
    return true;
  }
};

}  // namespace oracle

namespace oracle {

// Affine-correspondence homography estimator (test infrastructure only),
// restated from src/pygcransac/include/estimators/homography_affine_correspondence_estimator.h:58-403
// (RobustHomographyAffineCorrespondenceEstimator) with the minimal solver of
// solver_homography_two_affine.h:88-237. Rows hold eight values: the point
// pair (x1, y1, x2, y2) and the 2x2 local affine map (a11, a12, a21, a22);
// residuals, the non-minimal fit (four-point solver on the point columns) and
// the model check are the point estimator's.
struct HomographyAffineEstimator : HomographyEstimator {
  static constexpr size_t sample_size() { return 2; }
  static constexpr bool space_partitioning = false;
  size_t sample_size_rt() const { return 2; }
  size_t inlier_limit() const { return 7 * sample_size(); }

  // The 8 x 9 system of the minimal case: the two point rows of both
  // correspondences and the four affine rows of the first (the reference
  // stops after the second one's point rows). Its null vector with h33 = 1 is
  // the model the reference's SVD returns after dividing by h33; here it is
  // solved by Gaussian elimination with partial pivoting on the first eight
  // columns.
  static bool minimal_affine(const double* a, const double* b, Model& out) {
    double A[8][9];
    auto point_rows = [](double (*r)[9], const double* p) {
      const double x1 = p[0], y1 = p[1], x2 = p[2], y2 = p[3];
      const double r0[9] = {-x1, -y1, -1.0, 0.0, 0.0, 0.0, x2 * x1, x2 * y1, x2};
      const double r1[9] = {0.0, 0.0, 0.0, -x1, -y1, -1.0, y2 * x1, y2 * y1, y2};
      for (int k = 0; k < 9; ++k) {
        r[0][k] = r0[k];
        r[1][k] = r1[k];
      }
    };
    point_rows(A, a);
    {
      const double x1 = a[0], y1 = a[1], x2 = a[2], y2 = a[3];
      const double a11 = a[4], a12 = a[5], a21 = a[6], a22 = a[7];
      const double r2[9] = {-1.0, 0.0, 0.0, 0.0, 0.0, 0.0, x2 + a11 * x1, a11 * y1, a11};
      const double r3[9] = {0.0, -1.0, 0.0, 0.0, 0.0, 0.0, a12 * x1, x2 + a12 * y1, a12};
      const double r4[9] = {0.0, 0.0, 0.0, -1.0, 0.0, 0.0, y2 + a21 * x1, a21 * y1, a21};
      const double r5[9] = {0.0, 0.0, 0.0, 0.0, -1.0, 0.0, a22 * x1, y2 + a22 * y1, a22};
      for (int k = 0; k < 9; ++k) {
        A[2][k] = r2[k];
        A[3][k] = r3[k];
        A[4][k] = r4[k];
        A[5][k] = r5[k];
      }
    }
    point_rows(A + 6, b);
    // A[:, 0:8] h = -A[:, 8]
    for (int i = 0; i < 8; ++i) A[i][8] = -A[i][8];
    for (int col = 0; col < 8; ++col) {
      int piv = col;
      for (int r = col + 1; r < 8; ++r)
        if (std::abs(A[r][col]) > std::abs(A[piv][col])) piv = r;
      if (!(std::abs(A[piv][col]) > 0.0)) return false;
      if (piv != col)
        for (int k = 0; k < 9; ++k) std::swap(A[piv][k], A[col][k]);
      for (int r = col + 1; r < 8; ++r) {
        const double f = A[r][col] / A[col][col];
        for (int k = col; k < 9; ++k) A[r][k] -= f * A[col][k];
      }
    }
    double h[8];
    for (int i = 7; i >= 0; --i) {
      double s = A[i][8];
      for (int k = i + 1; k < 8; ++k) s -= A[i][k] * h[k];
      h[i] = s / A[i][i];
    }
    for (int i = 0; i < 8; ++i)
      if (!std::isfinite(h[i])) return false;
    out = {h[0], h[1], h[2], h[3], h[4], h[5], h[6], h[7], 1.0};
    return true;
  }

  bool estimate_minimal(const Mat& pts, const size_t* s, std::vector<Model>& models) const {
    Model h;
    if (!minimal_affine(pts.row(s[0]), pts.row(s[1]), h)) return false;
    models.push_back(h);
    return true;
  }

  // isValidSample (:346-400): the oriented test of the point estimator on the
  // two points and two points built from the first correspondence's affine
  // map, c = (1, 0, A (1, 0)^T) and d = (1, 0, A (0, 1)^T).
  bool is_valid_sample(const Mat& pts, const size_t* s) const {
    const double *a = pts.row(s[0]), *b = pts.row(s[1]);
    const double c[4] = {1.0, 0.0, a[4], a[6]};
    const double d[4] = {1.0, 0.0, a[5], a[7]};
    auto cross = [](double r[3], const double* u, const double* v) {
      r[0] = u[1] - v[1];
      r[1] = v[0] - u[0];
      r[2] = u[0] * v[1] - u[1] * v[0];
    };
    double p[3], q[3];
    cross(p, a, b);
    cross(q, a + 2, b + 2);
    if ((p[0] * c[0] + p[1] * c[1] + p[2]) * (q[0] * c[2] + q[1] * c[3] + q[2]) < 0) return false;
    if ((p[0] * d[0] + p[1] * d[1] + p[2]) * (q[0] * d[2] + q[1] * d[3] + q[2]) < 0) return false;
    cross(p, c, d);
    cross(q, c + 2, d + 2);
    if ((p[0] * a[0] + p[1] * a[1] + p[2]) * (q[0] * a[2] + q[1] * a[3] + q[2]) < 0) return false;
    if ((p[0] * b[0] + p[1] * b[1] + p[2]) * (q[0] * b[2] + q[1] * b[3] + q[2]) < 0) return false;
    return true;
  }
};

// Real roots, ascending, of c[0] + c[1] x + ... + c[deg] x^deg (deg <= 4):
// the quadratic derivative's roots in closed form, then each higher
// derivative's roots and the polynomial's own isolated between the next
// derivative's roots and the Cauchy bound and bisected to the last
// representable midpoint; exactly-zero leading coefficients lower the degree.
inline int poly_quadratic_roots(const double* c, double* roots) {
  const double disc = c[1] * c[1] - 4.0 * c[2] * c[0];
  if (disc < 0.0) return 0;
  const double q = -0.5 * (c[1] + std::copysign(std::sqrt(disc), c[1]));
  double r0 = q / c[2], r1 = q != 0.0 ? c[0] / q : r0;
  if (r1 < r0) std::swap(r0, r1);
  roots[0] = r0;
  roots[1] = r1;
  return 2;
}

inline int poly_bracketed_roots(const double* c, int deg, const double* cp, int ncp, double* roots) {
  double bound = 0.0;
  for (int i = 0; i < deg; ++i) bound = std::max(bound, std::abs(c[i] / c[deg]));
  bound += 1.0;
  auto f = [&](double x) {
    double v = c[deg];
    for (int i = deg - 1; i >= 0; --i) v = v * x + c[i];
    return v;
  };
  std::vector<double> edges{-bound};
  for (int i = 0; i < ncp; ++i)
    if (cp[i] > -bound && cp[i] < bound) edges.push_back(cp[i]);
  edges.push_back(bound);
  int nr = 0;
  for (size_t k = 0; k + 1 < edges.size(); ++k) {
    double lo = edges[k], hi = edges[k + 1];
    double flo = f(lo);
    const double fhi = f(hi);
    if (flo == 0.0) {
      if (nr == 0 || roots[nr - 1] != lo) roots[nr++] = lo;
      continue;
    }
    if ((flo < 0.0) == (fhi < 0.0)) continue;
    for (int it = 0; it < 200; ++it) {
      const double mid = 0.5 * (lo + hi);
      if (mid <= lo || mid >= hi) break;
      const double fm = f(mid);
      if (fm == 0.0) {
        lo = hi = mid;
        break;
      }
      if ((fm < 0.0) == (flo < 0.0)) {
        lo = mid;
        flo = fm;
      } else {
        hi = mid;
      }
    }
    roots[nr++] = 0.5 * (lo + hi);
  }
  return nr;
}

inline int poly_real_roots(const double* c_in, int deg, double* roots) {
  while (deg > 0 && c_in[deg] == 0.0) --deg;
  if (deg <= 0) return 0;
  if (deg == 1) {
    roots[0] = -c_in[0] / c_in[1];
    return std::isfinite(roots[0]) ? 1 : 0;
  }
  double lv[5][5];
  for (int i = 0; i <= deg; ++i) lv[deg][i] = c_in[i];
  for (int j = deg - 1; j >= 2; --j)
    for (int i = 0; i <= j; ++i) lv[j][i] = (i + 1) * lv[j + 1][i + 1];
  double cur[4], nxt[4];
  int n = poly_quadratic_roots(lv[2], cur);
  for (int j = 3; j <= deg; ++j) {
    n = poly_bracketed_roots(lv[j], j, cur, n, nxt);
    for (int i = 0; i < n; ++i) cur[i] = nxt[i];
  }
  for (int i = 0; i < n; ++i) roots[i] = cur[i];
  return n;
}

// findHomographySIFT_ (gcransac_python.cpp:4813-5069): the point estimator
// (RobustHomographyEstimator) on rows (x1, y1, x2, y2, q1, q2, o1, o2) with
// the minimal solver HomographyTwoSIFTSolver (solver_homography_two_sift.h:
// 113-480), which declares one solution (maximumSolutions, :83-86, the
// count SPRT uses) and returns every conic intersection.
struct HomographySiftEstimator : HomographyEstimator {
  static constexpr size_t sample_size() { return 2; }
  static constexpr bool space_partitioning = false;
  size_t sample_size_rt() const { return 2; }
  size_t inlier_limit() const { return 7 * sample_size(); }

  // Two point rows and one orientation row per correspondence (the
  // homography's Jacobian J at x1 maps the direction o1 onto a multiple of
  // o2): a 6 x 9 system, null space of dimension three. The scale ratio of
  // each correspondence is the quadratic q2 w(h)^2 - q1 D(h) = 0, with
  // w = h7 x1 + h8 y1 + h9 and D = (h1 h5 - h2 h4) + x2 (h4 h8 - h5 h7) +
  // y2 (h2 h7 - h1 h8) (the reference's coefficient expressions, :226-355).
  // The reference takes the null space from an SVD and intersects the two
  // conics with an elimination template and an eigenproblem (:356-478),
  // building a model from the real part of every eigenvalue. Here: the null
  // space by Gaussian elimination with full pivoting over h1..h8 (h9 free:
  // its basis vector has h9 = 1, the others h9 = 0), the intersections from
  // the resultant quartic in the second null-space coordinate (real roots by
  // bisection), the first coordinate from the conics' linear combination;
  // real intersections only, ascending in that root, each with h9 = 1.
  static int minimal_sift(const double* const rows[2], Model* out) {
    double A[6][9];
    double u1[2], v1[2], u2[2], v2[2], q1[2], q2[2];
    for (int c = 0; c < 2; ++c) {
      const double* p = rows[c];
      u1[c] = p[0]; v1[c] = p[1]; u2[c] = p[2]; v2[c] = p[3];
      q1[c] = p[4]; q2[c] = p[5];
      const double s1 = std::sin(p[6]), c1 = std::cos(p[6]);
      const double s2 = std::sin(p[7]), c2 = std::cos(p[7]);
      const double r0[9] = {0.0, 0.0, 0.0, u1[c], v1[c], 1.0, -u1[c] * v2[c], -v1[c] * v2[c], -v2[c]};
      const double r1[9] = {u1[c], v1[c], 1.0, 0.0, 0.0, 0.0, -u1[c] * u2[c], -v1[c] * u2[c], -u2[c]};
      const double r2[9] = {-c1 * s2, -s1 * s2, 0.0, c1 * c2, s1 * c2, 0.0,
                            u2[c] * c1 * s2 - v2[c] * c1 * c2, u2[c] * s1 * s2 - v2[c] * s1 * c2, 0.0};
      for (int k = 0; k < 9; ++k) {
        A[3 * c][k] = r0[k];
        A[3 * c + 1][k] = r1[k];
        A[3 * c + 2][k] = r2[k];
      }
    }
    int col_of[6];
    bool used[8] = {false, false, false, false, false, false, false, false};
    for (int k = 0; k < 6; ++k) {
      int pr = -1, pc = -1;
      double best = 0.0;
      for (int r = k; r < 6; ++r)
        for (int c = 0; c < 8; ++c)
          if (!used[c] && std::abs(A[r][c]) > best) {
            best = std::abs(A[r][c]);
            pr = r;
            pc = c;
          }
      if (!(best > 0.0)) return 0;
      if (pr != k)
        for (int j = 0; j < 9; ++j) std::swap(A[pr][j], A[k][j]);
      used[pc] = true;
      col_of[k] = pc;
      const double inv = 1.0 / A[k][pc];
      for (int j = 0; j < 9; ++j) A[k][j] *= inv;
      for (int r = 0; r < 6; ++r) {
        if (r == k) continue;
        const double fct = A[r][pc];
        if (fct != 0.0)
          for (int j = 0; j < 9; ++j) A[r][j] -= fct * A[k][j];
      }
    }
    int fr[3];
    int nf = 0;
    for (int c = 0; c < 8; ++c)
      if (!used[c]) fr[nf++] = c;
    fr[2] = 8;
    double N[3][9];
    for (int b = 0; b < 3; ++b) {
      for (int j = 0; j < 9; ++j) N[b][j] = 0.0;
      N[b][fr[b]] = 1.0;
      for (int k = 0; k < 6; ++k) N[b][col_of[k]] = -A[k][fr[b]];
    }
    double K[2][6];
    for (int c = 0; c < 2; ++c) {
      auto form = [&](const double* x, const double* y) {
        const double wx = x[6] * u1[c] + x[7] * v1[c] + x[8];
        const double wy = y[6] * u1[c] + y[7] * v1[c] + y[8];
        const double dxy = 0.5 * ((x[0] * y[4] + y[0] * x[4] - x[1] * y[3] - y[1] * x[3]) +
                                  u2[c] * (x[3] * y[7] + y[3] * x[7] - x[4] * y[6] - y[4] * x[6]) +
                                  v2[c] * (x[1] * y[6] + y[1] * x[6] - x[0] * y[7] - y[0] * x[7]));
        return q2[c] * wx * wy - q1[c] * dxy;
      };
      K[c][0] = form(N[0], N[0]);
      K[c][1] = 2.0 * form(N[0], N[1]);
      K[c][2] = form(N[1], N[1]);
      K[c][3] = 2.0 * form(N[0], N[2]);
      K[c][4] = 2.0 * form(N[1], N[2]);
      K[c][5] = form(N[2], N[2]);
    }
    const double a1 = K[0][0], a2 = K[1][0];
    const double p2 = a1 * K[1][2] - a2 * K[0][2], p1 = a1 * K[1][4] - a2 * K[0][4], p0 = a1 * K[1][5] - a2 * K[0][5];
    const double l1 = a1 * K[1][1] - a2 * K[0][1], l0 = a1 * K[1][3] - a2 * K[0][3];
    const double k3 = K[0][1] * K[1][2] - K[1][1] * K[0][2];
    const double k2 = K[0][1] * K[1][4] + K[0][3] * K[1][2] - K[1][1] * K[0][4] - K[1][3] * K[0][2];
    const double k1 = K[0][1] * K[1][5] + K[0][3] * K[1][4] - K[1][1] * K[0][5] - K[1][3] * K[0][4];
    const double k0 = K[0][3] * K[1][5] - K[1][3] * K[0][5];
    const double r[5] = {p0 * p0 - l0 * k0, 2.0 * p1 * p0 - (l1 * k0 + l0 * k1),
                         p1 * p1 + 2.0 * p2 * p0 - (l1 * k1 + l0 * k2), 2.0 * p2 * p1 - (l1 * k2 + l0 * k3),
                         p2 * p2 - l1 * k3};
    double roots[4];
    const int nr = poly_real_roots(r, 4, roots);
    int nm = 0;
    for (int i = 0; i < nr; ++i) {
      const double b = roots[i];
      const double L = l1 * b + l0, P = (p2 * b + p1) * b + p0;
      const double a = -P / L;
      Model h;
      bool fin = true;
      for (int j = 0; j < 9; ++j) {
        h[j] = a * N[0][j] + b * N[1][j] + N[2][j];
        fin = fin && std::isfinite(h[j]);
      }
      if (fin) out[nm++] = h;
    }
    return nm;
  }

  bool estimate_minimal(const Mat& pts, const size_t* s, std::vector<Model>& models) const {
    const double* rows[2] = {pts.row(s[0]), pts.row(s[1])};
    Model m[4];
    const int nm = minimal_sift(rows, m);
    for (int i = 0; i < nm; ++i) models.push_back(m[i]);
    return nm > 0;
  }

  // isValidSample (homography_estimator.h:350-351): not tested below four
  bool is_valid_sample(const Mat&, const size_t*) const { return true; }
};

}  // namespace oracle
