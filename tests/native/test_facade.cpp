// Test program of the C++ facade (include/rpgo_gb300.hpp), built with g++
// against librpgo_gb300.so by tests/test_facade.py.
//
//   test_facade params          parameter setters and argument checks (no GPU)
//   test_facade solve FILE DIM  read a g2o file, PCM + GNC-TLS update through
//                               the facade, print counts, weights and the
//                               estimate (GPU)
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "rpgo_gb300.hpp"

static int failures = 0;
#define EXPECT(c)                                                    \
  do {                                                               \
    if (!(c)) {                                                      \
      std::printf("FAIL %s:%d: %s\n", __FILE__, __LINE__, #c);       \
      ++failures;                                                    \
    }                                                                \
  } while (0)

static bool same(const rpgo_params& a, const rpgo_params& b) {
  bool ok = a.solver == b.solver && a.outlier_removal == b.outlier_removal && a.verbosity == b.verbosity &&
            a.odom_threshold == b.odom_threshold && a.lc_threshold == b.lc_threshold &&
            a.odom_trans_threshold == b.odom_trans_threshold && a.odom_rot_threshold == b.odom_rot_threshold &&
            a.dist_trans_threshold == b.dist_trans_threshold && a.dist_rot_threshold == b.dist_rot_threshold &&
            a.incremental == b.incremental && a.use_gnc == b.use_gnc &&
            a.gnc_threshold_mode == b.gnc_threshold_mode && a.gnc_inlier_threshold == b.gnc_inlier_threshold &&
            a.gnc_max_iterations == b.gnc_max_iterations && a.gnc_mu_step == b.gnc_mu_step &&
            a.gnc_relative_cost_tol == b.gnc_relative_cost_tol && a.gnc_weights_tol == b.gnc_weights_tol &&
            a.gnc_fix_prev_inliers == b.gnc_fix_prev_inliers && a.gnc_bias_odom == b.gnc_bias_odom &&
            a.lm_diagonal_damping == b.lm_diagonal_damping && a.num_special_symbols == b.num_special_symbols &&
            a.multirobot_align_method == b.multirobot_align_method &&
            a.multirobot_align_gnc_prob == b.multirobot_align_gnc_prob;
  for (int i = 0; ok && i < a.num_special_symbols; ++i) ok = a.special_symbols[i] == b.special_symbols[i];
  return ok;
}

static int test_params() {
  using namespace rpgo;
  rpgo_params ref;
  // defaults (SolverParams.h:82-94)
  rpgo_params_default(&ref);
  EXPECT(same(RobustSolverParams().toC(), ref));
  // setPcm3DParams
  {
    RobustSolverParams p;
    p.setPcm3DParams(8.0, 4.0, Verbosity::QUIET);
    rpgo_params_default(&ref);
    rpgo_params_set_pcm3d(&ref, 8.0, 4.0, RPGO_VERBOSITY_QUIET);
    EXPECT(same(p.toC(), ref));
    EXPECT(p.poseDim() == 3);
  }
  // setPcm2DParams + GNC at probability with all arguments
  {
    RobustSolverParams p;
    p.setPcm2DParams(1.0, 1.0);
    p.setGncInlierCostThresholdsAtProbability(0.95, 50, 1.3, 1e-6, 1e-3, true, true);
    rpgo_params_default(&ref);
    rpgo_params_set_pcm2d(&ref, 1.0, 1.0, RPGO_VERBOSITY_UPDATE);
    rpgo_params_set_gnc_probability(&ref, 0.95, 50, 1.3, 1e-6, 1e-3, 1, 1);
    EXPECT(same(p.toC(), ref));
    EXPECT(p.poseDim() == 2);
  }
  // GNC at a cost with the reference's defaults, then gncFixInliers / gncBiasOdom
  {
    RobustSolverParams p;
    p.setGncInlierCostThresholds(3.5);
    rpgo_params_default(&ref);
    rpgo_params_set_gnc_cost(&ref, 3.5, 100, 1.4, 1e-5, 1e-4, 0, 0);
    EXPECT(same(p.toC(), ref));
    p.gncFixInliers();
    p.gncBiasOdom();
    EXPECT(p.toC().gnc_fix_prev_inliers == 1 && p.toC().gnc_bias_odom == 1);
  }
  // PcmSimple, both overloads (the two-threshold one repeats the pair)
  {
    RobustSolverParams a, b;
    a.setPcmSimple3DParams(0.05, 0.01, Verbosity::QUIET);
    b.setPcmSimple3DParams(0.05, 0.01, 0.05, 0.01, Verbosity::QUIET);
    rpgo_params_default(&ref);
    rpgo_params_set_pcm_simple3d(&ref, 0.05, 0.01, 0.05, 0.01, RPGO_VERBOSITY_QUIET);
    EXPECT(same(a.toC(), ref) && same(b.toC(), ref));
    RobustSolverParams c;
    c.setPcmSimple2DParams(0.1, 0.02, 0.3, 0.04);
    rpgo_params_default(&ref);
    rpgo_params_set_pcm_simple2d(&ref, 0.1, 0.02, 0.3, 0.04, RPGO_VERBOSITY_UPDATE);
    EXPECT(same(c.toC(), ref));
    EXPECT(c.poseDim() == 2);
  }
  // setNoRejection, setIncremental, setLmDiagonalDamping, multi-robot alignment
  {
    RobustSolverParams p;
    p.setNoRejection(Verbosity::VERBOSE);
    p.dim = 2;
    p.setIncremental();
    p.setLmDiagonalDamping(false);
    p.setMultiRobotAlignMethod(MultiRobotAlignMethod::GNC);
    p.setMultiRobotGncAlignProbability(0.8);
    rpgo_params_default(&ref);
    rpgo_params_set_no_rejection(&ref, RPGO_VERBOSITY_VERBOSE);
    ref.dim = 2;
    ref.incremental = 1;
    ref.lm_diagonal_damping = 0;
    rpgo_params_set_multirobot_align(&ref, RPGO_ALIGN_GNC, 0.8);
    EXPECT(same(p.toC(), ref));
    EXPECT(p.poseDim() == 2);
  }
  // special symbols pass through; too many, a bad dimension or an iteration
  // count beyond int32 are argument errors
  {
    RobustSolverParams p;
    p.specialSymbols = {'l', 'u'};
    EXPECT(p.toC().num_special_symbols == 2 && p.toC().special_symbols[1] == 'u');
    p.specialSymbols.assign(RPGO_MAX_SPECIAL_SYMBOLS + 1, 'x');
    int status = -1;
    try {
      (void)p.toC();
    } catch (const Error& e) {
      status = e.status();
    }
    EXPECT(status == RPGO_ERR_ARG);
    RobustSolverParams q;
    q.setNoRejection();
    q.dim = 4;
    status = -1;
    try {
      (void)q.toC();
    } catch (const Error& e) {
      status = e.status();
    }
    EXPECT(status == RPGO_ERR_ARG);
    RobustSolverParams r;
    r.setGncInlierCostThresholdsAtProbability(0.9, size_t(1) << 40);
    status = -1;
    try {
      (void)r.toC();
    } catch (const Error& e) {
      status = e.status();
    }
    EXPECT(status == RPGO_ERR_ARG);
  }
  // keys, graph containers
  {
    const Key k = symbol('a', 42);
    EXPECT(symbolChr(k) == 'a' && symbolIndex(k) == 42);
    FactorGraph g(3);
    const double pose[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0.5, 0, 0};
    double cov[36] = {0};
    const double sig[6] = {0.005, 0.005, 0.005, 0.02, 0.02, 0.02};
    for (int i = 0; i < 6; ++i) cov[i * 6 + i] = sig[i] * sig[i];
    cov[3 * 6 + 4] = cov[4 * 6 + 3] = 1e-4;  // correlated translation
    g.addBetween(symbol('a', 0), symbol('a', 1), pose, cov);
    g.addPrior(symbol('a', 0), pose, cov);
    EXPECT(g.size() == 2 && g.kind[0] == RPGO_FACTOR_BETWEEN && g.kind[1] == RPGO_FACTOR_PRIOR);
    EXPECT(g.key_back[1] == symbol('a', 0));
    // R upper triangular and R^T R C = I
    const double* R = g.sqrt_information.data();
    double worst = 0.0;
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 6; ++j) {
        if (i > j) EXPECT(R[i * 6 + j] == 0.0);
        double s = 0.0;
        for (int k2 = 0; k2 < 6; ++k2) {
          double info = 0.0;
          for (int q = 0; q < 6; ++q) info += R[q * 6 + i] * R[q * 6 + k2];
          s += info * cov[k2 * 6 + j];
        }
        worst = std::fmax(worst, std::fabs(s - (i == j ? 1.0 : 0.0)));
      }
    EXPECT(worst < 1e-9);
    double bad[36] = {0};
    int status = -1;
    try {
      g.addBetween(symbol('a', 1), symbol('a', 2), pose, bad);
    } catch (const Error& e) {
      status = e.status();
    }
    EXPECT(status == RPGO_ERR_ARG && g.size() == 2);
    Values v(3);
    v.insert(symbol('a', 0), pose);
    EXPECT(v.exists(symbol('a', 0)) && !v.exists(symbol('a', 1)) && v.at(symbol('a', 0))[9] == 0.5);
    status = -1;
    try {
      (void)v.at(symbol('a', 9));
    } catch (const Error& e) {
      status = e.status();
    }
    EXPECT(status == RPGO_ERR_KEY);
    FactorGraph g2(2);
    status = -1;
    try {
      g.add(g2);
    } catch (const Error& e) {
      status = e.status();
    }
    EXPECT(status == RPGO_ERR_ARG);
  }
  // a bad enum is rejected by rpgo_create (the reference exits); a solver
  // either exists (GPU present) or construction reports the CUDA failure
  {
    RobustSolverParams p;
    p.outlierRemovalMethod = static_cast<OutlierRemovalMethod>(17);
    int status = -1;
    try {
      RobustSolver s(p);
    } catch (const Error& e) {
      status = e.status();
    }
    EXPECT(status != -1);
    RobustSolverParams q;
    status = -1;
    try {
      RobustSolver s(q);
      EXPECT(s.size() == 0 && s.getNumLC() == 0 && s.calculateEstimate().empty());
      status = 0;
    } catch (const Error& e) {
      status = e.status();
    }
    EXPECT(status == 0 || status == RPGO_ERR_CUDA);
  }
  std::printf("params: %d failures\n", failures);
  return failures ? 1 : 0;
}

static int test_solve(const char* path, int dim) {
  using namespace rpgo;
  auto gv = readG2o(path, dim);
  FactorGraph& graph = gv.first;
  // the first pose anchored by a prior at its initial value
  const Values& values = gv.second;
  const int d = dim == 3 ? 6 : 3;
  double cov[36] = {0};
  for (int i = 0; i < d; ++i) cov[i * d + i] = 1e-4;
  graph.addPrior(values.keys[0], values.poses.data(), cov);
  RobustSolverParams p;
  if (dim == 3) p.setPcm3DParams(10.0, 5.0, Verbosity::QUIET);
  else p.setPcm2DParams(3.0, 3.0, Verbosity::QUIET);
  p.setGncInlierCostThresholdsAtProbability(0.9);
  RobustSolver s(p);
  s.update(graph, values);
  std::printf("counts %zu %zu %zu\n", s.size(), s.getNumLC(), s.getNumLCInliers());
  const std::vector<double> w = s.getGncWeights();
  std::printf("weights");
  for (double x : w) std::printf(" %.17g", x);
  std::printf("\n");
  const Values est = s.calculateEstimate();
  std::printf("estimate %zu", est.size());
  for (double x : est.poses) std::printf(" %.17g", x);
  std::printf("\n");
  // edit API round trip: the last closure removed, then the estimate again
  EdgePtr e = s.removeLastLoopClosure();
  std::printf("removed %d %llu %llu\n", e ? 1 : 0, e ? (unsigned long long)e->from_key : 0ull,
              e ? (unsigned long long)e->to_key : 0ull);
  std::printf("after %zu %zu\n", s.size(), s.getNumLC());
  return 0;
}

int main(int argc, char** argv) {
  if (argc >= 2 && std::strcmp(argv[1], "params") == 0) return test_params();
  if (argc >= 4 && std::strcmp(argv[1], "solve") == 0) {
    try {
      return test_solve(argv[2], std::atoi(argv[3]));
    } catch (const rpgo::Error& e) {
      std::printf("error %d %s\n", e.status(), e.what());
      return 2;
    }
  }
  std::printf("usage: test_facade params | solve FILE DIM\n");
  return 64;
}
