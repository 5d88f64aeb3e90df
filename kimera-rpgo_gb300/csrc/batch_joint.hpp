// Joint batch: the GNC-TLS / LM solves of many independent graphs advanced
// in lock-step rounds, every stage one launch over all graphs.
//
// Each round, every graph that is still iterating takes exactly one damped
// solve: one linearisation launch pair, one block-Hessian launch and one
// cooperative direct-solve launch serve all of them (a merged plan of the
// graphs' own plans, each graph with its own damping lambda), then one
// retraction and one error launch. Between rounds every graph's host state
// machine takes the decisions of GTSAM's LevenbergMarquardtOptimizer /
// GaussNewtonOptimizer and GncOptimizer (as GpuNls::optimize and gnc_tls
// restate them) from its own results: accept or reject the step, change
// lambda, finish the LM run, update the TLS weights and mu, reset to the
// initial values. A graph that has finished drops out of the rounds (its
// items are skipped by every launch).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "solver.hpp"
#include "stores.hpp"

struct rpgo_solver;

namespace rpgo {

// One graph's optimisation problem, as RobustSolver::optimize would set it up.
struct JointProblem {
  std::vector<FactorRec> graph;       // factors to optimise (graph, then temporary)
  const FactorStore* store = nullptr; // their measurements
  ValueStore* values = nullptr;       // initial values; the result is written back here
  size_t n_known = 0;                 // known inliers (GNC weights fixed at 1)
  bool gnc = false;                   // GNC-TLS over LM/GN (else one LM/GN run)
  GncConfig gnc_cfg;
  LmParams lm;
  std::vector<double> init_weights;   // GNC's first weights (empty: all 1)
  // results
  std::vector<double> weights;        // final GNC weights (all 1 without GNC)
  NlsStats stats;
  bool failed = false;                // the GN step's system was indefinite
};

// Solves every problem (same dim, same LM / GNC parameters apart from the
// known-inlier counts and first weights) in lock-step rounds on stream st,
// the direct solve on coop_ctas CTAs (0: every co-resident CTA). Returns the
// number of rounds.
int solve_joint(int dim, std::vector<JointProblem*>& probs, cudaStream_t st, int coop_ctas = 0);

// Rounds are replayed from one captured CUDA graph (set_joint_graphs(false):
// launched stage by stage); returns the previous setting.
bool set_joint_graphs(bool on);
// rounds replayed from a captured graph so far (process-wide)
int64_t joint_graph_rounds();

// The solver side (capi.cpp). joint_prepare: the problem that
// RobustSolver::optimize would solve after the last update (made with
// optimize_graph = 0): kJointSolve (filled in *jp), kJointNone (no
// optimisation asked for), kJointOwn (a case that needs the solver's own
// path: temporary values, a warm start, the fixed-previous-inliers subset,
// the PCG solver, an empty graph). joint_commit: optimize's bookkeeping after
// solve_joint. joint_optimize_own: optimize itself.
enum { kJointSolve = 0, kJointNone = 1, kJointOwn = 2 };
int joint_prepare(rpgo_solver* s, JointProblem* jp);
int joint_commit(rpgo_solver* s, const JointProblem& jp, double solve_ms);
int joint_optimize_own(rpgo_solver* s, double* solve_ms);

}  // namespace rpgo
