/*
 * rpgo_gb300 — C ABI of the GB300-native Kimera-RPGO robust back-end.
 *
 * Plain C, plain pointers and sizes. Every compute call runs on CUDA device 0
 * of the calling process (one GPU, sm_103a); there is no CPU fallback: if the
 * device or the kernels are unavailable, calls fail with RPGO_ERR_CUDA.
 *
 * Pose layout (row-major, doubles):
 *   3D (Pose3): 12 values  R00 R01 R02 R10 R11 R12 R20 R21 R22 tx ty tz
 *   2D (Pose2):  4 values  cos(theta) sin(theta) x y
 * Tangent order follows GTSAM: Pose3 [omega; v], Pose2 [v_x, v_y, omega].
 * Covariance / square-root information blocks are dim x dim row-major with
 * dim = 6 (3D) or 3 (2D). sqrt_information is the upper-triangular R with
 * R^T R = information; the solver whitens residuals with it, PCM reads the
 * covariance (as the reference reads noiseModel()->covariance()).
 * Keys are 64-bit gtsam::Symbol values: (char << 56) | index.
 */
#ifndef RPGO_GB300_H
#define RPGO_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
enum {
  RPGO_OK = 0,
  RPGO_ERR_ARG = 1,        /* bad argument (null pointer, bad enum, size) */
  RPGO_ERR_CUDA = 2,       /* CUDA runtime / kernel failure */
  RPGO_ERR_KEY = 3,        /* value key already present, or missing key */
  RPGO_ERR_SOLVER = 4,     /* linear system not positive definite (GN) */
  RPGO_ERR_UNSUPPORTED = 5, /* feature outside the implemented path */
  RPGO_ERR_SIZE = 6         /* size beyond a fixed maximum of the entry point */
};

/* --------------------------------------------------------------- enumerants
 * Mirror of include/KimeraRPGO/SolverParams.h:13-27 (Solver,
 * OutlierRemovalMethod, Verbosity). */
enum { RPGO_SOLVER_LM = 0, RPGO_SOLVER_GN = 1 };
enum {
  RPGO_OUTLIER_NONE = 0,
  RPGO_OUTLIER_PCM2D = 1,
  RPGO_OUTLIER_PCM3D = 2,
  RPGO_OUTLIER_PCM_SIMPLE2D = 3,
  RPGO_OUTLIER_PCM_SIMPLE3D = 4
};
enum { RPGO_VERBOSITY_UPDATE = 0, RPGO_VERBOSITY_QUIET = 1, RPGO_VERBOSITY_VERBOSE = 2 };
enum { RPGO_GNC_COST = 0, RPGO_GNC_PROBABILITY = 1 };
enum { RPGO_FACTOR_BETWEEN = 0, RPGO_FACTOR_PRIOR = 1 };
/* Linear solver of the LM / GN step (GTSAM: NonlinearOptimizerParams::
 * linearSolverType, left at its default sparse Cholesky by the reference). */
enum { RPGO_LINEAR_CHOLESKY = 0, RPGO_LINEAR_PCG = 1 };

#define RPGO_MAX_SPECIAL_SYMBOLS 16

/* Flat mirror of RobustSolverParams (include/KimeraRPGO/SolverParams.h:80-299)
 * with PcmParams (33-56) and GncParams (58-78) inlined. */
typedef struct rpgo_params {
  int32_t solver;            /* RPGO_SOLVER_* */
  int32_t outlier_removal;   /* RPGO_OUTLIER_* */
  int32_t verbosity;         /* RPGO_VERBOSITY_* */
  int32_t dim;               /* 2 or 3; required when outlier_removal == NONE */
  /* PcmParams */
  double odom_threshold, lc_threshold;
  double odom_trans_threshold, odom_rot_threshold;
  double dist_trans_threshold, dist_rot_threshold;
  int32_t incremental;
  /* GncParams */
  int32_t use_gnc;
  int32_t gnc_threshold_mode; /* RPGO_GNC_* */
  double gnc_inlier_threshold;
  int32_t gnc_max_iterations;
  double gnc_mu_step, gnc_relative_cost_tol, gnc_weights_tol;
  int32_t gnc_fix_prev_inliers, gnc_bias_odom;
  /* additional */
  int32_t lm_diagonal_damping;
  int32_t linear_solver;      /* RPGO_LINEAR_*: direct sparse Cholesky (default) or PCG */
  /* GNC warm start (no counterpart in the reference; off by default, which
   * keeps GncOptimizer's plain mu continuation): RPGO_WARM_* */
  int32_t gnc_warm_start;
  double gnc_warm_mu;         /* mu of the first TLS weight update of the warm schedule */
  /* RobustSolverParams::specialSymbols (SolverParams.h:284): key prefixes of
   * landmarks, whose observations get landmark PCM (Pcm.h:180-220, 775-844) */
  int32_t num_special_symbols;
  char special_symbols[RPGO_MAX_SPECIAL_SYMBOLS];
  /* multirobot_align_method / multirobot_align_gnc_prob
   * (SolverParams.h:92-93, 264-272): RPGO_ALIGN_* */
  int32_t multirobot_align_method;
  double multirobot_align_gnc_prob;
} rpgo_params;

/* MultiRobotAlignMethod (SolverParams.h:26-31): after PCM, the initial
 * values of every robot but the one with the smallest prefix are moved by
 * the robust average (GNC-TLS at multirobot_align_gnc_prob, or L2) of the
 * frame offsets its inter-robot closures with that robot imply
 * (Pcm.h:1011-1131). */
enum { RPGO_ALIGN_NONE = 0, RPGO_ALIGN_L2 = 1, RPGO_ALIGN_GNC = 2 };

/* gnc_warm_start values.
 * OFF: the plain GNC-TLS schedule (GncOptimizer, src/RobustSolver.cpp:133-171).
 * ON: predicted inlier probabilities (the installed closure model, or the
 *   probabilities given by rpgo_set_warm_start_probs) pick the first inlier
 *   set, the mu continuation starts at gnc_warm_mu, each LM run starts from the
 *   previous estimate, and the result is accepted only when its weights are
 *   binary and agree with the TLS rule at the final estimate; otherwise the
 *   plain schedule runs from the start (counted in rpgo_timing.warm_fallbacks).
 * RECORD: the plain schedule, recording the closure features (training data).
 * CONTINUATION: plain GNC's mu continuation and TLS weight rule, with two
 *   changes: the first solve uses the predicted inlier set (probability >= 0.5;
 *   all ones without a model or probabilities) instead of all ones, and every
 *   later LM run starts from the previous estimate instead of the initial
 *   values. No certificate: the result is plain GNC's only as far as the two
 *   changes leave its decisions unchanged. */
enum { RPGO_WARM_OFF = 0, RPGO_WARM_ON = 1, RPGO_WARM_RECORD = 2, RPGO_WARM_CONTINUATION = 3 };

/* A batch of factors (structure of arrays). For priors key_back is ignored. */
typedef struct rpgo_factor_batch {
  int64_t count;
  const int32_t* kind;             /* RPGO_FACTOR_* */
  const uint64_t* key_front;
  const uint64_t* key_back;
  const double* measured;          /* count x pose stride (12 or 4) */
  const double* covariance;        /* count x dim x dim */
  const double* sqrt_information;  /* count x dim x dim */
} rpgo_factor_batch;

typedef struct rpgo_value_batch {
  int64_t count;
  const uint64_t* key;
  const double* pose;              /* count x pose stride */
} rpgo_value_batch;

typedef struct rpgo_counts {
  int64_t num_factors;        /* size of the graph to optimise (getFactorsUnsafe) */
  int64_t num_values;         /* calculateEstimate().size() */
  int64_t num_lc;             /* getNumLC */
  int64_t num_lc_inliers;     /* getNumLCInliers */
  int64_t num_odom;           /* odometry factors kept by PCM */
  int64_t num_special;        /* non-between factors (priors) */
  int64_t num_gnc_weights;    /* getGncWeights().size() */
  int64_t last_do_optimize;   /* value removeOutliers / addAndCheckIfOptimize returned in the last update */
} rpgo_counts;

typedef struct rpgo_timing {
  double pcm_ms;              /* classification, trajectory, odometry + pairwise checks, clique */
  double solve_ms;            /* GNC / LM / GN */
  int64_t pair_checks;        /* pairwise consistency tests run */
  int64_t lm_iterations;      /* accepted LM/GN iterations summed over the GNC schedule */
  int64_t linear_solves;      /* damped systems solved */
  int64_t gnc_iterations;     /* outer GNC iterations */
  int64_t cg_iterations;      /* preconditioned CG iterations */
  int64_t kernel_launches;    /* kernels of this library launched by the last update */
  /* device time of the dominant kernels (CUDA events on the library's stream) */
  double pcg_kernel_ms;       /* whole-GPU PCG launches (sum) */
  int64_t pcg_kernel_launches;
  double pcg_kernel_bytes;    /* algorithmic bytes those launches move (sum) */
  double chol_kernel_ms;      /* direct (Cholesky) solve launches (sum) */
  int64_t chol_kernel_launches;
  double chol_kernel_flops;   /* algorithmic FP64 flops of their factorisations (sum) */
  double chol_kernel_bytes;   /* algorithmic device-memory bytes of those solves (sum) */
  int64_t chol_levels;        /* elimination-tree levels of the sparse part (last plan) */
  int64_t chol_tail;          /* variables in the dense trailing block (last plan) */
  double pair_kernel_ms;      /* pairwise consistency launches (sum) */
  int64_t pair_kernel_launches;
  int64_t warm_runs;          /* warm-started GNC schedules run (RPGO_WARM_ON) */
  int64_t warm_fallbacks;     /* of those, not certified: the plain schedule was rerun */
} rpgo_timing;

typedef struct rpgo_solver rpgo_solver; /* opaque */

/* ------------------------------------------------------------------ params
 * RobustSolverParams::RobustSolverParams (SolverParams.h:82-94) defaults. */
void rpgo_params_default(rpgo_params* p);
/* SolverParams.h:97-100 */
void rpgo_params_set_no_rejection(rpgo_params* p, int32_t verbosity);
/* SolverParams.h:119-126 / 134-141 */
void rpgo_params_set_pcm2d(rpgo_params* p, double odom_threshold, double lc_threshold, int32_t verbosity);
void rpgo_params_set_pcm3d(rpgo_params* p, double odom_threshold, double lc_threshold, int32_t verbosity);
/* SolverParams.h:148-209 (four-threshold overloads; the two-threshold
 * overloads pass the same pair twice) */
void rpgo_params_set_pcm_simple2d(rpgo_params* p, double trans_odom, double rot_odom, double trans_pcm,
                                  double rot_pcm, int32_t verbosity);
void rpgo_params_set_pcm_simple3d(rpgo_params* p, double trans_odom, double rot_odom, double trans_pcm,
                                  double rot_pcm, int32_t verbosity);
/* SolverParams.h:264-272 */
void rpgo_params_set_multirobot_align(rpgo_params* p, int32_t method, double gnc_probability);
/* SolverParams.h:213-250 */
void rpgo_params_set_gnc_probability(rpgo_params* p, double alpha, int32_t max_iterations, double mu_step,
                                     double rel_cost_tol, double weight_tol, int32_t fix_prev_inliers,
                                     int32_t bias_odom);
void rpgo_params_set_gnc_cost(rpgo_params* p, double cost, int32_t max_iterations, double mu_step,
                              double rel_cost_tol, double weight_tol, int32_t fix_prev_inliers,
                              int32_t bias_odom);

/* ------------------------------------------------------------------ solver
 * RobustSolver::RobustSolver (src/RobustSolver.cpp:29-103). Returns NULL on a
 * bad parameter set (the reference calls exit(EXIT_FAILURE)) or when no CUDA
 * device is usable. */
rpgo_solver* rpgo_create(const rpgo_params* p);
void rpgo_destroy(rpgo_solver* s);

/* RobustSolver::update (src/RobustSolver.cpp:337-369): PCM outlier rejection
 * (Pcm::removeOutliers, include/KimeraRPGO/outlier/Pcm.h:148-281) then, if
 * something changed and optimize_graph != 0, the GNC / LM / GN solve
 * (RobustSolver::optimize, src/RobustSolver.cpp:115-306). */
int rpgo_update(rpgo_solver* s, const rpgo_factor_batch* factors, const rpgo_value_batch* values,
                int32_t optimize_graph);
/* rpgo_update for callers that keep the graph in GPU memory: the bulk arrays
 * (factors->measured, ->covariance, ->sqrt_information and values->pose) are
 * DEVICE pointers of the calling process's CUDA device 0; the metadata
 * (kind, key_front, key_back, key) stays on the host. Same semantics as
 * rpgo_update; the measurements are copied device to device. */
int rpgo_update_dev(rpgo_solver* s, const rpgo_factor_batch* factors, const rpgo_value_batch* values,
                    int32_t optimize_graph);
/* RobustSolver::forceUpdate (src/RobustSolver.cpp:308-335) */
int rpgo_force_update(rpgo_solver* s, const rpgo_factor_batch* factors, const rpgo_value_batch* values);

/* README.md:114-118 loadGraph / addGraph, written as update() wrappers:
 * loadGraph(nfg, values, prior) = update(nfg + prior, values);
 * addGraph(nfg, values, between) = update(nfg + between, values). The extra
 * factor is a batch of one appended after `factors`. */
int rpgo_load_graph(rpgo_solver* s, const rpgo_factor_batch* factors, const rpgo_value_batch* values,
                    const rpgo_factor_batch* prior);
int rpgo_add_graph(rpgo_solver* s, const rpgo_factor_batch* factors, const rpgo_value_batch* values,
                   const rpgo_factor_batch* between);

/* getters (RobustSolver.h:40-47, 110-117; GenericSolver.h:38-41) */
int rpgo_get_counts(const rpgo_solver* s, rpgo_counts* out);
/* calculateEstimate(): keys ascending; arrays sized by counts.num_values */
int rpgo_get_estimate(const rpgo_solver* s, uint64_t* keys, double* poses, int64_t capacity);
/* getGncWeights(): sized by counts.num_gnc_weights */
int rpgo_get_gnc_weights(const rpgo_solver* s, double* weights, int64_t capacity);
/* getFactorsUnsafe(): the graph handed to the optimiser, in its order */
int rpgo_get_factors(const rpgo_solver* s, int32_t* kind, uint64_t* key_front, uint64_t* key_back,
                     double* measured, int64_t capacity);
/* Test hook: the bit-packed symmetric adjacency of loop-closure group `group`
 * (groups in the order buildGraphToOptimize visits them, Pcm.h:977-1005),
 * n x ceil(n/32) uint32 words, bit j of row i set when closures i and j are
 * pairwise consistent. Returns the group size in *n. */
int rpgo_get_adjacency(const rpgo_solver* s, int32_t group, uint32_t* words, int64_t capacity, int64_t* n);
int rpgo_get_timing(const rpgo_solver* s, rpgo_timing* out);

/* ---- temporary factors and values (GenericSolver.h:46-65,
 * RobustSolver.cpp:115-121, 169, 208, 264, 295; GenericSolver.cpp:37-45).
 * They are optimised together with the graph by every later optimisation
 * (appended after it; under GNC they are not known inliers), never pass
 * outlier rejection, and are not part of calculateEstimate(); the solve
 * updates their values. Host pointers. */
/* updateTempFactorsValues: append (RPGO_ERR_KEY when a value key exists in
 * the graph's or the temporary values) */
int rpgo_update_temp_factors_values(rpgo_solver* s, const rpgo_factor_batch* factors,
                                    const rpgo_value_batch* values);
/* replaceTempFactorsValues: replace both sets */
int rpgo_replace_temp_factors_values(rpgo_solver* s, const rpgo_factor_batch* factors,
                                     const rpgo_value_batch* values);
/* clearTempFactorsValues */
int rpgo_clear_temp_factors_values(rpgo_solver* s);
/* getTempFactorsUnsafe().size() and getTempValues().size() */
int rpgo_get_temp_sizes(const rpgo_solver* s, int64_t* num_factors, int64_t* num_values);
/* getTempValues(): keys ascending, poses as rpgo_get_estimate */
int rpgo_get_temp_values(const rpgo_solver* s, uint64_t* keys, double* poses, int64_t capacity);
/* getGncTempWeights(): one weight per temporary factor of the last
 * optimisation (all 1 when it ran without GNC); *n = their number */
int rpgo_get_gnc_temp_weights(const rpgo_solver* s, double* weights, int64_t capacity, int64_t* n);
/* ---- edit API (src/RobustSolver.cpp:371-446, Pcm.h:299-408). Each edit
 * then re-optimises like the reference (removePriorFactorsWithPrefix only when
 * optimize_graph != 0); values are not changed by the edit itself. */
/* removeLastLoopClosure(prefix_1, prefix_2) when by_id != 0, else
 * removeLastLoopClosure(): *removed = 0 where the reference returns NULL
 * (unknown group, no closure left); the removed closure's keys otherwise.
 * Without outlier rejection the last factor of the graph is removed
 * (GenericSolver::removeLastFactor). */
int rpgo_remove_last_loop_closure(rpgo_solver* s, int32_t by_id, char prefix_1, char prefix_2, uint64_t* key_front,
                                  uint64_t* key_back, int32_t* removed);
/* ignorePrefix / revivePrefix: closures of groups involving the prefix leave
 * / rejoin the graph (no-op with a warning without outlier rejection). */
int rpgo_ignore_prefix(rpgo_solver* s, char prefix);
int rpgo_revive_prefix(rpgo_solver* s, char prefix);
/* getIgnoredPrefixes(): *n prefixes in the order they were ignored; out may
 * be NULL to query *n. */
int rpgo_get_ignored_prefixes(const rpgo_solver* s, char* out, int32_t capacity, int32_t* n);
/* removePriorFactorsWithPrefix(prefix, optimize_graph) */
int rpgo_remove_prior_factors_with_prefix(rpgo_solver* s, char prefix, int32_t optimize_graph);

/* GNC warm start (no counterpart in the reference): inlier probabilities for
 * the factors of the next GNC solve, in the order of the graph it optimises
 * (rpgo_get_factors after the update; odometry and priors first, their
 * entries are ignored). Used by that solve when gnc_warm_start is
 * RPGO_WARM_ON and n equals the graph size (else the installed closure model
 * predicts them), then cleared. */
int rpgo_set_warm_start_probs(rpgo_solver* s, const double* probs, int64_t n);

/* Closure network of the warm start (no counterpart in the reference): 16
 * features -> 64 ReLU -> 64 ReLU -> 1, sigmoid; one flat FP32 parameter
 * array of RPGO_MLP_PARAMS floats:
 *   [0,16) feature mean, [16,32) 1/std, [32,1056) W1 (64x16, row = unit),
 *   [1056,1120) b1, [1120,5216) W2 (64x64), [5216,5280) b2,
 *   [5280,5344) W3, [5344] b3.
 * The kernels multiply with the weights rounded to BF16 (nearest even) and
 * accumulate in FP32.
 * Features of closure (i -> j, Z, R = sqrt information) at the initial
 * values X: e = Logmap(Z^-1 Xi^-1 Xj), r = R e, c = |r|^2, gap = |i - j|
 * (0 between robots):
 *   0-5 log1p|r_k| (2D: 0-2, rest 0), 6 log1p(c), 7 rotation angle of e,
 *   8 log1p|translation of e|, 9 log1p(gap), 10 log1p(c / max(1, gap)),
 *   11 PCM degree / (group size - 1), 12 log1p(PCM degree),
 *   13 neighbours in the PCM consistent set / (set size - 1),
 *   14 log1p|translation of Z|, 15 rotation angle of Z. */
#define RPGO_MLP_FEATURES 16
#define RPGO_MLP_PARAMS 5345
/* Installs a closure network (host array of RPGO_MLP_PARAMS floats; NULL
 * removes it). With gnc_warm_start = RPGO_WARM_ON its predictions are the
 * warm start's inlier probabilities. */
int rpgo_set_warm_start_model(rpgo_solver* s, const float* params);
/* Features of the closures of the last GNC solve run with gnc_warm_start ON
 * or RECORD: *n rows of RPGO_MLP_FEATURES floats in the order of the
 * graph's closures (factors after the odometry and priors). out may be NULL
 * to query *n. */
int rpgo_get_closure_features(const rpgo_solver* s, float* out, int64_t capacity, int64_t* n);
/* prob[k] = network(features[k]) for k < n (device pointers). */
int rpgo_mlp_forward_dev(const float* params, int64_t n, const float* features, float* prob, void* stream);
/* One training step on n labelled closures (device pointers; labels 0/1):
 * grad (RPGO_MLP_PARAMS floats) receives the gradient of the mean binary
 * cross-entropy (normalisation slots zero), *loss (host, optional) the loss;
 * with lr > 0 one Adam step (beta 0.9 / 0.999, eps 1e-8, bias-corrected with
 * step >= 1) updates params[32:] and the moments adam_m, adam_v. */
int rpgo_mlp_train_step_dev(float* params, float* adam_m, float* adam_v, int64_t step, float lr, int64_t n,
                            const float* features, const float* labels, float* grad, double* loss, void* stream);
/* RobustSolver::saveData (src/RobustSolver.cpp:448-465): result.g2o and
 * gnc_weights.csv in `folder`. */
int rpgo_save_data(const rpgo_solver* s, const char* folder);

/* ---------------------------------------------------------------------- g2o
 * Native reader of the g2o format of Kimera-RPGO's fixtures and results
 * (GTSAM readG2o / load3D / load2D semantics, as examples/RpgoReadG2o.cpp:
 * 129-143 use them): VERTEX_SE3:QUAT / EDGE_SE3:QUAT (dim 3; quaternions
 * normalised, the information reordered from g2o's [t; R] to [R; t]) or
 * VERTEX_SE2 / EDGE_SE2 (dim 2); noise models as
 * noiseModel::Gaussian::Information(I, smart = true). rpgo_g2o_view points
 * batches into the reader's arrays (valid until rpgo_g2o_free); they can be
 * passed to rpgo_update as they are. The writer is rpgo_save_data
 * (src/Logger.cpp:64-164 writeG2o). */
typedef struct rpgo_g2o rpgo_g2o; /* opaque */
rpgo_g2o* rpgo_g2o_read(const char* path, int32_t dim, int32_t* status);
int rpgo_g2o_view(const rpgo_g2o* g, rpgo_factor_batch* factors, rpgo_value_batch* values);
void rpgo_g2o_free(rpgo_g2o* g);

/* ------------------------------------------------------------------ batches
 * Many independent graphs (Monte-Carlo trials, submaps) solved in one call.
 * No counterpart in the reference, whose RobustSolver solves one graph per
 * instance: graph g gives exactly what RobustSolver(p).update(factors[g],
 * values[g]) gives (the same PCM, GNC and LM steps). The graphs run
 * concurrently on `workers` host threads, each solver on its own CUDA stream
 * with its cooperative direct solve limited to `coop_ctas` CTAs so that
 * several solves share the GPU (workers <= 0, coop_ctas <= 0: defaults).
 * Outputs (caller-allocated, graphs in order):
 *   poses: sum_g values[g].count x stride doubles; graph g's estimate in
 *     ascending key order at offset sum_{h<g} values[h].count x stride;
 *   gnc_weights (optional): sum_g factors[g].count doubles; graph g's
 *     getGncWeights() at offset sum_{h<g} factors[h].count, its length in
 *     num_weights[g];
 *   status: per graph, the rpgo_update status;
 *   timing (optional): per graph, the rpgo_timing of its update.
 * Returns RPGO_OK when every graph ran (check status per graph). */
typedef struct rpgo_batch_out {
  double* poses;
  double* gnc_weights;
  int64_t* num_weights;
  int32_t* status;
  rpgo_timing* timing;
} rpgo_batch_out;
int rpgo_solve_batch(const rpgo_params* p, int32_t n, const rpgo_factor_batch* factors,
                     const rpgo_value_batch* values, int32_t workers, int32_t coop_ctas, rpgo_batch_out* out);
/* The same batch with the solves in lock-step (no counterpart in the
 * reference): every graph's PCM runs on its own solver as in
 * rpgo_solve_batch; then the GNC-TLS / LM (or GN) solves of the graphs advance
 * together, one damped solve per graph per round, and every stage of a round
 * (linearisation, block Hessian, the direct solve, retraction, errors, TLS
 * weights) is one launch over all graphs, each graph with its own damping
 * and decisions. Graphs are grouped by size; `streams` groups (0: 4) run
 * concurrently on their own streams, each group of `group` graphs (0: the
 * graphs shared evenly over the streams). Graphs whose solve needs the
 * solver's own path (temporary values, a warm start, the PCG solver) are
 * solved by it. Outputs as rpgo_solve_batch; timing.solve_ms is the wall
 * time of the graph's group. */
int rpgo_solve_batch_joint(const rpgo_params* p, int32_t n, const rpgo_factor_batch* factors,
                           const rpgo_value_batch* values, int32_t group, int32_t streams, rpgo_batch_out* out);
/* The joint batch replays each round from one captured CUDA graph (on = 1,
 * the default) or launches its stages one by one (on = 0); process-wide.
 * Returns the previous setting. */
int32_t rpgo_set_joint_graphs(int32_t on);
/* Rounds of joint batches replayed from a captured graph so far (process-wide). */
int64_t rpgo_joint_graph_rounds(void);

/* ------------------------------------------------------------ stage kernels
 * Device-resident entry points of the hot path, one per reference function
 * family, for callers that keep the graph in GPU memory. All pointers are
 * device pointers; `stream` is a cudaStream_t (0 = legacy default stream).
 * Trajectory entries are addressed by slot (int32); slot layout:
 *   pose: stride 12 (3D) or 4 (2D) doubles; cov: dim*dim doubles;
 *   node: int32 (PcmSimple); rot_info: uint8.
 */

/* Odometry chain composition, Pcm::updateOdom (Pcm.h:516-557) applied in
 * order for `count` odometry factors: traj[dst[k]] = traj[src[k]] o delta[k].
 * mode 0: PoseWithCovariance, 1: PoseWithNode. */
int rpgo_trajectory_scan_dev(int32_t dim, int32_t mode, int64_t count, const int32_t* src, const int32_t* dst,
                             const double* delta_pose, const double* delta_cov, double* traj_pose, double* traj_cov,
                             int32_t* traj_node, uint8_t* traj_rot_info, void* stream);

/* Odometry consistency, Pcm::isOdomConsistent + checkOdomConsistent
 * (Pcm.h:564-629) for `count` closures i -> j with measurement z:
 * ok[k] = 1 when consistent. mode 0: Mahalanobis against th0; mode 1:
 * average translation/rotation norms against th0/th1. */
int rpgo_odometry_check_dev(int32_t dim, int32_t mode, int64_t count, const int32_t* slot_i, const int32_t* slot_j,
                            const double* z_pose, const double* z_cov, const double* traj_pose,
                            const double* traj_cov, const int32_t* traj_node, const uint8_t* traj_rot_info,
                            double th0, double th1, uint8_t* ok, void* stream);

/* Pairwise consistency, Pcm::incrementAdjMatrix + areLoopsConsistent
 * (Pcm.h:670-768) for rows [row_begin, n) of an n-closure group: for every
 * i < j with j >= row_begin, closure i = (a_i -> b_i, z_i) is tested against
 * closure j = (c_j -> d_j, z_j) (c/d swapped when `flip` of i and j differ),
 * and bits (i, j), (j, i) of `adj` (n rows of `words` uint32) are set or
 * cleared. Rows and columns below row_begin in the upper-left block are left
 * as they are. */
int rpgo_pairwise_adjacency_dev(int32_t dim, int32_t mode, int32_t n, int32_t row_begin, const int32_t* slot_a,
                                const int32_t* slot_b, const uint8_t* flip, const double* z_pose,
                                const double* z_cov, const double* traj_pose, const double* traj_cov,
                                const int32_t* traj_node, const uint8_t* traj_rot_info, double th0, double th1,
                                uint32_t* adj, int32_t words, void* stream);

/* Greedy max clique, findMaxCliqueHeu / findMaxCliqueHeuIncremental
 * (src/utils/GraphUtils.cpp:19-44, findCliqueHeu.cpp:32-209) on the
 * bit-packed adjacency (device): candidates first..n-1, running best seeded
 * with `seed` (-1 for the full search). Writes the size to *size_out (host)
 * and the first *size_out entries of the winning work buffer to clique_out
 * (host, capacity n); *size_out equals `seed` when nothing improved. */
int rpgo_max_clique_heu_dev(int32_t n, const uint32_t* adj, int32_t words, int32_t first, int32_t seed,
                            int32_t* clique_out, int32_t* size_out, void* stream);

/* Allocation-free variant of rpgo_max_clique_heu_dev. It has no counterpart
 * in the reference: it exists for callers that must not allocate GPU memory
 * (no cudaMalloc / cudaFree, no library allocator) on their call path. Same
 * arguments, results and error codes, with a fixed maximum size:
 * n <= RPGO_CLIQUE_NOALLOC_MAX_N and words <= RPGO_CLIQUE_NOALLOC_MAX_WORDS,
 * else RPGO_ERR_SIZE with a message on stderr. Its device work arrays live in
 * one file-scope __device__ array of RPGO_CLIQUE_NOALLOC_SCRATCH_BYTES, held
 * by every device that loads the library until the process exits. The first
 * call on a device (with that device current) looks up the array's address
 * with cudaGetSymbolAddress. Every call synchronises `stream` once per
 * candidate window (it reads the window's scores back), so it cannot be
 * captured into a CUDA graph. The address is kept for the process: do not
 * call this entry point again after a cudaDeviceReset of that device. Every
 * call shares the one array: calls that overlap on the GPU (from several host
 * threads, or on several streams) race and give wrong results. */
#define RPGO_CLIQUE_NOALLOC_MAX_N 4096
#define RPGO_CLIQUE_NOALLOC_MAX_WORDS 128
#define RPGO_CLIQUE_NOALLOC_SCRATCH_BYTES 2245632
int rpgo_max_clique_heu_dev_noalloc(int32_t n, const uint32_t* adj, int32_t words, int32_t first, int32_t seed,
                                    int32_t* clique_out, int32_t* size_out, void* stream);

/* ------------------------------------------------------------- host copies
 * The same stages on host arrays (copies in, copies out), for tests and for
 * callers without device memory management. */
int rpgo_pairwise_adjacency(int32_t dim, int32_t mode, int32_t n, const int32_t* slot_a, const int32_t* slot_b,
                            const uint8_t* flip, const double* z_pose, const double* z_cov, int32_t num_slots,
                            const double* traj_pose, const double* traj_cov, const int32_t* traj_node,
                            const uint8_t* traj_rot_info, double th0, double th1, uint32_t* adj);
int rpgo_max_clique_heu(int32_t n, const uint32_t* adj, int32_t first, int32_t seed, int32_t* clique_out,
                        int32_t* size_out);

/* Fill-in guard of the direct solve (no counterpart in the reference, whose
 * GTSAM solve always factors): when the symbolic plan of a graph predicts
 * more than `flops` factorisation flops (default 1e10, about 30 ms per damped
 * system), the first damped system of each solve is solved by both the
 * direct sparse Cholesky and the whole-GPU PCG path, the direct result is
 * kept, and the later systems use the faster path (prefer 0), or always the
 * direct one (1), or always PCG (2). Both reach a relative residual of 1e-12.
 * Process-wide; returns the previous threshold. */
double rpgo_set_direct_solve_guard(double flops, int32_t prefer);

/* Library / device information (name of the loaded device, SM count). */
int rpgo_device_info(char* name, int32_t name_capacity, int32_t* sm_count);
/* Number of CUDA kernels this library has launched in this process. */
int64_t rpgo_kernel_launch_count(void);
/* Number of device (cudaMallocAsync) and pinned host (cudaMallocHost)
 * allocations this library's buffers have made in this process; no
 * counterpart in the reference (it lets a caller check that a call path
 * allocates nothing). */
int64_t rpgo_buffer_alloc_count(void);

#ifdef __cplusplus
}
#endif
#endif /* RPGO_GB300_H */
