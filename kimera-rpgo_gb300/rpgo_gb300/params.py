"""RobustSolverParams mirror (include/KimeraRPGO/SolverParams.h:13-299).

Same fields, defaults and setters as the reference, flattened the way the C
ABI's ``rpgo_params`` lays them out.
"""
from __future__ import annotations

# enum class Solver { LM, GN }
LM, GN = 0, 1
# enum class OutlierRemovalMethod
NONE, PCM2D, PCM3D, PCM_SIMPLE2D, PCM_SIMPLE3D = 0, 1, 2, 3, 4
# enum class Verbosity { UPDATE, QUIET, VERBOSE }
UPDATE, QUIET, VERBOSE = 0, 1, 2
# GncParams::GncThresholdMode
COST, PROBABILITY = 0, 1
# linear solver of the LM / GN step (GTSAM linearSolverType; the reference keeps the default)
LINEAR_CHOLESKY, LINEAR_PCG = 0, 1
# MultiRobotAlignMethod (SolverParams.h:26-31)
ALIGN_NONE, ALIGN_L2, ALIGN_GNC = 0, 1, 2
# GNC warm start modes (rpgo_params.gnc_warm_start)
WARM_OFF, WARM_ON, WARM_RECORD, WARM_CONTINUATION = 0, 1, 2, 3


class RobustSolverParams:
    def __init__(self):
        # SolverParams.h:82-94
        self.solver = LM
        self.outlier_removal = PCM3D
        self.verbosity = UPDATE
        self.dim = 3
        # PcmParams, SolverParams.h:35-42
        self.odom_threshold = 10.0
        self.lc_threshold = 5.0
        self.odom_trans_threshold = 0.05
        self.odom_rot_threshold = 0.005
        self.dist_trans_threshold = 0.01
        self.dist_rot_threshold = 0.001
        self.incremental = 0
        # GncParams, SolverParams.h:60-68
        self.use_gnc = 0
        self.gnc_threshold_mode = PROBABILITY
        self.gnc_inlier_threshold = 0.9
        self.gnc_max_iterations = 100
        self.gnc_mu_step = 1.4
        self.gnc_relative_cost_tol = 1e-5
        self.gnc_weights_tol = 1e-4
        self.gnc_fix_prev_inliers = 0
        self.gnc_bias_odom = 0
        self.lm_diagonal_damping = 1
        self.linear_solver = LINEAR_CHOLESKY
        # GNC warm start (no counterpart in the reference): off by default
        self.gnc_warm_start = WARM_OFF
        self.gnc_warm_mu = 1e2
        # specialSymbols (SolverParams.h:284): landmark key prefixes
        self.num_special_symbols = 0
        self.special_symbols = b""
        # SolverParams.h:92-93
        self.multirobot_align_method = ALIGN_NONE
        self.multirobot_align_gnc_prob = 0.99

    # SolverParams.h:97-100
    def setNoRejection(self, verbosity=UPDATE, dim=3):
        self.outlier_removal = NONE
        self.verbosity = verbosity
        self.dim = dim
        return self

    def setIncremental(self):
        self.incremental = 1
        return self

    def setLmDiagonalDamping(self, flag: bool):
        self.lm_diagonal_damping = int(bool(flag))
        return self

    def setLinearSolver(self, kind: int):
        """LINEAR_CHOLESKY (default, GTSAM's sparse Cholesky) or LINEAR_PCG."""
        self.linear_solver = int(kind)
        return self

    def setSolver(self, solver):
        self.solver = solver
        return self

    def setPcm2DParams(self, odom, lc, verbosity=UPDATE):
        self.outlier_removal, self.dim = PCM2D, 2
        self.odom_threshold, self.lc_threshold, self.verbosity = odom, lc, verbosity
        return self

    def setPcm3DParams(self, odom, lc, verbosity=UPDATE):
        self.outlier_removal, self.dim = PCM3D, 3
        self.odom_threshold, self.lc_threshold, self.verbosity = odom, lc, verbosity
        return self

    def _simple(self, method, dim, t_odom, r_odom, t_pcm, r_pcm, verbosity):
        self.outlier_removal, self.dim = method, dim
        self.odom_trans_threshold, self.odom_rot_threshold = t_odom, r_odom
        self.dist_trans_threshold, self.dist_rot_threshold = t_pcm, r_pcm
        self.verbosity = verbosity
        return self

    def setPcmSimple2DParams(self, trans, rot, *rest):
        """(trans, rot[, verbosity]) or (trans_odom, rot_odom, trans_pcm, rot_pcm[, verbosity])."""
        if len(rest) >= 2:
            return self._simple(PCM_SIMPLE2D, 2, trans, rot, rest[0], rest[1], rest[2] if len(rest) > 2 else UPDATE)
        return self._simple(PCM_SIMPLE2D, 2, trans, rot, trans, rot, rest[0] if rest else UPDATE)

    def setPcmSimple3DParams(self, trans, rot, *rest):
        if len(rest) >= 2:
            return self._simple(PCM_SIMPLE3D, 3, trans, rot, rest[0], rest[1], rest[2] if len(rest) > 2 else UPDATE)
        return self._simple(PCM_SIMPLE3D, 3, trans, rot, trans, rot, rest[0] if rest else UPDATE)

    def _gnc(self, mode, thr, max_iterations, mu_step, rel_cost_tol, weight_tol, fix_prev_inliers, bias_odom):
        self.use_gnc = 1
        self.gnc_threshold_mode = mode
        self.gnc_inlier_threshold = thr
        self.gnc_max_iterations = max_iterations
        self.gnc_mu_step = mu_step
        self.gnc_relative_cost_tol = rel_cost_tol
        self.gnc_weights_tol = weight_tol
        self.gnc_fix_prev_inliers = int(bool(fix_prev_inliers))
        self.gnc_bias_odom = int(bool(bias_odom))
        return self

    # SolverParams.h:213-250
    def setGncInlierCostThresholdsAtProbability(self, alpha, max_iterations=100, mu_step=1.4, rel_cost_tol=1e-5,
                                                weight_tol=1e-4, fix_prev_inliers=False, bias_odom=False):
        return self._gnc(PROBABILITY, alpha, max_iterations, mu_step, rel_cost_tol, weight_tol, fix_prev_inliers,
                         bias_odom)

    def setGncInlierCostThresholds(self, cost, max_iterations=100, mu_step=1.4, rel_cost_tol=1e-5, weight_tol=1e-4,
                                   fix_prev_inliers=False, bias_odom=False):
        return self._gnc(COST, cost, max_iterations, mu_step, rel_cost_tol, weight_tol, fix_prev_inliers, bias_odom)

    def gncFixInliers(self):
        self.gnc_fix_prev_inliers = 1
        return self

    def gncBiasOdom(self):
        self.gnc_bias_odom = 1
        return self

    # SolverParams.h:264-272
    def setMultiRobotAlignMethod(self, method):
        self.multirobot_align_method = int(method)
        return self

    def setMultiRobotGncAlignProbability(self, probability):
        self.multirobot_align_gnc_prob = float(probability)
        return self

    @property
    def specialSymbols(self):
        return [chr(c) for c in self.special_symbols[:self.num_special_symbols]]

    @specialSymbols.setter
    def specialSymbols(self, symbols):
        b = "".join(symbols).encode()
        if len(b) > 16:
            raise ValueError("at most 16 special symbols")
        self.special_symbols, self.num_special_symbols = b, len(b)

    def setGncWarmStart(self, mode=WARM_ON, mu=None):
        """Warm-started GNC schedule (WARM_ON), plain schedule with closure
        features recorded (WARM_RECORD), plain mu continuation with the
        predicted first inlier set and LM from the previous estimate
        (WARM_CONTINUATION), or the plain schedule (WARM_OFF)."""
        self.gnc_warm_start = int(mode)
        if mu is not None:
            self.gnc_warm_mu = float(mu)
        return self
