"""GB300-native Kimera-RPGO robust back-end (PCM + GNC-TLS over LM/GN).

Python front-end of librpgo_gb300.so: the RobustSolver / RobustSolverParams
API of the reference (include/KimeraRPGO/RobustSolver.h, SolverParams.h) over
the C ABI declared in include/rpgo_gb300.h.
"""
from .params import (COST, GN, LM, NONE, PCM2D, PCM3D, PCM_SIMPLE2D, PCM_SIMPLE3D, PROBABILITY, QUIET, UPDATE,
                     VERBOSE, RobustSolverParams)
from .graph import (BETWEEN, PRIOR, Graph, diagonal_sigmas, gaussian_covariance, gaussian_information,
                    isotropic_sigma, isotropic_variance, pose2, pose3, symbol)


def build(force: bool = False) -> str:
    import importlib.util
    import os

    here = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location("_rpgo_build", os.path.join(here, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(force)


def RobustSolver(params):
    from .capi import RobustSolver as _RS

    return _RS(params)
