"""The C ABI library builds, loads and exports every entry point the public
header declares (no compute calls: CPU only)."""
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "rpgo_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(?:void|int|int32_t|int64_t|double|rpgo_\w+\s*\*)\s*\*?\s*(rpgo_\w+)\s*\(", text)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from rpgo_gb300 import build
    from rpgo_gb300 import capi

    build()
    return capi.load()


def test_header_declares_entry_points():
    names = declared_functions()
    assert "rpgo_create" in names and "rpgo_update" in names and "rpgo_pairwise_adjacency_dev" in names
    assert len(names) >= 25


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from rpgo_gb300.capi import SIGNATURES

    assert sorted(SIGNATURES) == declared_functions()


def test_params_defaults_match_reference(lib):
    # SolverParams.h:35-42, 60-68, 82-94 (host-only call)
    from rpgo_gb300.capi import Params
    import ctypes

    p = Params()
    lib.rpgo_params_default(ctypes.byref(p))
    assert (p.odom_threshold, p.lc_threshold) == (10.0, 5.0)
    assert (p.odom_trans_threshold, p.odom_rot_threshold) == (0.05, 0.005)
    assert (p.dist_trans_threshold, p.dist_rot_threshold) == (0.01, 0.001)
    assert p.gnc_threshold_mode == 1 and p.gnc_inlier_threshold == 0.9 and p.gnc_max_iterations == 100
    assert (p.gnc_mu_step, p.gnc_relative_cost_tol, p.gnc_weights_tol) == (1.4, 1e-5, 1e-4)
    assert p.lm_diagonal_damping == 1 and p.use_gnc == 0 and p.outlier_removal == 2 and p.solver == 0
    lib.rpgo_params_set_pcm_simple3d(ctypes.byref(p), 0.1, 0.2, 0.3, 0.4, 1)
    assert (p.outlier_removal, p.odom_trans_threshold, p.odom_rot_threshold, p.dist_trans_threshold,
            p.dist_rot_threshold, p.verbosity) == (4, 0.1, 0.2, 0.3, 0.4, 1)


def test_python_params_mirror_matches_c_defaults(lib):
    from rpgo_gb300.capi import Params
    from rpgo_gb300.params import RobustSolverParams
    import ctypes

    p = Params()
    lib.rpgo_params_default(ctypes.byref(p))
    q = RobustSolverParams()
    for name, _ in Params._fields_:
        assert getattr(p, name) == getattr(q, name), name
