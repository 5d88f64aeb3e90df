"""C++ facade (include/rpgo_gb300.hpp): the reference's RobustSolverParams /
RobustSolver class API over the C ABI, compiled with g++ against
librpgo_gb300.so (tests/native/test_facade.cpp).

CPU: every parameter setter produces the flat parameters the C ABI's own
setters produce, and the facade's argument checks throw rpgo::Error with the
C ABI status. GPU: a PCM + GNC-TLS update of a graph read from a g2o file
through the facade equals the same update through the Python bindings.
"""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "kimera-rpgo_gb300", "rpgo_gb300")


@pytest.fixture(scope="module")
def facade_bin(tmp_path_factory):
    from rpgo_gb300 import build

    build()
    out = str(tmp_path_factory.mktemp("facade") / "test_facade")
    subprocess.run(["g++", "-O2", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "native", "test_facade.cpp"), "-L", LIBDIR, "-lrpgo_gb300",
                    f"-Wl,-rpath,{LIBDIR}", "-o", out], check=True)
    return out


def test_facade_params_and_argument_checks(facade_bin):
    r = subprocess.run([facade_bin, "params"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "params: 0 failures" in r.stdout


@pytest.mark.gpu
def test_facade_update_equals_python_bindings(facade_bin, tmp_path):
    from rpgo_gb300 import capi, synth
    from rpgo_gb300.graph import isotropic_variance, write_g2o
    from rpgo_gb300.params import QUIET, RobustSolverParams

    s = synth.walk3d(400, 90, 30, seed=61)
    g = s.graph
    path = str(tmp_path / "walk.g2o")
    write_g2o(path, 3, g.value_keys, g.value_poses, g.kind, g.key1, g.key2, g.measured, g.sqrt_info)
    r = subprocess.run([facade_bin, "solve", path, "3"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = {ln.split()[0]: ln.split()[1:] for ln in r.stdout.splitlines() if ln.strip()}
    # the same file and prior through the Python bindings
    py = capi.read_g2o(path, 3)
    py.add_prior(py.value_keys[0], py.value_poses[0], isotropic_variance(6, 1e-4))
    p = RobustSolverParams().setPcm3DParams(10.0, 5.0, QUIET).setGncInlierCostThresholdsAtProbability(0.9)
    ref = capi.RobustSolver(p)
    assert ref.update(py) == 0
    c = ref.counts()
    assert [int(x) for x in lines["counts"]] == [c.num_factors, c.num_lc, c.num_lc_inliers]
    w = np.array([float(x) for x in lines["weights"]])
    assert np.array_equal(np.round(w), np.round(ref.gnc_weights()))
    est = np.array([float(x) for x in lines["estimate"][1:]]).reshape(-1, 12)
    _, pe = ref.estimate()
    assert est.shape == pe.shape
    assert np.max(np.abs(est - pe) / np.maximum(1.0, np.abs(pe))) <= 1e-9
    removed = ref.removeLastLoopClosure()
    assert lines["removed"][0] == "1" and (int(lines["removed"][1]), int(lines["removed"][2])) == removed
    assert [int(x) for x in lines["after"]] == [ref.counts().num_factors, ref.counts().num_lc]
