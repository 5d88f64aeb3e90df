"""Native g2o reader (rpgo_g2o_read) against the Python statement of GTSAM's
load3D / load2D (rpgo_gb300.graph.parse_g2o_*), on the reference's fixture
numbers (robot_a / robot_b) and on synthetic 2D / 3D graphs written by the
Kimera-RPGO writeG2o restatement. Host-only: no GPU needed."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from rpgo_gb300 import capi, synth
from rpgo_gb300.graph import parse_g2o_2d, parse_g2o_3d, write_g2o


def _fixture_text(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    lines = []
    for k, v in zip(z["vertex_keys"], z["vertex_vals"]):
        lines.append("VERTEX_SE3:QUAT %d %s" % (int(k), " ".join(repr(float(x)) for x in v[:7])))
    for (a, b), v in zip(z["edge_keys"], z["edge_vals"]):
        lines.append("EDGE_SE3:QUAT %d %d %s" % (int(a), int(b), " ".join(repr(float(x)) for x in v[:28])))
    return "\n".join(lines) + "\n"


def _same(g, ref, tol=1e-12):
    A, B = g.arrays(), ref.arrays()
    for k in ("kind", "key1", "key2", "value_keys"):
        assert np.array_equal(A[k], B[k]), k
    for k in ("measured", "value_poses"):
        np.testing.assert_array_equal(A[k], B[k])
    for k in ("cov", "sqrt_info"):
        np.testing.assert_allclose(A[k], B[k], rtol=tol, atol=tol * np.abs(B[k]).max())


@pytest.mark.parametrize("name", ["robot_a", "robot_b"])
def test_reader_matches_load3d_on_reference_fixtures(tmp_path, name):
    text = _fixture_text(name)
    path = tmp_path / (name + ".g2o")
    path.write_text(text)
    _same(capi.read_g2o(str(path), 3), parse_g2o_3d(text))


def test_reader_round_trips_writer_3d_and_2d(tmp_path):
    for dim, s, parse in ((3, synth.walk3d(300, 40, 10, seed=9), parse_g2o_3d),
                          (2, synth.grid2d(200, 30, 5, seed=9), parse_g2o_2d)):
        a = s.graph.arrays()
        between = a["kind"] == 0
        path = tmp_path / f"w{dim}.g2o"
        write_g2o(str(path), dim, a["value_keys"], a["value_poses"], a["kind"], a["key1"], a["key2"], a["measured"],
                  a["sqrt_info"])
        text = path.read_text()
        g = capi.read_g2o(str(path), dim)
        _same(g, parse(text))
        assert g.num_factors == int(between.sum())


def test_reader_errors(tmp_path):
    with pytest.raises(capi.RpgoError):
        capi.read_g2o(str(tmp_path / "missing.g2o"), 3)
    bad = tmp_path / "bad.g2o"
    bad.write_text("EDGE_SE3:QUAT 0 1 0.5 0 0\n")
    with pytest.raises(capi.RpgoError):
        capi.read_g2o(str(bad), 3)
    other = tmp_path / "other.g2o"
    other.write_text("# comment\nFIX 0\nVERTEX_SE3:QUAT 0 0 0 0 0 0 0 1\n")
    g = capi.read_g2o(str(other), 3)
    assert g.value_keys == [0] and g.num_factors == 0
