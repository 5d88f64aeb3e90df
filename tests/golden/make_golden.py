"""Regenerate the golden fixtures in this folder from the reference tree.

The reference's own integration tests (tests/testLoadGraph.cpp,
tests/testGnc.cpp) read tests/data/robot_a.g2o and tests/data/robot_b.g2o.
This script copies the numbers of those two fixture files, token for token,
into robot_a.npz / robot_b.npz so that the tests here (which run where the
reference tree is absent) build the same graphs. Run it where the reference
tree is mounted:

    python tests/golden/make_golden.py /path/to/reference
"""
import os
import sys

import numpy as np


def convert(src: str, dst: str) -> None:
    vkeys, vvals, ekeys, evals = [], [], [], []
    with open(src) as f:
        for line in f:
            tok = line.split()
            if not tok:
                continue
            if tok[0] == "VERTEX_SE3:QUAT":
                vkeys.append(int(tok[1]))
                vvals.append([float(x) for x in tok[2:9]])
            elif tok[0] == "EDGE_SE3:QUAT":
                ekeys.append([int(tok[1]), int(tok[2])])
                evals.append([float(x) for x in tok[3:31]])
    np.savez(dst, vertex_keys=np.array(vkeys, dtype=np.uint64), vertex_vals=np.array(vvals),
             edge_keys=np.array(ekeys, dtype=np.uint64).reshape(-1, 2), edge_vals=np.array(evals))


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path to the Kimera-RPGO source tree>")
    ref = sys.argv[1]
    here = os.path.dirname(os.path.abspath(__file__))
    for name in ("robot_a", "robot_b"):
        convert(os.path.join(ref, "tests", "data", name + ".g2o"), os.path.join(here, name + ".npz"))


if __name__ == "__main__":
    main()
