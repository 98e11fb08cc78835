"""The restatement's calculate_gradientT against the reference's own code.

tests/golden/ref_pins_dmm.json ("gradientT") holds the gradients that the
reference's calculate_gradientT (src/geometry_2d.cpp:524-575, its Eigen
complete orthogonal decomposition included) returned, compiled by
oracle/build_ref.py from its line range, on two seeded geometries: a grid
with a staircase pore and random Teq (4 to 8 neighbours per cell, corners
included) and a ribbon between reservoirs (collinear neighbours, the
minimum-norm case).  The restatement (oracle/rta_oracle.cpp, cod_solve)
solves the same least-squares problems by Householder QR with column
pivoting; the gradients must agree to rounding."""
import json
import os

import numpy as np
import pytest

import build_ref
import pyoracle
import synth

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "ref_pins_dmm.json")))["gradientT"]


@pytest.mark.parametrize("case", range(len(GOLD)))
def test_gradientT_matches_the_reference(case):
    g, _ = build_ref.gradient_geometries()[case]
    assert np.array_equal(np.asarray(g["Teq"]), np.asarray(GOLD[case]["Teq"]))
    m = synth.mode_table(8, 3, 3, 300.0, config=100)
    got = pyoracle.gradient_T(m, g)
    ref = np.asarray(GOLD[case]["gradients"], dtype=float)
    assert got.shape == ref.shape
    scale = np.abs(ref).max()
    assert scale > 0
    assert np.abs(got - ref).max() <= 1e-12 * scale, np.abs(got - ref).max() / scale
