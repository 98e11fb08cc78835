"""Known-answer tests of single pieces of the restatement, computed by hand
from the reference's code: process_segment's bin split (src/RTA_MC2D.cpp:
699-769), Grid_distribution sampling (src/sampling.cpp:26-44,
include/sampling.hpp:92-102), propagator_H::get on a 4 x 4 matrix
(src/collision_operator.cpp:892-903) and the *.P.eigen.bin layout of
save_P / load_P (src/collision_operator.cpp:931-1013)."""
import numpy as np
import pytest

import pyoracle
import synth

GRID = [0.0, 10.0, 20.0, 30.0]


@pytest.mark.parametrize("t0,t1,sign,bins", [
    (5.0, 25.0, -1, [-5.0, -10.0, -5.0]),      # three bins, negative particle
    (12.0, 18.0, 1, [0.0, 6.0, 0.0]),          # inside one bin
    (10.0, 20.0, 1, [0.0, 10.0, 0.0]),         # on both borders
    (25.0, 40.0, 1, [0.0, 0.0, 5.0]),          # past maxtime: the rest is dropped
    (0.0, 0.0, 1, [0.0, 0.0, 0.0]),            # empty segment
])
def test_segment_bin_split(built, t0, t1, sign, bins):
    assert np.array_equal(pyoracle.kat_segment(GRID, t0, t1, sign), bins)


@pytest.mark.parametrize("u,k", [
    (0.1, 1), (0.125, 1), (0.3, 2), (0.5, 2), (0.5000001, 4), (0.99, 4),
    (0.0, 0),  # lower_bound at u = 0 lands on a zero-weight first mode (a reference quirk)
])
def test_cdf_sample(built, u, k):
    assert pyoracle.kat_cdf_sample([0.0, 1.0, 3.0, 0.0, 4.0], u) == k


def test_cdf_sample_rejects_negative_weights(built):
    assert pyoracle.kat_cdf_sample([1.0, -1.0], 0.5) == -1


P4 = np.array([[0.5, 0.1, 0.0, 0.2],
               [-0.25, 0.6, 0.3, -0.2],
               [0.25, -0.3, 0.7, 0.2],
               [0.0, 0.0, 0.0, 0.4]])


@pytest.mark.parametrize("col,u,mode,sign", [
    (0, 0.4, 3, 1),     # |cumm| of column 0 = 0.5, 0.75, 1.0, 1.0 with signs +, -, +, +
    (0, 0.6, 4, -1),
    (0, 0.9, 5, 1),
    (0, 1.0, 5, 1),     # the first |cumm| >= 1
    (1, 0.05, 3, 1),    # column 1: 0.1, 0.7, 1.0 (-), 1.0 -> 0.1, 0.7, 1.0, 1.0
    (1, 0.95, 5, -1),
    (3, 0.3, 4, -1),    # column 3: 0.2, 0.4 (-), 0.6, 1.0
])
def test_propagator_get(built, col, u, mode, sign):
    assert pyoracle.kat_propagator(P4, col, u) == (mode, sign)


def test_propagator_file_round_trip(tmp_path):
    """int64 row count, then the matrix column by column in FP64."""
    P = np.arange(9.0).reshape(3, 3) / 7.0
    synth.write_propagator(str(tmp_path / "p.P.eigen.bin"), P)
    raw = (tmp_path / "p.P.eigen.bin").read_bytes()
    assert len(raw) == 8 + 9 * 8 and int.from_bytes(raw[:8], "little") == 3
    assert np.array_equal(np.frombuffer(raw[8:], dtype="<f8"), P.ravel(order="F"))
    assert np.array_equal(synth.read_propagator(str(tmp_path / "p.P.eigen.bin")), P)
