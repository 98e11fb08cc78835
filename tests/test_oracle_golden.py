"""Pin the CPU restatement against golden vectors produced by the reference's
own vendored headers (oracle/build_ref.py -> tests/golden/ref_kat.json):
pcg64 streams, the libstdc++ uniform mappings, the Eigen time grid and -log."""
import json
import os

import numpy as np
import pytest

import pyoracle

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "ref_kat.json")))


@pytest.mark.parametrize("key", ["pcg64_s0_t0", "pcg64_s42_t54", "pcg64_s20261203_t7", "pcg64_big"])
def test_pcg64_raw_matches_reference(key):
    g = GOLD[key]
    raw, _, _ = pyoracle.pcg64(g["seed"], g["stream"], len(g["raw"]))
    assert [int(x) for x in raw] == [int(x) for x in g["raw"]]


def test_canonical_matches_uniform_real_distribution():
    g = GOLD["canonical"]
    _, can, _ = pyoracle.pcg64(g["seed"], g["stream"], len(g["u"]))
    assert np.array_equal(can, np.array(g["u"]))  # bit-exact doubles


def test_uniform_int_matches_libstdcxx():
    g = GOLD["uniform_int"]
    # the golden run drew all cases from one stream in sequence; replay it
    # with a mixed-range generator built from the same raw stream
    import ctypes as C
    lib = pyoracle.load()
    his = [c[0] for c in g["cases"]]
    # draw sequentially: each uniform_int consumes >= 1 raw output; emulate by
    # re-seeding and drawing with the oracle's own routine one value at a time
    raw, _, _ = pyoracle.pcg64(g["seed"], g["stream"], 4 * len(his))
    # Lemire without rejection for these ranges (rejection probability < 2^-30)
    vals = []
    k = 0
    for hi in his:
        rng = hi + 1
        x = int(raw[k])
        k += 1
        prod = x * rng
        lo = prod & ((1 << 64) - 1)
        if lo < rng:
            thr = ((1 << 64) - rng) % rng
            while lo < thr:
                x = int(raw[k]); k += 1
                prod = x * rng
                lo = prod & ((1 << 64) - 1)
        vals.append(prod >> 64)
    assert vals == [c[1] for c in g["cases"]]
    # and the oracle's compiled routine agrees on a single range
    _, _, ints = pyoracle.pcg64(g["seed"], g["stream"], 8, int_hi=0)
    assert all(v == 0 for v in ints)


def test_oracle_uniform_int_routine_matches_golden_range():
    g = GOLD["uniform_int"]
    # first 8 cases have hi = 0, then 1, ...: check the compiled routine on hi=0
    # and the pure-Python restatement above on all; here the compiled routine
    # on a fresh stream against the Python restatement for hi = 6
    raw, _, ints = pyoracle.pcg64(7, 11, 64, int_hi=6)
    py = [(int(x) * 7) >> 64 for x in raw]
    assert list(ints) == py


@pytest.mark.parametrize("idx", range(5))
def test_time_grid_matches_eigen_linspaced(idx):
    g = GOLD["linspaced"][idx]
    grid = pyoracle.timegrid(g["dt"], g["maxtime"])
    assert np.array_equal(grid, np.array(g["grid"]))


def test_neglog_of_uniforms():
    g = GOLD["canonical"]
    u = np.array(g["u"])
    ref = np.array(g["neglog"])
    glibc = -pyoracle.log(u, impl=1)
    assert np.array_equal(glibc, ref)
    own = -pyoracle.log(u, impl=0)
    ulp = np.abs(own - ref) / np.spacing(np.abs(ref))
    assert ulp.max() <= 4.0


def test_bte_log_accuracy_wide_range():
    rng = np.random.default_rng(5)
    x = np.concatenate([rng.uniform(0, 1, 20000), 10.0 ** rng.uniform(-300, 300, 20000),
                        np.array([5e-324, 2.2250738585072014e-308, 0.5, 1.0, 2.0, 1e308])])
    own = pyoracle.log(x, impl=0)
    ref = pyoracle.log(x, impl=1)
    ok = ref != 0
    ulp = np.abs(own[ok] - ref[ok]) / np.spacing(np.abs(ref[ok]))
    assert ulp.max() <= 4.0
    assert own[x == 1.0][0] == 0.0
    assert np.isneginf(pyoracle.log(np.array([0.0]))[0])
