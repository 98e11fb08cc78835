"""The restatement's diffuse mismatch model against the reference's own code.

tests/golden/ref_pins_dmm.json holds, for two seeded 4x4 x 6 mode tables
(A and B) and two interface normals, every lookup entry of the reference's
Diffuse_mismatch_distribution (src/sampling.cpp:437-830: allowed
transitions by Gaussian DOS overlap, the closest-frequency reflection for
incident modes without one, the cumulative probabilities over each side's
incident modes) and draws of its reemit (:831-902) from the object's own
pcg64, compiled by oracle/build_ref.py from the cited line ranges.  The
restatement (oracle/rta_oracle.cpp, build_dmm / dmm_reemit) must give the
same entries, the cumulative values to 1e-14, and the same draws."""
import json
import os

import numpy as np
import pytest

import pyoracle

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "ref_pins_dmm.json")))


def _modes(d):
    m = dict(d)
    m["grid"] = (4, 4, 1)
    for k in ("omega", "vg", "w", "dq"):
        m[k] = np.ascontiguousarray(m[k], dtype=np.float64)
    return m


A, B = _modes(GOLD["modes_A"]), _modes(GOLD["modes_B"])


@pytest.mark.parametrize("case", range(len(GOLD["cases"])))
def test_dmm_lookup_tables_match_the_reference(case):
    c = GOLD["cases"][case]
    tab = pyoracle.dmm_table(A, B, c["normal"], GOLD["thickness"], GOLD["Tref"])
    for s, key in enumerate(("A", "B")):
        ref = c[key]
        assert len(tab[s]) == len(ref)
        nonempty = 0
        for i, (side, idx, cum) in enumerate(tab[s]):
            r = np.asarray(ref[i], dtype=float).reshape(-1, 3)
            assert len(side) == len(r), (key, i)
            if len(r):
                nonempty += 1
                assert np.array_equal(side, r[:, 0].astype(int)), (key, i)
                assert np.array_equal(idx, r[:, 1].astype(int)), (key, i)
                assert np.allclose(cum, r[:, 2], rtol=1e-14, atol=0), (key, i)
        assert nonempty > 0
        last = max(float(np.asarray(x, float).reshape(-1, 3)[-1, 2]) for x in ref if len(x))
        assert abs(last - 1.0) < 1e-12


@pytest.mark.parametrize("case", range(len(GOLD["cases"])))
def test_dmm_reemit_draws_match_the_reference(case):
    c = GOLD["cases"][case]
    r = np.asarray(c["reemit"], dtype=np.int64)
    side, idx = pyoracle.dmm_reemit(A, B, c["normal"], GOLD["thickness"], GOLD["Tref"], c["seed"], c["stream"],
                                    r[:, 0])
    nb = np.where(side == 0, int(A["nb"]), int(B["nb"]))
    assert np.array_equal(side, r[:, 1])
    assert np.array_equal(idx // nb, r[:, 2]) and np.array_equal(idx % nb, r[:, 3])
