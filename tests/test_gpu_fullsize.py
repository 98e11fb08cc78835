"""The benchmark workloads at their full sizes, checked through properties
that do not depend on size (the restatement cannot run them in a test):

- transient RTA at scale (64x64x9 = 36864 modes, 2 um x 500 nm, 2422 cells,
  200 bins to 10 ns, p = 0.3, initial hot spot), one 2 M-particle slice of
  its N = 1e8: nothing is absorbed, so every particle spends each whole bin
  in some box and the tally of every bin is (N+ - N-) dt to FP64 rounding;
  the same seed draws the same trajectories, so the integer counters repeat
  exactly and the tallies to FP64 atomic-order rounding;
- the CPU-runnable ribbon (6144 modes, 50 cells, reservoirs, N = 1e6): the
  time budget |gz| <= N maxtime and the same repeatability."""
import numpy as np
import pytest

import btegpu
import synth

pytestmark = pytest.mark.gpu

KEYS = ("events", "wall_hits", "crossings", "absorbed", "specular_hits", "tally_updates")


def _run(engine, c, **kw):
    args = dict(T0=c["T0"], dt=c["dt"], maxtime=c["maxtime"], N=c["N"], specularity=c["specularity"],
                source=btegpu.SOURCE_INITIAL if c["source"] == "initial" else btegpu.SOURCE_WALLS)
    args.update(kw)
    return engine.rta_run(**args)


def test_transient_benchmark_at_scale_conserves_time_and_repeats(engine):
    c = synth.config1()
    engine.load_modes(c["modes"])
    engine.load_geometry(c["geom"])
    assert c["geom"]["nboxes"] == 2422
    a = _run(engine, c, seed=11, begin=0, end=2_000_000)
    b = _run(engine, c, seed=11, begin=0, end=2_000_000)
    assert a["absorbed"] == 0 and a["events"] > 3e9
    per_bin = a["gz"].sum(axis=0)
    assert per_bin.size == 200
    n = per_bin[0] / c["dt"]
    assert abs(n - round(n)) < 1e-3 and abs(round(n)) <= 2_000_000
    assert np.allclose(per_bin, per_bin[0], rtol=1e-9, atol=1e-9 * abs(per_bin[0]))
    for k in KEYS:
        if k in a:
            assert a[k] == b[k], k
    scale = np.abs(a["gz"]).max()
    assert np.allclose(a["gz"], b["gz"], rtol=0, atol=1e-12 * scale * 1e3)


def test_ribbon_benchmark_full_size_budget_and_repeats(engine):
    c = synth.config0()
    engine.load_modes(c["modes"])
    engine.load_geometry(c["geom"])
    a = _run(engine, c, seed=5)
    b = _run(engine, c, seed=5)
    tot = np.abs(a["gz"]).sum()
    assert 0 < tot <= c["N"] * c["maxtime"] * (1 + 1e-12)
    assert a["absorbed"] > 0 and a["events"] > c["N"]
    for k in KEYS:
        if k in a:
            assert a[k] == b[k], k
    scale = np.abs(a["gz"]).max()
    assert np.allclose(a["gz"], b["gz"], rtol=0, atol=1e-12 * scale * 1e3)
