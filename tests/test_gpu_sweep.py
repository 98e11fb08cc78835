"""GPU tests of the batched sweep: every case's ribbon in one geometry with
per-case rates (materials) and particle shares, run by the grid kernel in
one launch, against the restatement (replay: bit-exact) and against
per-case plain runs (production: within 4.5 sigma)."""
import numpy as np
import pytest

import btegpu
import pyoracle
import synth

pytestmark = pytest.mark.gpu


def _sweep(n=8):
    temps = (200.0, 300.0)
    tabs = {T: synth.mode_table(n, 3, 3, T, config=100) for T in temps}
    cs = [{"T": T, "width": w, "budget": N} for T in temps for w, N in ((30.0, 1000), (120.0, 3000))]
    return tabs, cs


def test_union_replay_bit_exact(engine):
    tabs, cs = _sweep()
    g = synth.sweep_union_geometry(cs, length=200.0, ncells=5)
    share = np.array([c["budget"] for c in cs], float)
    share /= share.sum()
    mats = ([tabs[c["T"]]["w"] for c in cs], [c["T"] for c in cs], share)
    N = sum(c["budget"] for c in cs)
    engine.load_modes(tabs[300.0])
    engine.load_geometry(g)
    engine.load_materials(*mats)
    gr = engine.rta_run(300.0, 10.0, 200.0, N, seed=9, mode=btegpu.MODE_REPLAY, exact=True)
    case = {"modes": tabs[300.0], "geom": g, "T0": 300.0, "dt": 10.0, "maxtime": 200.0, "N": N}
    o = pyoracle.rta_run(case, seed=9, nthreads=8, materials=mats)
    assert np.array_equal(gr["exact"], o["exact"])
    assert gr["events"] == o["events"]
    assert np.abs(gr["temperature"] - o["temperature"]).max() <= 1e-12 * 300.0
    assert np.allclose(gr["jx"], o["jx"], rtol=1e-12, atol=0)


def test_union_production_matches_plain_cases(engine):
    """kappa_eff of each case from the batched launch agrees with the same
    case run alone."""
    tabs, cs = _sweep()
    g = synth.sweep_union_geometry(cs, length=200.0, ncells=5)
    share = np.array([c["budget"] for c in cs], float)
    share /= share.sum()
    N = sum(c["budget"] for c in cs) * 4
    R = 6
    engine.load_modes(tabs[300.0])
    engine.load_geometry(g)
    engine.load_materials([tabs[c["T"]]["w"] for c in cs], [c["T"] for c in cs], share)
    kb = np.array([[synth.sweep_kappa(r["jx"], slice(7 * i, 7 * i + 5), length=200.0)
                    for i in range(len(cs))]
                   for r in (engine.rta_run(300.0, 10.0, 200.0, N, seed=30 + k) for k in range(R))])
    kp = np.zeros((R, len(cs)))
    for i, c in enumerate(cs):
        e = btegpu.Engine(0)
        e.load_modes(tabs[c["T"]])
        e.load_geometry(synth.sweep_ribbon(c["width"], c["T"], length=200.0, ncells=5))
        for k in range(R):
            r = e.rta_run(c["T"], 10.0, 200.0, c["budget"] * 4, seed=60 + k)
            kp[k, i] = synth.sweep_kappa(r["jx"], slice(0, 5), length=200.0)
        e.close()
    d = kb.mean(0) - kp.mean(0)
    se = np.sqrt(kb.var(0, ddof=1) / R + kp.var(0, ddof=1) / R)
    z = np.abs(d) / np.maximum(se, 1e-300)
    assert z.max() < 4.5, (z, kb.mean(0), kp.mean(0))


def test_share_update_and_geometry_reload(engine):
    tabs, cs = _sweep()
    g = synth.sweep_union_geometry(cs, length=200.0, ncells=5)
    engine.load_modes(tabs[300.0])
    engine.load_geometry(g)
    rates = [tabs[c["T"]]["w"] for c in cs]
    Ts = [c["T"] for c in cs]
    engine.load_materials(rates, Ts, [0.25, 0.25, 0.25, 0.25])
    engine.rta_run(300.0, 10.0, 100.0, 2000, seed=1)
    engine.load_materials(rates, Ts, [0.0, 0.5, 0.0, 0.5])   # shares only: walls reweighted
    r = engine.rta_run(300.0, 10.0, 100.0, 2000, seed=1, mode=btegpu.MODE_REPLAY)
    per = np.abs(r["gz"]).reshape(len(cs), 7, -1).sum(axis=(1, 2))
    assert per[0] == 0.0 and per[2] == 0.0 and per[1] > 0 and per[3] > 0
    # a new geometry with the same wall normals keeps the Lambert table; the
    # run equals a fresh context's
    engine.load_materials([], [])
    rib = synth.sweep_ribbon(60.0, 300.0, length=200.0, ncells=5)
    engine.load_geometry(rib)
    a = engine.rta_run(300.0, 10.0, 100.0, 1500, seed=4, mode=btegpu.MODE_REPLAY, exact=True)
    e = btegpu.Engine(0)
    e.load_modes(tabs[300.0])
    e.load_geometry(rib)
    b = e.rta_run(300.0, 10.0, 100.0, 1500, seed=4, mode=btegpu.MODE_REPLAY, exact=True)
    e.close()
    assert np.array_equal(a["exact"], b["exact"])


def test_replica_groups_sum_to_the_run_and_estimate_it(engine):
    """bte_set_groups: particle p tallies into group p mod G.  The run's
    outputs are the groups' sum, so a grouped run repeats the plain run
    (same particles, same counters, tallies to atomic-order rounding), the
    mean of the group results (each scaled to the whole run) is the run's
    result, and the spread of the groups is the batch-means error: it
    agrees with the spread of independent plain runs."""
    c = synth.config0(n_particles=400000)
    engine.load_modes(c["modes"])
    engine.load_geometry(c["geom"])
    args = dict(T0=c["T0"], dt=c["dt"], maxtime=c["maxtime"], N=c["N"])
    plain = engine.rta_run(seed=41, **args)
    G = 8
    engine.set_groups(G)
    try:
        grouped = engine.rta_run(seed=41, **args)
        shape = grouped["jx"].shape
        groups = [engine.group_result(g, shape, raw=True) for g in range(G)]
    finally:
        engine.set_groups(0)
    for k in ("events", "wall_hits", "crossings", "absorbed", "tally_updates"):
        assert grouped[k] == plain[k], k
    for k in ("gz", "gz_jx", "gz_jy", "jx"):
        scale = np.abs(plain[k]).max()
        assert np.abs(grouped[k] - plain[k]).max() <= 1e-9 * scale, k
        mean = np.mean([g[k] for g in groups], axis=0)
        assert np.abs(mean - grouped[k]).max() <= 1e-9 * scale, k
    ncell = int(c["geom"]["nboxes"]) - 2
    kap = lambda r: synth.sweep_kappa(r["jx"], slice(0, ncell), length=1000.0)
    kg = np.array([kap(g) for g in groups])
    assert abs(kg.mean() - kap(grouped)) <= 1e-9 * abs(kap(grouped))
    # the groups' spread estimates the error of one run of N/G particles;
    # independent runs of N/G particles give the same spread
    runs = np.array([kap(engine.rta_run(seed=500 + i, **{**args, "N": c["N"] // G})) for i in range(G)])
    ratio = kg.var(ddof=1) / runs.var(ddof=1)
    assert 1 / 9.0 < ratio < 9.0, (kg.std(ddof=1), runs.std(ddof=1))  # F(7, 7): about 1 % two-sided
    assert abs(kg.mean() - runs.mean()) < 4.5 * np.sqrt(kg.var(ddof=1) / G + runs.var(ddof=1) / G)
