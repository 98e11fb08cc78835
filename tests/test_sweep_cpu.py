"""CPU tests of the batched sweep layout: every case's ribbon in one
geometry (void gaps between ribbons, box material = case), per-case rates
and particle shares, in the restatement."""
import numpy as np

import btegpu
import pyoracle
import synth


def _tables(temps, n=8):
    return {T: synth.mode_table(n, 3, 3, T, config=100) for T in temps}


def test_union_geometry_is_one_grid(built):
    cases = synth.sweep_cases(n_widths=4, temps=(100.0, 300.0), w_min=20.0, w_max=200.0)
    g = synth.sweep_union_geometry(cases, ncells=10)
    ok, nx, ny = btegpu.debug_grid(g)
    assert ok == 1 and nx == 12 and ny == 2 * len(cases) - 1
    assert np.array_equal(np.unique(g["material"]), np.arange(len(cases)))


def test_single_case_union_equals_plain_ribbon():
    """A one-case union with material rates and share 1 is the plain ribbon
    run, draw for draw."""
    tab = _tables((300.0,))[300.0]
    cs = [{"T": 300.0, "width": 50.0, "budget": 800}]
    gu = synth.sweep_union_geometry(cs, length=200.0, ncells=5)
    gp = synth.sweep_ribbon(50.0, 300.0, length=200.0, ncells=5)
    base = {"modes": tab, "T0": 300.0, "dt": 10.0, "maxtime": 200.0, "N": 800}
    u = pyoracle.rta_run(dict(base, geom=gu), seed=3, nthreads=4,
                         materials=([tab["w"]], [300.0], [1.0]))
    p = pyoracle.rta_run(dict(base, geom=gp), seed=3, nthreads=4)
    assert np.array_equal(u["exact"], p["exact"])
    assert np.array_equal(u["jx"], p["jx"]) and np.array_equal(u["temperature"], p["temperature"])


def test_shares_split_the_particles():
    """With shares, the events of each case follow its budget; a case with
    share 0 gets no particle."""
    temps = (200.0, 300.0)
    tabs = _tables(temps)
    cs = [{"T": 200.0, "width": 40.0, "budget": 1}, {"T": 300.0, "width": 40.0, "budget": 1},
          {"T": 300.0, "width": 80.0, "budget": 1}]
    g = synth.sweep_union_geometry(cs, length=200.0, ncells=5)
    mats = ([tabs[c["T"]]["w"] for c in cs], [c["T"] for c in cs])
    case = {"modes": tabs[300.0], "geom": g, "T0": 300.0, "dt": 10.0, "maxtime": 100.0, "N": 3000}
    r = pyoracle.rta_run(case, seed=5, nthreads=4, materials=mats + ([0.5, 0.0, 0.5],))
    per = np.abs(r["gz"]).reshape(len(cs), 7, -1).sum(axis=(1, 2))
    assert per[1] == 0.0 and per[0] > 0 and per[2] > 0
