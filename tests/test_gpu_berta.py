"""GPU tests of the beyond-RTA (beRTAMC2D) step loop against the CPU
restatement: per-step energy density and flux agree within 4.5 sigma over
independent replicas, for propagator scattering (with sign branching) and
for the RTA alternative."""
import numpy as np
import pytest

import btegpu
import pyoracle
import synth

pytestmark = pytest.mark.gpu


def _case():
    m = synth.mode_table(8, 3, 3, 300.0, config=100)
    g = synth.ribbon_geometry(200.0, 50.0, 5)
    P = synth.propagator(m)
    return m, g, P


def _obs(r):
    # late-time energy density of the 5 interior boxes and the mean x flux
    ed = r["ed"][-10:, :5].mean(axis=0) * 1e-6
    fx = r["flux"][-10:, :5, 0].mean() * 1e-8
    return np.concatenate([ed, [fx]])


@pytest.mark.parametrize("rta", [False, True])
def test_berta_agrees_with_restatement(engine, rta):
    m, g, P = _case()
    engine.load_modes(m)
    engine.load_geometry(g)
    engine.load_propagator(P)
    R = 5
    kw = dict(dt=1.0, maxtime=40.0, Eeff=2e-23, rta=rta)
    gpu = np.array([_obs(engine.berta_run(seed=10 + i, **kw)) for i in range(R)])
    cpu = np.array([_obs(pyoracle.berta_run(m, g, P, seed=20 + i, **kw)) for i in range(R)])
    d = gpu.mean(0) - cpu.mean(0)
    se = np.sqrt(gpu.var(0, ddof=1) / R + cpu.var(0, ddof=1) / R)
    z = np.abs(d) / np.maximum(se, 1e-300)
    assert z.max() < 4.5, (z, gpu.mean(0), cpu.mean(0))


def test_berta_counts_and_branching(engine):
    m, g, P = _case()
    engine.load_modes(m)
    engine.load_geometry(g)
    engine.load_propagator(P)
    r = engine.berta_run(1.0, 20.0, 2e-23, seed=3, histogram=True)
    o = pyoracle.berta_run(m, g, P, 1.0, 20.0, 2e-23, seed=3)
    assert r["nsteps"] == o["nsteps"] == 21
    assert r["branchings"] > 0 and r["particle_steps"] > 0
    # particle numbers follow the same growth within a few percent
    assert abs(r["nparticles"][-1] - o["nparticles"][-1]) < 0.1 * o["nparticles"][-1]
    # the histogram of the last step sums to the signed particle count
    assert r["H"].sum() != 0
