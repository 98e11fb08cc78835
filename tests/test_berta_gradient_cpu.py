"""Gradient source term of the beyond-RTA loop (source_term_gradient,
src/beyondRTA_MC2d.cpp:597-676): with RTA scattering in an infinite medium
(a block closed by periodic boxes) the flux under a homogeneous gradient
follows the bulk conductivity with the loop's discrete lifetime,
synth.kappa_berta_steps, at every step of the transient."""
import numpy as np

import pyoracle
import synth

GX, DT = 0.01, 1.0


def berta_kappa(runs, start):
    """Per-run mean of -flux_x / grad over the rows from `start` on."""
    k = np.array([-r["flux"][start:, :4, 0].mean(axis=1) / (GX * 1e9) for r in runs])
    return k.mean(axis=1)


def test_restatement_gradient_source_gives_bulk_kappa():
    m = synth.mode_table(9, 3, 3, 300.0, config=100, even=True)
    g = synth.periodic_cell_geometry(40.0, 40.0, 2, 2)
    runs = [pyoracle.berta_run(m, g, None, DT, 300.0, 1e-23, seed=3 + k, rta=True, gradient=(GX, 0.0))
            for k in range(4)]
    nrow = runs[0]["flux"].shape[0]
    per = berta_kappa(runs, 100)
    expect = synth.kappa_berta_steps(m, 300.0, DT, np.arange(100, nrow)).mean()
    z = abs(per.mean() - expect) / (per.std(ddof=1) / np.sqrt(len(per)))
    assert z < 4.0, (per, expect)
    # no gradient, no source: the loop stays empty
    r0 = pyoracle.berta_run(m, g, None, DT, 20.0, 1e-23, seed=3, rta=True)
    assert r0["nparticles"].max() == 0
