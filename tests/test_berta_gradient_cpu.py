"""Gradient source term of the beyond-RTA loop (source_term_gradient,
src/beyondRTA_MC2d.cpp:597-676): with RTA scattering in an infinite medium
(a block closed by periodic boxes) the flux under a homogeneous gradient
follows the bulk conductivity with the loop's discrete lifetime,
synth.kappa_berta_steps, at every step of the transient."""
import numpy as np

import pyoracle
import synth

GRAD, DT = (0.01, 0.004), 1.0


def berta_flux(runs, start):
    """Per-run mean flux (x, y) per unit gradient, -flux / (K/m), over the
    rows from `start` on."""
    return np.array([-r["flux"][start:, :4].mean(axis=(0, 1)) / 1e9 for r in runs])


def expected_flux(m, start, nrow):
    """-flux / (K/m) expected from the discrete-time conductivity."""
    K = synth.kappa_berta_steps(m, 300.0, DT, np.arange(start, nrow)).mean(axis=0)
    return K @ np.array(GRAD)


def check_bulk(runs, m, start, zmax):
    per = berta_flux(runs, start)
    expect = expected_flux(m, start, runs[0]["flux"].shape[0])
    z = np.abs(per.mean(0) - expect) / (per.std(0, ddof=1) / np.sqrt(len(per)))
    assert z.max() < zmax, (z, per.mean(0), expect)


def test_restatement_gradient_source_gives_bulk_kappa():
    m = synth.mode_table(9, 3, 3, 300.0, config=100, even=True)
    g = synth.periodic_cell_geometry(40.0, 40.0, 2, 2)
    runs = [pyoracle.berta_run(m, g, None, DT, 300.0, 1e-23, seed=3 + k, rta=True, gradient=GRAD)
            for k in range(5)]
    check_bulk(runs, m, 100, 4.0)
    # no gradient, no source: the loop stays empty
    r0 = pyoracle.berta_run(m, g, None, DT, 20.0, 1e-23, seed=3, rta=True)
    assert r0["nparticles"].max() == 0
