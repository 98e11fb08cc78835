"""Propagators tabulated in temperature (Scattering, src/beyondRTA_MC2d.cpp:
1130-1165; lirp, src/collision_operator.cpp:918-929) in the restatement: a
run at a tabulated Teq uses that propagator; otherwise it interpolates the
signed CDFs linearly between the first tabulated temperature above Teq and
the next one, and refuses when those do not exist or Teq is below the
lowest."""
import numpy as np
import pytest

import btegpu
import pyoracle
import synth


def _case():
    m = synth.mode_table(8, 3, 3, 300.0, config=100)
    g = synth.ribbon_geometry(200.0, 50.0, 5)
    return m, g


KW = dict(dt=1.0, maxtime=8.0, Eeff=2e-23, seed=5)


def test_tabulated_temperature_is_used_as_is():
    m, g = _case()
    P = synth.propagator(m)
    a = pyoracle.berta_run(m, g, P, **KW)
    b = pyoracle.berta_run(m, g, {280.0: np.eye(P.shape[0]), 300.0: P,
                                  320.0: synth.propagator(m, T=320.0, flip=0.1)}, **KW)
    assert np.array_equal(a["ed"], b["ed"]) and np.array_equal(a["H"], b["H"])


def test_interpolation_between_the_two_temperatures_above():
    """With equal matrices at 310 and 330 the interpolation at 300 returns
    that matrix's CDFs exactly; the one at 290 takes no part."""
    m, g = _case()
    P = synth.propagator(m)
    a = pyoracle.berta_run(m, g, P, **KW)
    b = pyoracle.berta_run(m, g, {290.0: np.eye(P.shape[0]), 310.0: P, 330.0: P}, **KW)
    assert np.array_equal(a["ed"], b["ed"]) and np.array_equal(a["H"], b["H"])


@pytest.mark.parametrize("temps", [(290.0, 310.0), (310.0, 330.0), (250.0, 280.0)])
def test_extrapolation_is_refused(temps):
    m, g = _case()
    P = synth.propagator(m)
    with pytest.raises(btegpu.BteError, match="Extrapolation"):
        pyoracle.berta_run(m, g, {t: P for t in temps}, **KW)
