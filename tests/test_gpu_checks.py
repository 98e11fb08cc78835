"""Index checks and fault injection on the GPU, without faulting it:

- BTE_FLAG_CHECKS runs the production grid kernel in its checked variant
  (every table, tally and grid index tested before use; a violation stops
  the particle with BTE_ERR_CHECK).  Its checks draw nothing, so on the
  same seed it must give the plain variant's integer counters exactly, and
  no check may fire on the benchmark-shaped cases;
- a small flight cap per particle (a host-side parameter) sends every
  kernel down its limit path: the run returns BTE_ERR_LIMIT and the context
  stays usable."""
import numpy as np
import pytest

import btegpu
import synth

pytestmark = pytest.mark.gpu

KEYS = ("events", "wall_hits", "crossings", "absorbed", "specular_hits", "tally_updates")


def _hotspot_case():
    g = synth.grid_geometry(400.0, 200.0, 20, 10, pore_center=(200.0, 100.0), pore_diameter=80.0,
                           hot_center=(100.0, 100.0), hot_sigma=30.0, hot_dT=1.0)
    return {"modes": synth.mode_table(8, 3, 3, 300.0, config=100), "geom": g, "T0": 300.0,
            "dt": 10.0, "maxtime": 200.0, "N": 50000}


@pytest.mark.parametrize("which", ["hotspot", "ribbon"])
def test_checked_kernel_repeats_the_plain_one(engine, which):
    if which == "hotspot":
        c, kw = _hotspot_case(), dict(source=btegpu.SOURCE_INITIAL, specularity=0.3)
    else:
        c, kw = synth.config0(n_particles=200000), dict(source=btegpu.SOURCE_WALLS)
    engine.load_modes(c["modes"])
    engine.load_geometry(c["geom"])
    args = dict(T0=c["T0"], dt=c["dt"], maxtime=c["maxtime"], N=c["N"], seed=17, **kw)
    plain = engine.rta_run(**args)
    checked = engine.rta_run(flags=btegpu.FLAG_CHECKS, **args)
    for k in KEYS:
        assert plain[k] == checked[k], k
    scale = np.abs(plain["gz"]).max()
    assert np.allclose(plain["gz"], checked["gz"], rtol=0, atol=1e-9 * scale)


def test_flight_cap_injects_the_limit_path(engine):
    c = _hotspot_case()
    engine.load_modes(c["modes"])
    engine.load_geometry(c["geom"])
    args = dict(T0=c["T0"], dt=c["dt"], maxtime=c["maxtime"], N=2000, seed=3, source=btegpu.SOURCE_INITIAL)
    for mode, flags in ((btegpu.MODE_PRODUCTION, 0), (btegpu.MODE_PRODUCTION, btegpu.FLAG_CHECKS),
                        (btegpu.MODE_REPLAY, 0)):
        with pytest.raises(btegpu.BteError) as ex:
            engine.rta_run(mode=mode, flags=flags, flight_cap=3, **args)
        assert ex.value.code == btegpu.BTE_ERR_LIMIT
        r = engine.rta_run(mode=mode, flags=flags, **args)   # the context stays usable
        assert r["events"] > 3 * 2000
    # the general kernel (boxes that are not a grid) takes the same path
    engine.load_modes(synth.mode_table(8, 3, 3, 300.0, config=100))
    engine.load_geometry(synth.periodic_bar_geometry())
    with pytest.raises(btegpu.BteError) as ex:
        engine.rta_run(300.0, 10.0, 200.0, 2000, seed=3, flight_cap=2)
    assert ex.value.code == btegpu.BTE_ERR_LIMIT
    assert engine.rta_run(300.0, 10.0, 200.0, 2000, seed=3)["events"] > 0
