"""Index checks and fault injection on the GPU, without faulting it:

- BTE_FLAG_CHECKS runs the production grid kernel in its checked variant
  (every table, tally and grid index tested before use; a violation stops
  the particle with BTE_ERR_CHECK).  Its checks draw nothing, so on the
  same seed it must give the plain variant's integer counters exactly, and
  no check may fire on the benchmark-shaped cases;
- a small flight cap per particle (a host-side parameter) sends every
  kernel down its limit path: the run returns BTE_ERR_LIMIT and the context
  stays usable;
- the grid kernel with two particles per thread draws the same streams and
  runs the same FP64 sequence per particle as the one-per-thread kernel, so
  it repeats its integer counters exactly and its tallies to FP64
  atomic-order rounding."""
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


@pytest.mark.parametrize("which", ["benchmark_slice", "ribbon"])
@pytest.mark.parametrize("shape", [(256, 1), (128, 4)])
def test_two_particles_per_thread_repeat_one_per_thread(engine, which, shape):
    if which == "benchmark_slice":
        c = synth.config1()
        kw = dict(source=btegpu.SOURCE_INITIAL, specularity=0.3, begin=3_000_000, end=3_200_000)
    else:
        c, kw = synth.config0(n_particles=200000), dict(source=btegpu.SOURCE_WALLS)
    engine.load_modes(c["modes"])
    engine.load_geometry(c["geom"])
    args = dict(T0=c["T0"], dt=c["dt"], maxtime=c["maxtime"], N=c["N"], seed=23, **kw)
    try:
        engine.set_tuning(block_threads=256, blocks_per_sm=3, smem_tally=0, particles_per_thread=1)
        one = engine.rta_run(**args)
        engine.set_tuning(block_threads=shape[0], blocks_per_sm=shape[1], smem_tally=0, particles_per_thread=2)
        two = engine.rta_run(**args)
    finally:  # back to the context's defaults
        engine.set_tuning(block_threads=0, blocks_per_sm=0, smem_tally=0, particles_per_thread=0)
    assert one["events"] > 0
    for k in KEYS:
        assert one[k] == two[k], k
    for k in ("gz", "gz_jx", "gz_jy"):
        scale = np.abs(one[k]).max()
        assert np.abs(two[k] - one[k]).max() <= 1e-9 * scale, k
