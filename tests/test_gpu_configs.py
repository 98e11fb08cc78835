"""GPU parity on the benchmark configurations' own inputs, through the C ABI.

The other GPU tests run small tables; these feed the CUDA path and the CPU
restatement the inputs the benchmark lines are measured on:

- the transient benchmark at scale (64x64x9 = 36864 modes, 2 um x 500 nm,
  100x25 cells with a 200 nm staircase pore, 2422 boxes, p = 0.3, 1 K hot
  spot of sigma 50 nm, 200 bins to 10 ns): replay mode bit for bit (128-bit
  tallies and every counter) on a few hundred particles, both as a small run
  and as a slice deep inside the N = 1e8 run; production mode against the
  restatement over 8 replicas on each side;
- the CPU-runnable ribbon (32x32x6 = 6144 modes, 50 cells, reservoirs):
  production against the restatement;
- beRTAMC2D on that ribbon with the 6141 x 6141 propagator of the beyond-RTA
  benchmark (dt = 1 ps), production against the restatement's step loop.

Production observables are compared per observable against 3 sigma and as
a family against 4.5 sigma (parity_stats)."""
import numpy as np
import pytest

import btegpu
import pyoracle
import synth
from parity_stats import check

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12
COUNTERS = ("events", "wall_hits", "crossings", "absorbed", "specular_hits")


def _load(engine, c):
    engine.load_modes(c["modes"])
    engine.load_geometry(c["geom"])


def _gpu(engine, c, **kw):
    args = dict(T0=c["T0"], dt=c["dt"], maxtime=c["maxtime"], N=c["N"], specularity=c["specularity"],
                source=btegpu.SOURCE_INITIAL if c["source"] == "initial" else btegpu.SOURCE_WALLS)
    args.update(kw)
    return engine.rta_run(**args)


def _replay_equal(g, o):
    assert np.array_equal(g["exact"], o["exact"])
    for k in COUNTERS:
        assert g[k] == o[k], k
    for k in ("gz", "gz_jx", "gz_jy"):
        s = np.abs(o[k]).max()
        assert s > 0 and np.abs(g[k] - o[k]).max() <= REL_TOL * s, k
    assert np.abs(g["temperature"] - o["temperature"]).max() <= REL_TOL * 300.0
    assert g["Eeff"] == o["Eeff"]


@pytest.fixture(scope="module")
def c1_engine(built):
    e = btegpu.Engine(0)
    yield e
    e.close()


def test_config1_replay_bit_exact(c1_engine):
    """400 particles of the transient benchmark's own tables and geometry."""
    c = synth.config1(n_particles=400)
    _load(c1_engine, c)
    assert c["geom"]["nboxes"] == 2422
    g = _gpu(c1_engine, c, seed=31, mode=btegpu.MODE_REPLAY, exact=True)
    o = pyoracle.rta_run(c, seed=31, nthreads=16)
    assert g["events"] > 400 * 100 and g["specular_hits"] > 0 and g["wall_hits"] > 0
    _replay_equal(g, o)


def test_config1_replay_slice_of_full_run(c1_engine):
    """Particles [5e7, 5e7 + 200) of the N = 1e8 run: the same Eeff, the
    per-cell generators of the full budget, particle streams deep in the
    index range."""
    c = synth.config1()
    _load(c1_engine, c)
    b, e = 50_000_000, 50_000_200
    g = _gpu(c1_engine, c, seed=5, mode=btegpu.MODE_REPLAY, exact=True, begin=b, end=e)
    o = pyoracle.rta_run(c, seed=5, nthreads=16, begin=b, end=e)
    _replay_equal(g, o)


def _centres(geom):
    v = np.asarray(geom["vertices"], float).reshape(-1, 4, 2)
    return v.mean(axis=1)


def _c1_observables(c):
    """Region x time-window means of the temperature and two flux means."""
    xy = _centres(c["geom"])
    rh = np.hypot(xy[:, 0] - 500.0, xy[:, 1] - 250.0)
    rp = np.hypot(xy[:, 0] - 1000.0, xy[:, 1] - 250.0)
    regions = {"hot": rh < 50.0, "ring": (rh >= 50.0) & (rh < 120.0),
               "pore": (rp < 140.0), "left": (rh >= 120.0) & (xy[:, 0] < 1000.0) & (rp >= 140.0),
               "right": (xy[:, 0] >= 1000.0) & (rp >= 140.0)}
    windows = {"b0-1": slice(0, 2), "b2-9": slice(2, 10), "b10-39": slice(10, 40), "b40-199": slice(40, 200)}
    names = [f"T_{r}_{w}" for r in regions for w in windows] + ["jx_east_b0-9", "jy_north_b0-9"]
    east = (xy[:, 0] > 550.0) & (xy[:, 0] < 900.0) & (np.abs(xy[:, 1] - 250.0) < 100.0)
    north = (xy[:, 1] > 300.0) & (np.abs(xy[:, 0] - 500.0) < 100.0)

    def obs(r):
        T = r["temperature"] - c["T0"]
        out = [T[m][:, s].mean() * 1e3 for m in regions.values() for s in windows.values()]
        out.append(r["jx"][east][:, :10].mean() * 1e-6)
        out.append(r["jy"][north][:, :10].mean() * 1e-6)
        return np.array(out)
    return names, obs


def test_config1_production_agrees_with_restatement(c1_engine):
    c = synth.config1(n_particles=20000)
    _load(c1_engine, c)
    names, obs = _c1_observables(c)
    R = 8
    gpu = np.array([obs(_gpu(c1_engine, c, seed=700 + i)) for i in range(R)])
    cpu = np.array([obs(pyoracle.rta_run(c, seed=800 + i, nthreads=16)) for i in range(R)])
    check(gpu, cpu, names, "config1 production")


def test_config0_production_agrees_with_restatement(engine):
    c = synth.config0(n_particles=20000)
    _load(engine, c)
    ncell = int(c["geom"]["nboxes"]) - 2
    groups = [slice(k * 10, (k + 1) * 10) for k in range(ncell // 10)]
    names = ([f"T_cells{g.start}-{g.stop - 1}_late" for g in groups]
             + [f"T_cells{g.start}-{g.stop - 1}_early" for g in groups] + ["jx_late", "jx_early"])

    def obs(r):
        T = r["temperature"][:ncell] - c["T0"]
        late = [T[g, -20:].mean() * 1e2 for g in groups]
        early = [T[g, 5:20].mean() * 1e2 for g in groups]
        return np.array(late + early + [r["jx"][:ncell, -20:].mean() * 1e-8,
                                        r["jx"][:ncell, 5:20].mean() * 1e-8])
    R = 8
    gpu = np.array([obs(_gpu(engine, c, seed=900 + i)) for i in range(R)])
    cpu = np.array([obs(pyoracle.rta_run(c, seed=1000 + i, nthreads=16)) for i in range(R)])
    check(gpu, cpu, names, "config0 production")


def test_config2_berta_agrees_with_restatement(engine):
    """The beyond-RTA benchmark's mode table and 6141 x 6141 propagator
    (dt = 1 ps) on the ribbon, 30 steps with Eeff giving ~1e4 particles."""
    c = synth.config0()
    m, g = c["modes"], c["geom"]
    P = synth.propagator(m, dt=1.0, T=300.0, use_torch=True)
    assert P.shape == (6141, 6141)
    engine.load_modes(m)
    engine.load_geometry(g)
    engine.load_propagator(P, 300.0)
    kw = dict(dt=1.0, maxtime=30.0, Eeff=2e-22)
    probe = engine.berta_run(seed=1, **kw)
    assert 2000 < probe["nparticles"][-1] < 1_000_000, probe["nparticles"][-1]
    assert probe["branchings"] > 0
    ncell = int(g["nboxes"]) - 2
    # after 30 ps the particles injected at the two reservoirs fill the
    # cells near the ends; the middle of the 1 um ribbon stays empty
    groups = [slice(0, 3), slice(3, 6), slice(6, 10), slice(10, 15), slice(35, 40), slice(40, 44),
              slice(44, 47), slice(47, 50)]
    names = [f"ed_cells{s.start}-{s.stop - 1}" for s in groups] + ["flux_x", "N_alive"]

    def obs(r):
        ed = r["ed"][-10:, :ncell]
        return np.array([ed[:, s].mean() * 1e-3 for s in groups]
                        + [r["flux"][-10:, :ncell, 0].mean() * 1e-8, r["nparticles"][-1] * 1e-3])
    R = 6
    gpu = np.array([obs(engine.berta_run(seed=40 + i, **kw)) for i in range(R)])
    cpu = np.array([obs(pyoracle.berta_run(m, g, P, seed=60 + i, **kw)) for i in range(R)])
    check(gpu, cpu, names, "config2 beRTA")
