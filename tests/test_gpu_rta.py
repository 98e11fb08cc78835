"""GPU parity tests of the RTA particle loop, through the C ABI.

Replay mode must reproduce the CPU restatement bit for bit: identical
128-bit fixed-point tallies and event counters, and FP64 tallies within
1e-12 of the largest tally (the benchmark spec's tolerance).  Production mode
(Philox streams, alias tables, FP64 atomics) must agree with the restatement
within 4 sigma over independent replicas, conserve particles, and keep the
same physics as the replay mode."""
import os
import subprocess

import numpy as np
import pytest

import btegpu
import pyoracle
import synth

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12


def _run(engine, case, **kw):
    engine.load_modes(case["modes"])
    engine.load_geometry(case["geom"])
    args = dict(T0=case["T0"], dt=case["dt"], maxtime=case["maxtime"], N=case["N"])
    args.update(kw)
    return engine.rta_run(**args)


def _triangle_ribbon(length=200.0, width=50.0, ncells=4, T_hot=301.0, T_cold=299.0, closed=False):
    """Ribbon whose cells are split into two triangles (not an axis-aligned
    grid: exercises the general convex-box kernels).  `closed`: the end boxes
    are ordinary boxes at T_hot and T_cold instead of reservoirs."""
    boxes, Teq, res = [], [], []
    dx = length / ncells
    for i in range(ncells):
        x0, x1 = i * dx, (i + 1) * dx
        boxes.append([(x0, 0.0), (x1, 0.0), (x0, width)])
        boxes.append([(x1, 0.0), (x1, width), (x0, width)])
        Teq += [300.0, 300.0]
        res += [0, 0]
    boxes.append([(-20.0, 0.0), (-20.0, width), (0.0, width), (0.0, 0.0)])
    boxes.append([(length, 0.0), (length, width), (length + 20.0, width), (length + 20.0, 0.0)])
    Teq += [T_hot, T_cold]
    if closed:  # initial deviation of the end boxes; Teq = T0 everywhere
        return synth._pack(boxes, [300.0] * len(Teq), Teq, res + [0, 0], synth.C_LAT)
    return synth._pack(boxes, Teq, list(Teq), res + [1, 1], synth.C_LAT)


@pytest.mark.parametrize("seed", [1, 7])
def test_replay_bit_exact_small(engine, seed):
    case = synth.small_case(n_particles=3000)
    g = _run(engine, case, seed=seed, mode=btegpu.MODE_REPLAY, exact=True)
    o = pyoracle.rta_run(case, seed=seed)
    assert np.array_equal(g["exact"], o["exact"])
    for k in ("events", "wall_hits", "crossings", "absorbed"):
        assert g[k] == o[k], k
    scale = np.abs(o["gz"]).max()
    for k in ("gz", "gz_jx", "gz_jy"):
        s = np.abs(o[k]).max()
        assert np.abs(g[k] - o[k]).max() <= REL_TOL * s, k
    assert np.abs(g["temperature"] - o["temperature"]).max() <= REL_TOL * 300.0
    assert g["Eeff"] == o["Eeff"]
    assert scale > 0


def test_replay_bit_exact_config0_table(engine):
    """The 32x32x6 mode table and 50-cell ribbon of the plain benchmark."""
    case = synth.config0(n_particles=1500)
    g = _run(engine, case, seed=3, mode=btegpu.MODE_REPLAY, exact=True)
    o = pyoracle.rta_run(case, seed=3, nthreads=8)
    assert np.array_equal(g["exact"], o["exact"])
    assert g["events"] == o["events"] and g["wall_hits"] == o["wall_hits"]
    s = np.abs(o["gz"]).max()
    assert np.abs(g["gz"] - o["gz"]).max() <= REL_TOL * s


def test_replay_bit_exact_general_geometry(engine):
    case = synth.small_case(n_particles=1500)
    case["geom"] = _triangle_ribbon()
    g = _run(engine, case, seed=5, mode=btegpu.MODE_REPLAY, exact=True)
    o = pyoracle.rta_run(case, seed=5)
    assert np.array_equal(g["exact"], o["exact"])
    assert g["events"] == o["events"] and g["crossings"] == o["crossings"]


def _hotspot_case(p=0.3, N=3000):
    g = synth.grid_geometry(400.0, 200.0, 20, 10, pore_center=(200.0, 100.0), pore_diameter=80.0,
                           hot_center=(100.0, 100.0), hot_sigma=30.0, hot_dT=1.0)
    return {"modes": synth.mode_table(8, 3, 3, 300.0, config=100), "geom": g, "T0": 300.0,
            "dt": 10.0, "maxtime": 200.0, "N": N, "source": "initial", "specularity": p}


@pytest.mark.parametrize("p", [0.0, 0.3])
def test_replay_bit_exact_hotspot_pore_specular(engine, p):
    """Scaled-down transient benchmark: staircase pore, initial Gaussian hot
    spot (outTref_distribution per cell), specular fraction p."""
    case = _hotspot_case(p)
    g = _run(engine, case, seed=8, mode=btegpu.MODE_REPLAY, source=btegpu.SOURCE_INITIAL,
             specularity=p, exact=True)
    o = pyoracle.rta_run(case, seed=8, nthreads=8)
    assert np.array_equal(g["exact"], o["exact"])
    for k in ("events", "wall_hits", "crossings", "specular_hits"):
        assert g[k] == o[k], k
    assert np.abs(g["temperature"] - o["temperature"]).max() <= REL_TOL * 300.0


def test_production_hotspot_agrees_with_restatement(engine):
    case = _hotspot_case(0.3, N=8000)
    R = 6
    def obs(r):
        return r["temperature"][:, [2, 5, 10, 19]].mean(axis=0)
    prod = np.array([obs(_run(engine, case, seed=500 + i, source=btegpu.SOURCE_INITIAL,
                              specularity=0.3)) for i in range(R)])
    orc = np.array([obs(pyoracle.rta_run(case, seed=600 + i, nthreads=8)) for i in range(R)])
    d = prod.mean(0) - orc.mean(0)
    se = np.sqrt(prod.var(0, ddof=1) / R + orc.var(0, ddof=1) / R)
    assert (np.abs(d) / np.maximum(se, 1e-300)).max() < 4.5


def test_replay_particle_ranges(engine):
    case = synth.small_case(n_particles=2000)
    g = _run(engine, case, seed=2, mode=btegpu.MODE_REPLAY, begin=500, end=1300, exact=True)
    o = pyoracle.rta_run(case, seed=2, begin=500, end=1300)
    assert np.array_equal(g["exact"], o["exact"])


def _observables(r):
    # late-time temperature of each interior box and the mean late flux
    nin = r["temperature"].shape[0] - 2
    T = r["temperature"][:nin, -5:].mean(axis=1)
    J = r["jx"][:nin, -5:].mean()
    return np.concatenate([T, [J * 1e-8]])


def test_production_agrees_with_restatement(engine):
    case = synth.small_case(n_particles=6000, maxtime=300.0)
    R = 6
    prod = np.array([_observables(_run(engine, case, seed=100 + i)) for i in range(R)])
    orc = np.array([_observables(pyoracle.rta_run(case, seed=200 + i, nthreads=8)) for i in range(R)])
    d = prod.mean(0) - orc.mean(0)
    se = np.sqrt(prod.var(0, ddof=1) / R + orc.var(0, ddof=1) / R)
    z = np.abs(d) / np.maximum(se, 1e-300)
    assert z.max() < 4.5, (z, prod.mean(0), orc.mean(0))


@pytest.mark.parametrize("flags", [0, btegpu.FLAG_GENERAL], ids=["polygon", "general"])
def test_production_general_kernel_agrees(engine, flags):
    """Boxes off a grid: the convex-polygon kernel (default) and the
    evolparticle-faithful kernel both agree with the restatement."""
    case = synth.small_case(n_particles=4000, maxtime=300.0)
    case["geom"] = _triangle_ribbon()
    R = 6
    prod = np.array([_observables(_run(engine, case, seed=300 + i, flags=flags)) for i in range(R)])
    orc = np.array([_observables(pyoracle.rta_run(case, seed=400 + i, nthreads=8)) for i in range(R)])
    d = prod.mean(0) - orc.mean(0)
    se = np.sqrt(prod.var(0, ddof=1) / R + orc.var(0, ddof=1) / R)
    assert (np.abs(d) / np.maximum(se, 1e-300)).max() < 4.5


def test_production_conserves_particle_time(engine):
    """Without reservoirs no particle is lost: every particle spends the whole
    bin width in some box, so the tally of each bin sums to N * dt exactly
    (up to FP64 rounding)."""
    g = synth.grid_geometry(400.0, 200.0, 20, 10, pore_center=(200.0, 100.0), pore_diameter=80.0,
                           hot_center=(100.0, 100.0), hot_sigma=30.0, hot_dT=1.0)
    case = {"modes": synth.mode_table(8, 3, 3, 300.0, config=100), "geom": g, "T0": 300.0,
            "dt": 10.0, "maxtime": 200.0, "N": 20000}
    for p in (0.0, 0.5):
        r = _run(engine, case, seed=9, source=btegpu.SOURCE_INITIAL, specularity=p)
        per_bin = r["gz"].sum(axis=0)
        n = per_bin[0] / case["dt"]
        assert abs(n - round(n)) < 1e-6
        assert np.allclose(per_bin, per_bin[0], rtol=1e-9, atol=0)
        assert r["absorbed"] == 0
        if p > 0:
            assert r["specular_hits"] > 0


@pytest.mark.parametrize("spec", [0.0, 0.6])
def test_polygon_kernel_conserves_particle_time(engine, spec):
    """Closed triangle ribbon (no reservoirs), initial deviation: every
    particle of the polygon kernel spends each whole bin in some box, so the
    tally of every bin is N * dt to FP64 rounding."""
    g = _triangle_ribbon(ncells=6, T_hot=300.5, T_cold=299.5, closed=True)
    case = {"modes": synth.mode_table(8, 3, 3, 300.0, config=100), "geom": g, "T0": 300.0,
            "dt": 10.0, "maxtime": 200.0, "N": 20000}
    r = _run(engine, case, seed=11, source=btegpu.SOURCE_INITIAL, specularity=spec)
    per_bin = r["gz"].sum(axis=0)
    n = per_bin[0] / case["dt"]
    assert n > 0 and abs(n - round(n)) < 1e-6
    assert np.allclose(per_bin, per_bin[0], rtol=1e-9, atol=0)
    assert r["absorbed"] == 0 and r["crossings"] > 0 and r["wall_hits"] > 0
    if spec > 0:
        assert r["specular_hits"] > 0


def test_walls_source_time_budget(engine):
    case = synth.small_case(n_particles=5000)
    r = _run(engine, case, seed=4)
    tot = np.abs(r["gz"]).sum()
    assert 0 < tot <= case["N"] * case["maxtime"] * (1 + 1e-12)
    assert r["events"] > case["N"] and r["absorbed"] > 0


def test_specular_walls_raise_conductance(engine):
    case = synth.small_case(n_particles=20000, maxtime=300.0)
    j0 = _run(engine, case, seed=11, specularity=0.0)["jx"][:5, -5:].mean()
    j1 = _run(engine, case, seed=11, specularity=1.0)["jx"][:5, -5:].mean()
    assert j1 > j0


def test_errors_are_reported(built):
    e = btegpu.Engine(0)
    with pytest.raises(btegpu.BteError) as ex:
        e.rta_run(300.0, 10.0, 100.0, 10)
    assert ex.value.code == btegpu.BTE_ERR_STATE
    case = synth.small_case(n_particles=10)
    m = dict(case["modes"])
    m["w"] = np.zeros_like(m["w"])
    e.load_modes(m)
    e.load_geometry(case["geom"])
    with pytest.raises(btegpu.BteError) as ex:
        e.rta_run(300.0, 10.0, 100.0, 10)
    assert ex.value.code == btegpu.BTE_ERR_VALUE
    e.load_modes(case["modes"])
    with pytest.raises(btegpu.BteError) as ex:
        e.rta_run(300.0, -1.0, 100.0, 10)
    assert ex.value.code == btegpu.BTE_ERR_INPUT
    with pytest.raises(btegpu.BteError) as ex:
        e.rta_run(300.0, 10.0, 100.0, 10, specularity=2.0)
    assert ex.value.code == btegpu.BTE_ERR_INPUT
    r = e.rta_run(300.0, 10.0, 100.0, 10)   # the context stays usable
    assert r["events"] > 0
    e.close()


def test_cli_dropin_writes_reference_csvs(built, tmp_path):
    case = synth.small_case(n_particles=2000)
    synth.write_geometry_xml(str(tmp_path / "beam.xml"), case["geom"])
    synth.write_modes_file(str(tmp_path / "modes.bin"), case["modes"])
    (tmp_path / "input.xml").write_text(
        '<RTA_MC2d>\n  <geometry file="beam.xml"/>\n  <time dt="10" maxtime="200"/>\n'
        '  <material name="synthetic" database="modes.bin" thickness="0.335" T0="300.0"/>\n'
        '  <particles N="2000"/>\n  <engine mode="replay" seed="5"/>\n</RTA_MC2d>\n')
    exe = os.path.join(os.path.dirname(built), "rtamc2d_gpu")
    r = subprocess.run([exe, "input.xml", "4", "2"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    T = np.loadtxt(tmp_path / "temperature_300K_run_0.csv", delimiter=",")
    assert T.shape == (20, 1 + case["geom"]["nboxes"])
    assert np.allclose(T[:, 0], (np.arange(20) + 0.5) * 10.0)
    assert (tmp_path / "jx_300K_run_1.csv").exists() and (tmp_path / "jy_300K_run_1.csv").exists()
    o = pyoracle.rta_run(case, seed=5)
    assert np.allclose(T[:, 1:], o["temperature"].T, rtol=0, atol=6e-4)  # CSV keeps 6 digits


def test_production_pulse_follows_the_analytic_response(engine):
    """Production mode, single pulse in an infinite medium (periodic boxes on
    all sides): Fourier components of the temperature against the exact RTA
    response of transient_analytic1d (src/analytic1d.cpp:1233-1283)."""
    import test_pulse_cpu as tp
    m = synth.mode_table(9, 3, 3, 300.0, config=100, even=True)
    case = {"modes": m, "geom": synth.pulse_geometry(tp.LX, tp.NX), "T0": 300.0, "dt": tp.DT,
            "maxtime": tp.TMAX, "N": 400000, "source": "initial"}
    runs = [_run(engine, case, seed=70 + k, source=btegpu.SOURCE_INITIAL) for k in range(8)]
    comps = tp.pulse_components(runs)
    for n, a in comps.items():
        an = tp.analytic_components(m, n)
        mu, se = a.mean(0), a.std(0, ddof=1) / np.sqrt(len(a))
        z = np.abs(mu - an) / se
        assert np.median(z) < 2.0 and z.max() < 6.0, (n, z)
