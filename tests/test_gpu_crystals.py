"""GPU parity of several crystals joined by diffuse mismatch interfaces
(bte_load_mode_tables; change_material_diffuse, src/RTA_MC2D.cpp:871-964,
Diffuse_mismatch_distribution::reemit, src/sampling.cpp:831-902): replay
mode bit for bit against the restatement (transient runs from walls and
from an initial deviation, and the periodic steady state), the production
polygon kernel and the evolparticle-faithful kernel statistically, particle
time conserved across interfaces, and the outputs crystals do not take."""
import os
import subprocess

import numpy as np
import pytest

import btegpu
import pyoracle
import synth
from parity_stats import check

pytestmark = pytest.mark.gpu


def _tables():
    return synth.mode_table(8, 3, 3, 300.0, config=100), synth.mode_table(8, 3, 3, 300.0, config=101)


def _ribbon():
    """Ten 20 nm cells between a 301 K and a 299 K reservoir; cells 0-4 and
    the hot reservoir in crystal 0, cells 5-9 and the cold one in crystal 1."""
    g = synth.ribbon_geometry(200.0, 50.0, 10, T_hot=301.0, T_cold=299.0)
    g["material"] = np.array([0] * 5 + [1] * 5 + [0, 1], dtype=np.int32)
    return g


def test_two_crystal_ribbon_agrees_with_restatement(engine):
    A, B = _tables()
    g = _ribbon()
    engine.load_mode_tables([A, B])
    engine.load_geometry(g)
    kw = dict(T0=300.0, dt=10.0, maxtime=300.0)
    N = 20000
    names = ([f"T_cell{i}_late" for i in range(10)] + [f"T_cell{i}_early" for i in range(10)]
             + ["jx_late", "transmitted"])

    def obs(r):
        T = r["temperature"][:10] - 300.0
        return np.concatenate([T[:, -10:].mean(axis=1) * 10, T[:, 3:8].mean(axis=1) * 10,
                               [r["jx"][:10, -10:].mean() * 1e-7,
                                r["interface_transmissions"] / max(r["interface_hits"], 1)]])
    R = 6
    gpu = []
    for i in range(R):
        r = engine.rta_run(N=N, seed=100 + i, **kw)
        assert r["interface_hits"] > 0
        gpu.append(obs(r))
    cpu = [obs(pyoracle.rta_run_multi([A, B], g, N=N, seed=200 + i, nthreads=16, **kw)) for i in range(R)]
    check(np.array(gpu), np.array(cpu), names, "two crystals")
    # the interface resists: a temperature step between cells 4 and 5
    Tl = np.array(gpu)[:, :10].mean(0)
    assert Tl[4] - Tl[5] > 2.0 * max(Tl[3] - Tl[4], Tl[5] - Tl[6])


def test_two_crystals_conserve_particle_time(engine):
    A, B = _tables()
    g = synth.grid_geometry(200.0, 50.0, 10, 2)
    v = np.asarray(g["vertices"], float).reshape(-1, 4, 2).mean(axis=1)
    g["material"] = (v[:, 0] > 100.0).astype(np.int32)
    g["Tinit"] = np.where(g["material"] == 0, 300.5, 300.0)
    engine.load_mode_tables([A, B])
    engine.load_geometry(g)
    r = engine.rta_run(300.0, 10.0, 200.0, 20000, seed=9, source=btegpu.SOURCE_INITIAL, raw=True)
    assert r["interface_hits"] > 0 and 0 < r["interface_transmissions"] < r["interface_hits"]
    assert r["absorbed"] == 0
    per_bin = r["gz"].sum(axis=0)
    n = per_bin[0] / 10.0
    assert n > 0 and abs(n - round(n)) < 1e-6
    assert np.allclose(per_bin, per_bin[0], rtol=1e-9, atol=0)


def _closed_block():
    g = synth.grid_geometry(200.0, 50.0, 10, 2)
    v = np.asarray(g["vertices"], float).reshape(-1, 4, 2).mean(axis=1)
    g["material"] = (v[:, 0] > 100.0).astype(np.int32)
    g["Tinit"] = np.where(g["material"] == 0, 300.5, 300.0)
    return g


@pytest.mark.parametrize("source,thickness", [("walls", None), ("initial", None), ("walls", (0.335, 0.5)),
                                              ("initial", (0.6, 0.335))])
def test_two_crystals_replay_is_bit_exact(engine, source, thickness):
    """Replay mode (pcg64 streams, CDF inversion, the interface drawing its
    re-emission from the particle's stream as the restatement does)
    reproduces the restatement's multi-crystal run draw for draw: identical
    128-bit tallies and counters, on the ribbon with reservoirs in each
    crystal and on the closed block with an initial deviation."""
    A, B = _tables()
    if source == "walls":
        g, src, N = _ribbon(), btegpu.SOURCE_WALLS, 4000
    else:
        g, src, N = _closed_block(), btegpu.SOURCE_INITIAL, 4000
    engine.load_mode_tables([A, B], thickness=thickness)
    engine.load_geometry(g)
    kw = dict(T0=300.0, dt=10.0, maxtime=200.0)
    r = engine.rta_run(N=N, seed=5, mode=btegpu.MODE_REPLAY, source=src, exact=True, **kw)
    o = pyoracle.rta_run_multi([A, B], g, N=N, seed=5, nthreads=16, source=src, thickness=thickness, **kw)
    assert r["interface_hits"] > 0 and 0 < r["interface_transmissions"] < r["interface_hits"]
    for k in ("events", "wall_hits", "crossings", "absorbed", "interface_hits", "interface_transmissions"):
        assert r[k] == o[k], (k, r[k], o[k])
    assert np.array_equal(r["exact"], o["exact"])
    assert r["Eeff"] == o["Eeff"]
    # the outputs: each box's volume and C_v correction at its crystal's thickness
    rr = engine.rta_run(N=N, seed=5, mode=btegpu.MODE_REPLAY, source=src, **kw)
    assert np.allclose(rr["temperature"], o["temperature"], rtol=0, atol=1e-12 * 300.0)
    assert np.allclose(rr["jx"], o["jx"], rtol=1e-12, atol=1e-12 * np.abs(o["jx"]).max())


def test_two_crystals_general_kernel_agrees_with_restatement(engine):
    """The evolparticle-faithful production kernel (BTE_FLAG_GENERAL) with
    the interfaces: the ribbon's temperatures and transmitted fraction
    against the restatement."""
    A, B = _tables()
    g = _ribbon()
    engine.load_mode_tables([A, B])
    engine.load_geometry(g)
    kw = dict(T0=300.0, dt=10.0, maxtime=300.0)
    N, R = 20000, 6
    names = [f"T_cell{i}_late" for i in range(10)] + ["transmitted"]

    def obs(r):
        T = r["temperature"][:10] - 300.0
        return np.concatenate([T[:, -10:].mean(axis=1) * 10,
                               [r["interface_transmissions"] / max(r["interface_hits"], 1)]])
    gpu = [obs(engine.rta_run(N=N, seed=300 + i, flags=btegpu.FLAG_GENERAL, **kw)) for i in range(R)]
    cpu = [obs(pyoracle.rta_run_multi([A, B], g, N=N, seed=400 + i, nthreads=16, **kw)) for i in range(R)]
    check(np.array(gpu), np.array(cpu), names, "two crystals, evolparticle-faithful kernel")


def test_crystals_refuse_rate_sets_and_mixed_q_grids_in_spectral_outputs(engine):
    """Rate sets are for one mode table; spectral locations in crystals of
    different q grids have no common fd_q layout."""
    A, _ = _tables()
    B = synth.mode_table(12, 3, 3, 300.0, config=102)
    engine.load_mode_tables([A, B])
    engine.load_geometry(_ribbon())
    with pytest.raises(btegpu.BteError, match="rate sets"):
        engine.load_materials([A["w"]], [300.0])
    engine.set_spectral([2, 7], 10)
    try:
        r = engine.rta_run(300.0, 10.0, 100.0, 1000)
        with pytest.raises(btegpu.BteError, match="different q grids"):
            engine.get_spectral(r["gz"].shape[1])
    finally:
        engine.set_spectral([], 0)


def test_two_crystal_steady_state_agrees_with_restatement(engine):
    """Steady state of the layered periodic bar (strips 0-4 in crystal 0,
    5-9 in crystal 1): the polygon kernel's interface re-emissions, carried
    into the next generation, against the restatement."""
    A, B = _tables()
    g = synth.layered_bar_geometry()
    engine.load_mode_tables([A, B])
    engine.load_geometry(g)
    # per crystal (the strips of one crystal move together), plus the
    # interface's own counts.  The generation chains make a replica's flux
    # heavy-tailed at a few thousand particles; 16000 per replica keeps the
    # two-sample z near normal (100 replicas of 4000 each agreed to
    # |z| < 2 on every observable)
    N, R = 16000, 12
    names = ["T_crystal0", "T_crystal1", "jy_crystal0", "jy_crystal1", "transmitted", "hits_per_N"]

    def obs(r):
        T = r["temperature"][:10] - 300.0
        return np.array([T[:5].mean(), T[5:].mean(), r["jy"][:5].mean() * 1e-8, r["jy"][5:10].mean() * 1e-8,
                         r["interface_transmissions"] / max(r["interface_hits"], 1), r["interface_hits"] / N])
    gpu = []
    for i in range(R):
        r = engine.steady_run(300.0, (0.0, -0.01), N, seed=300 + i)
        assert r["interface_hits"] > 0
        assert r["events"] == N + r["births"] + r["interface_hits"]
        gpu.append(obs(r))
    cpu = [obs(pyoracle.steady_run_multi([A, B], g, 300.0, (0.0, -0.01), N, seed=400 + i, nthreads=16))
           for i in range(R)]
    check(np.array(gpu), np.array(cpu), names, "two-crystal steady state")
    # the evolparticle-faithful kernel with the same interfaces
    gen = [obs(engine.steady_run(300.0, (0.0, -0.01), N, seed=500 + i, flags=btegpu.FLAG_GENERAL))
           for i in range(R)]
    check(np.array(gen), np.array(cpu), names, "two-crystal steady state, evolparticle-faithful kernel")


def test_two_crystal_steady_replay_is_bit_exact(engine):
    """The steady state of the layered bar (its crystals 0.335 and 0.45 nm
    thick) in replay mode against the restatement's steady run over several
    materials: every generation, its 128-bit tallies and the counters,
    interface re-emissions included, and the temperatures."""
    A, B = _tables()
    g = synth.layered_bar_geometry()
    engine.load_mode_tables([A, B], thickness=(0.335, 0.45))
    engine.load_geometry(g)
    r = engine.steady_run(300.0, (0.0, -0.01), 3000, seed=6, mode=btegpu.MODE_REPLAY)
    o = pyoracle.steady_run_multi([A, B], g, 300.0, (0.0, -0.01), 3000, seed=6, nthreads=16,
                                  thickness=(0.335, 0.45))
    assert r["generations"] == o["generations"] > 1
    assert r["interface_hits"] > 0
    for k in ("events", "wall_hits", "crossings", "absorbed", "translations", "scattered", "births", "lost",
              "interface_hits", "interface_transmissions"):
        assert r[k] == o[k], (k, r[k], o[k])
    assert np.array_equal(r["exact"], o["exact"])
    assert np.array_equal(r["log"], o["log"])
    assert r["Eeff"] == o["Eeff"]
    assert np.abs(r["temperature"] - o["temperature"]).max() <= 1e-12 * 300.0


def test_rtamc2d_cli_reads_several_materials(built, tmp_path):
    """rtamc2d_gpu with two <material>s of different thickness and boxes
    naming theirs in <MaterialID> runs the crystals path: the CSV's late
    temperatures step down at the interface."""
    A, B = _tables()
    g = _ribbon()
    synth.write_geometry_xml(str(tmp_path / "beam.xml"), g, material="mat")
    synth.write_modes_file(str(tmp_path / "a.bin"), A)
    synth.write_modes_file(str(tmp_path / "b.bin"), B)
    (tmp_path / "input.xml").write_text(
        '<RTA_MC2d>\n  <geometry file="beam.xml"/>\n  <time dt="10" maxtime="200"/>\n'
        '  <material name="mat0" database="a.bin" thickness="0.335" T0="300.0"/>\n'
        '  <material name="mat1" database="b.bin" thickness="0.5" T0="300.0"/>\n'
        '  <particles N="20000"/>\n  <engine seed="5"/>\n</RTA_MC2d>\n')
    exe = os.path.join(os.path.dirname(built), "rtamc2d_gpu")
    r = subprocess.run([exe, "input.xml", "4", "1"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    T = np.loadtxt(tmp_path / "temperature_300K_run_0.csv", delimiter=",")
    assert T.shape == (20, 1 + g["nboxes"])
    late = T[-5:, 1:11].mean(axis=0)
    assert late[4] - late[5] > 2.0 * max(late[3] - late[4], late[5] - late[6])


def test_two_crystal_spectral_outputs(engine):
    """Spectral decomposition at a box of each crystal (crystals 0.335 and
    0.5 nm thick): replay's per-mode time tally equals the restatement's
    over the concatenated modes, and each location's outputs use its own
    crystal's modes, omega ticks, broadening, volume and heat capacity."""
    A, B = _tables()
    g = _ribbon()
    th = (0.335, 0.5)
    engine.load_mode_tables([A, B], thickness=th)
    engine.load_geometry(g)
    kw = dict(T0=300.0, dt=10.0, maxtime=200.0)
    locs, nw = [2, 7], 200
    engine.set_spectral(locs, nomega=nw)
    try:
        r = engine.rta_run(N=4000, seed=8, mode=btegpu.MODE_REPLAY, **kw)
        nbins = r["gz"].shape[1]
        sp = engine.get_spectral(nbins)
    finally:
        engine.set_spectral([])
    nA, nB = A["omega"].size, B["omega"].size
    pyoracle.set_spectral(locs)
    try:
        pyoracle.rta_run_multi([A, B], g, N=4000, seed=8, nthreads=8, thickness=th, **kw)
        _, val = pyoracle.spectral_raw((2, nbins, nA + nB))
    finally:
        pyoracle.set_spectral([])
    assert np.array_equal(sp["raw"], val)
    assert np.abs(val[0, :, nA:]).max() == 0 and np.abs(val[1, :, :nA]).max() == 0
    for l, (tab, off) in enumerate(((A, 0), (B, nA))):
        raw = sp["raw"][l:l + 1, :, off:off + tab["omega"].size]
        grid, dT, jx, jy, fq = pyoracle.spectral_post(tab, raw, nw)
        assert np.allclose(sp["omega"][l], grid, rtol=1e-14)
        # dT per tick and the box temperature share the factor Eeff / V_box / (C_v / vcorr)
        c = (r["temperature"][locs[l], -1] - 300.0) / raw[0].sum()
        assert np.allclose(sp["dT_omega"][l], c * dT[0], rtol=1e-9, atol=1e-12 * np.abs(sp["dT_omega"][l]).max())
        for mine, ref in ((sp["jx_omega"][l], jx[0]), (sp["jy_omega"][l], jy[0]), (sp["fd_q"][l], fq[0])):
            i = np.argmax(np.abs(ref))
            k = mine.flat[i] / ref.flat[i]
            assert np.allclose(mine, k * ref, rtol=1e-9, atol=1e-12 * np.abs(mine).max())


def _periodic_two_crystal_cell():
    """A ribbon periodic in x (2 x 2 cells of 20 nm x 50 nm between diffuse
    walls) with its left column in crystal 0 and its right column in
    crystal 1; each periodic box takes the crystal of the cells its
    translation leads to (right box -> left column: crystal 0, left box ->
    right column: crystal 1), so that particles meet an interface on their
    way into a periodic box as well as between the columns."""
    g = synth.periodic_ribbon_geometry(40.0, 100.0, 2, 2)
    g["material"] = np.array([0, 0, 1, 1, 0, 1], dtype=np.int32)
    g["Tinit"] = np.where(np.arange(g["nboxes"]) < 2, 300.5, 300.0)
    return g


def test_two_crystals_meet_interfaces_at_periodic_boxes(engine):
    """Interfaces into periodic boxes of the other crystal (re-emission,
    then the translation): replay bit for bit against the restatement,
    transient from an initial deviation and steady state under a gradient;
    the production kernels run the same geometry without error."""
    A, B = _tables()
    g = _periodic_two_crystal_cell()
    engine.load_mode_tables([A, B])
    engine.load_geometry(g)
    kw = dict(T0=300.0, dt=10.0, maxtime=200.0)
    r = engine.rta_run(N=3000, seed=3, mode=btegpu.MODE_REPLAY, source=btegpu.SOURCE_INITIAL, exact=True, **kw)
    o = pyoracle.rta_run_multi([A, B], g, N=3000, seed=3, nthreads=8, source=btegpu.SOURCE_INITIAL, **kw)
    assert r["interface_hits"] > 0 and r["translations"] > 0
    for k in ("events", "crossings", "interface_hits", "interface_transmissions", "translations"):
        assert r[k] == o[k], (k, r[k], o[k])
    assert np.array_equal(r["exact"], o["exact"])
    s = engine.steady_run(300.0, (-0.01, 0.0), 2000, seed=4, mode=btegpu.MODE_REPLAY)
    so = pyoracle.steady_run_multi([A, B], g, 300.0, (-0.01, 0.0), 2000, seed=4, nthreads=8)
    assert s["interface_hits"] > 0 and s["generations"] == so["generations"]
    assert np.array_equal(s["exact"], so["exact"]) and np.array_equal(s["log"], so["log"])
    # production: the polygon kernels (transient and steady) on the same geometry
    p = engine.rta_run(N=20000, seed=5, source=btegpu.SOURCE_INITIAL, **kw)
    assert p["interface_hits"] > 0 and np.isfinite(p["temperature"]).all()
    ps = engine.steady_run(300.0, (-0.01, 0.0), 20000, seed=6)
    assert ps["interface_hits"] > 0 and np.isfinite(ps["temperature"]).all()
