"""Spectral decomposition at selected boxes (<spectral>, src/RTA_MC2D.cpp:
150-175, :699-766, :2350-2420): the per-mode time tally, exact in replay
mode, and the four outputs built from it."""
import os
import subprocess

import numpy as np
import pytest

import btegpu
import pyoracle
import synth


def _case():
    return synth.small_case(n_particles=2000)


def test_restatement_spectral_tally_sums_to_the_box_tally():
    """Summed over modes, the per-mode time of a location is the box's gz
    tally, to the last fixed-point unit."""
    case = _case()
    pyoracle.set_spectral([1, 3])
    try:
        r = pyoracle.rta_run(case, seed=4, nthreads=4)
        nb = r["gz"].shape[1]
        n = case["modes"]["omega"].size
        ex, val = pyoracle.spectral_raw((2, nb, n))
    finally:
        pyoracle.set_spectral([])
    exact = ex[..., 0].astype(object) * 2 ** 64 + ex[..., 1].astype(np.uint64).astype(object)
    tot = exact.sum(axis=2)
    gz = r["exact"][..., 0, 0].astype(object) * 2 ** 64 + r["exact"][..., 0, 1].astype(np.uint64).astype(object)
    assert np.all(tot[0] == gz[1]) and np.all(tot[1] == gz[3])
    assert np.abs(val).sum() > 0


def _check_outputs(case, g, sp, nomega):
    """The engine's four outputs against the restated post-processing: the
    temperature per tick carries the box temperature's own scale (its time
    integral summed over modes is the box's gz), the fluxes and the q-mesh
    distribution one constant each."""
    grid, dT, jx, jy, fq = pyoracle.spectral_post(case["modes"], sp["raw"], nomega)
    assert np.allclose(sp["omega"], grid[None, :], rtol=1e-14)
    dT_box = g["temperature"][[1, 3]] - case["T0"]
    cum = np.cumsum(sp["raw"].sum(axis=2), axis=1)
    for l in range(2):
        b = np.nonzero(np.abs(cum[l]) > 1e-6 * np.abs(cum[l]).max())[0]
        scale = dT_box[l, b] / cum[l, b]
        assert np.allclose(scale, scale[0], rtol=1e-9)
        assert np.allclose(sp["dT_omega"][l], scale[0] * dT[l], rtol=1e-9,
                           atol=1e-12 * np.abs(sp["dT_omega"][l]).max())
        for mine, ref in ((sp["jx_omega"][l], jx[l]), (sp["jy_omega"][l], jy[l]), (sp["fd_q"][l], fq[l])):
            i = np.argmax(np.abs(ref))
            c = mine.flat[i] / ref.flat[i]
            assert np.allclose(mine, c * ref, rtol=1e-9, atol=1e-12 * np.abs(mine).max())


@pytest.mark.gpu
def test_spectral_replay_bit_exact_and_outputs(engine):
    case = _case()
    engine.load_modes(case["modes"])
    engine.load_geometry(case["geom"])
    engine.set_spectral([1, 3], nomega=400)
    g = engine.rta_run(case["T0"], case["dt"], case["maxtime"], case["N"], seed=4,
                       mode=btegpu.MODE_REPLAY)
    nb = g["gz"].shape[1]
    sp = engine.get_spectral(nb)
    pyoracle.set_spectral([1, 3])
    try:
        pyoracle.rta_run(case, seed=4, nthreads=4)
        n = case["modes"]["omega"].size
        _, val = pyoracle.spectral_raw((2, nb, n))
    finally:
        pyoracle.set_spectral([])
    assert np.array_equal(sp["raw"], val)
    _check_outputs(case, g, sp, 400)
    assert sp["fd_q"].shape == (2, nb, case["modes"]["nq"])
    engine.set_spectral([])
    # production: the same tallies, statistically; the grid kernel tallies them
    engine.set_spectral([1, 3], nomega=400)
    p = engine.rta_run(case["T0"], case["dt"], case["maxtime"], 20000, seed=5)
    sp2 = engine.get_spectral(nb)
    assert np.allclose(sp2["raw"].sum(axis=2), p["gz"][[1, 3]], rtol=1e-9, atol=1e-9)
    engine.set_spectral([])


@pytest.mark.gpu
def test_cli_writes_spectral_csvs(built, tmp_path):
    case = _case()
    synth.write_geometry_xml(str(tmp_path / "beam.xml"), case["geom"])
    synth.write_modes_file(str(tmp_path / "modes.bin"), case["modes"])
    (tmp_path / "input.xml").write_text(
        '<RTA_MC2d>\n  <geometry file="beam.xml"/>\n  <time dt="10" maxtime="200"/>\n'
        '  <material name="synthetic" database="modes.bin" thickness="0.335" T0="300.0"/>\n'
        '  <particles N="2000"/>\n  <engine mode="replay" seed="4"/>\n'
        '  <spectral>\n    <resolution ticks="60"/>\n    <location bin="1"/>\n'
        '    <location bin="3"/>\n  </spectral>\n</RTA_MC2d>\n')
    exe = os.path.join(os.path.dirname(built), "rtamc2d_gpu")
    r = subprocess.run([exe, "input.xml", "1"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    for loc in (1, 3):
        d = np.loadtxt(tmp_path / f"deltaT_omega_{loc}_300K_run_0.csv", delimiter=",")
        assert d.shape == (21, 61) and d[0, 0] == -1.0
        assert np.allclose(d[1:, 0], (np.arange(1, 21) + 0.5) * 10.0)
        for name in ("jx_omega", "jy_omega"):
            assert np.loadtxt(tmp_path / f"{name}_{loc}_300K_run_0.csv", delimiter=",").shape == (21, 61)
        lines = (tmp_path / f"fd_q_{loc}_300K_run_0.csv").read_text().splitlines()
        assert lines[0].startswith("# ") and lines[1].startswith("# ") and lines[2].startswith("# ")
        assert len(lines) == 2 + 20


def _exact(pairs):
    return pairs[..., 0].astype(object) * 2 ** 64 + pairs[..., 1].astype(np.uint64).astype(object)


def test_restatement_steady_spectral_sums_to_the_box_tally():
    """Steady state (process_segment, src/RTA_MC2D.cpp:784-834): the per-mode
    time of a location, summed over modes, is the box's gz to the last
    fixed-point unit, and every segment there is counted once with its sign."""
    case = synth.periodic_case(n_particles=1500)
    n = case["modes"]["omega"].size
    pyoracle.set_spectral([0, 2])
    try:
        r = pyoracle.steady_run(case, (0.0, -0.01), seed=4, nthreads=4)
        ex, val = pyoracle.spectral_raw((2, 1, n))
        cnt = pyoracle.spectral_counts((2, n))
    finally:
        pyoracle.set_spectral([])
    tot = _exact(ex).sum(axis=2)[:, 0]
    gz = _exact(np.asarray(r["exact"]).reshape(-1, 3, 2))[:, 0]
    assert tot[0] == gz[0] and tot[1] == gz[2]
    assert np.abs(cnt).sum() > 0 and np.abs(val).sum() > 0
    # the signed counts of a location follow its per-mode time in sign
    nz = (val[:, 0] != 0) & (cnt != 0)
    assert np.mean(np.sign(val[:, 0][nz]) == np.sign(cnt[nz])) > 0.9


@pytest.mark.gpu
def test_steady_spectral_replay_bit_exact_and_outputs(engine):
    case = synth.periodic_case(n_particles=1500)
    n = case["modes"]["omega"].size
    engine.load_modes(case["modes"])
    engine.load_geometry(case["geom"])
    engine.set_spectral([0, 2], nomega=200)
    g = engine.steady_run(case["T0"], (0.0, -0.01), case["N"], seed=4, mode=btegpu.MODE_REPLAY)
    sp = engine.get_spectral(1)
    engine.set_spectral([])
    pyoracle.set_spectral([0, 2])
    try:
        pyoracle.steady_run(case, (0.0, -0.01), seed=4, nthreads=4)
        _, val = pyoracle.spectral_raw((2, 1, n))
        cnt = pyoracle.spectral_counts((2, n))
    finally:
        pyoracle.set_spectral([])
    assert sp["steady"]
    assert np.array_equal(sp["raw"], val)
    assert np.array_equal(sp["counts"], cnt.astype(float))
    grid, dT, jx, jy, fq = pyoracle.spectral_post(case["modes"], sp["raw"], 200, counts=sp["counts"])
    assert np.allclose(sp["omega"], grid[None, :], rtol=1e-14)
    # the temperature per tick carries the box temperature's own scale
    dT_box = g["temperature"][[0, 2]] - case["T0"]
    for l in range(2):
        scale = dT_box[l] / sp["raw"][l, 0].sum()
        assert np.allclose(sp["dT_omega"][l, 0], scale * dT[l, 0], rtol=1e-9,
                           atol=1e-12 * np.abs(sp["dT_omega"][l]).max())
        for mine, ref in ((sp["jx_omega"][l], jx[l]), (sp["jy_omega"][l], jy[l]), (sp["fd_q"][l], fq[l])):
            i = np.argmax(np.abs(ref))
            c = mine.flat[i] / ref.flat[i]
            assert np.allclose(mine, c * ref, rtol=1e-9, atol=1e-12 * np.abs(mine).max())


@pytest.mark.gpu
def test_cli_writes_steady_spectral_csvs(built, tmp_path):
    case = synth.periodic_case(n_particles=1500)
    synth.write_geometry_xml(str(tmp_path / "beam.xml"), case["geom"])
    synth.write_modes_file(str(tmp_path / "modes.bin"), case["modes"])
    (tmp_path / "input.xml").write_text(
        '<RTA_MC2d>\n  <geometry file="beam.xml"/>\n  <time dt="10" maxtime="200"/>\n'
        f'  <material name="synthetic" database="modes.bin" thickness="{case["geom"]["thickness"]!r}"'
        ' T0="300.0"/>\n'
        '  <particles N="1500"/>\n  <gradient x="0.0" y="-0.01"/>\n'
        '  <engine mode="replay" seed="4"/>\n'
        '  <spectral>\n    <resolution ticks="50"/>\n    <location bin="0"/>\n'
        '    <location bin="2"/>\n  </spectral>\n</RTA_MC2d>\n')
    exe = os.path.join(os.path.dirname(built), "rtamc2d_gpu")
    r = subprocess.run([exe, "input.xml", "1"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    for loc in (0, 2):
        for name in ("steady_deltaT_omega", "steady_jx_omega", "steady_jy_omega"):
            d = np.loadtxt(tmp_path / f"{name}_{loc}_300K_run_0.csv", delimiter=",")
            assert d.shape == (2, 50) and np.all(np.diff(d[0]) > 0)
        lines = (tmp_path / f"steady_fd_q_{loc}_300K_run_0.csv").read_text().splitlines()
        assert len(lines) == 3 and all(ln.startswith("# ") for ln in lines)
        assert len(lines[2][2:].split(",")) == case["modes"]["nq"]
