"""GPU parity of the periodic / gradient steady state (bte_steady_run,
src/RTA_MC2D.cpp:2544-2842) against the restatement.

Replay mode must reproduce every generation bit for bit: identical 128-bit
tallies, convergence table and counters.  Production mode (Philox streams,
alias tables, FP64 atomics) must agree with the restatement within 4.5 sigma
over replicas and give the bulk RTA conductivity in an infinite medium."""
import os
import subprocess

import numpy as np
import pytest

import btegpu
import pyoracle
import synth

pytestmark = pytest.mark.gpu


def _load(engine, case):
    engine.load_modes(case["modes"])
    engine.load_geometry(case["geom"])


def _cell_case(N=20000, even=False):
    m = synth.mode_table(9, 3, 3, 300.0, config=100, even=True) if even else \
        synth.mode_table(8, 3, 3, 300.0, config=100)
    return {"modes": m, "geom": synth.periodic_cell_geometry(40.0, 40.0, 2, 2), "T0": 300.0, "N": N}


@pytest.mark.parametrize("which,grad", [("bar", (0.0, -0.01)), ("cell", (-0.01, 0.004))])
def test_steady_replay_bit_exact(engine, which, grad):
    case = synth.periodic_case(n_particles=3000) if which == "bar" else _cell_case(4000)
    _load(engine, case)
    g = engine.steady_run(case["T0"], grad, case["N"], seed=6, mode=btegpu.MODE_REPLAY)
    o = pyoracle.steady_run(case, grad, seed=6)
    assert g["generations"] == o["generations"] > 1
    assert np.array_equal(g["exact"], o["exact"])
    assert np.array_equal(g["log"], o["log"])
    for k in ("events", "wall_hits", "crossings", "absorbed", "translations", "scattered",
              "births", "lost"):
        assert g[k] == o[k], k
    assert g["Eeff"] == o["Eeff"]
    assert np.abs(g["temperature"] - o["temperature"]).max() <= 1e-12 * 300.0
    assert np.array_equal(g["jx"], o["jx"]) and np.array_equal(g["jy"], o["jy"])


@pytest.mark.parametrize("flags", [0, btegpu.FLAG_GENERAL], ids=["polygon", "general"])
def test_steady_production_agrees_with_restatement(engine, flags):
    """The convex-polygon kernel (default) and the evolparticle-faithful
    kernel both agree with the restatement."""
    case = synth.periodic_case(n_particles=4000)
    _load(engine, case)
    R = 6

    def obs(r):
        return np.concatenate([r["temperature"][:10], [r["jy"][:10].mean() * 1e-8]])

    prod = np.array([obs(engine.steady_run(300.0, (0.0, -0.01), case["N"], seed=40 + i, flags=flags))
                     for i in range(R)])
    orc = np.array([obs(pyoracle.steady_run(case, (0.0, -0.01), seed=60 + i)) for i in range(R)])
    d = prod.mean(0) - orc.mean(0)
    se = np.sqrt(prod.var(0, ddof=1) / R + orc.var(0, ddof=1) / R)
    z = np.abs(d) / np.maximum(se, 1e-300)
    assert z.max() < 4.5, (z, prod.mean(0), orc.mean(0))


@pytest.mark.parametrize("flags", [0, btegpu.FLAG_GENERAL], ids=["polygon", "general"])
def test_steady_production_bulk_kappa(engine, flags):
    case = _cell_case(200000, even=True)
    _load(engine, case)
    K = synth.kappa_rta(case["modes"], 300.0)[0, 0]
    ks = np.array([-engine.steady_run(300.0, (-0.01, 0.0), case["N"], seed=90 + i, flags=flags)["jx"][:4].mean()
                   / (-0.01e9) for i in range(6)])
    se = ks.std(ddof=1) / np.sqrt(len(ks))
    assert abs(ks.mean() - K) < 4.5 * se, (ks.mean(), se, K)


def test_steady_specular_replay_bit_exact_and_production_kappa(engine):
    """Specular fraction p = 0.5: replay matches the restatement bit for bit;
    production gives the analytic1d in-plane film conductivity."""
    case = {"modes": synth.mode_table(9, 3, 3, 300.0, config=100, even=True),
            "geom": synth.periodic_ribbon_geometry(40.0, 100.0, 2, 2), "T0": 300.0, "N": 3000}
    _load(engine, case)
    g = engine.steady_run(300.0, (-0.01, 0.0), 3000, seed=8, mode=btegpu.MODE_REPLAY, specularity=0.5)
    o = pyoracle.steady_run(case, (-0.01, 0.0), N=3000, seed=8, specularity=0.5)
    assert np.array_equal(g["exact"], o["exact"]) and np.array_equal(g["log"], o["log"])
    K = synth.kappa_ribbon(case["modes"], 300.0, 100.0, p=0.5)
    ks = np.array([-engine.steady_run(300.0, (-0.01, 0.0), 200000, seed=140 + i, specularity=0.5)["jx"][:4].mean()
                   / (-0.01e9) for i in range(6)])
    se = ks.std(ddof=1) / np.sqrt(len(ks))
    assert abs(ks.mean() - K) < 4.5 * se, (ks.mean(), se, K)


@pytest.mark.parametrize("width", [50.0, 500.0])
def test_steady_production_ribbon_kappa(engine, width):
    """Diffuse-wall nanoribbon (scale_tau_nanoribbon, src/nanos.cpp:77-112)."""
    case = {"modes": synth.mode_table(9, 3, 3, 300.0, config=100, even=True),
            "geom": synth.periodic_ribbon_geometry(40.0, width, 2, 2), "T0": 300.0, "N": 200000}
    _load(engine, case)
    K = synth.kappa_ribbon(case["modes"], 300.0, width)
    ks = np.array([-engine.steady_run(300.0, (-0.01, 0.0), case["N"], seed=120 + i)["jx"][:4].mean()
                   / (-0.01e9) for i in range(6)])
    se = ks.std(ddof=1) / np.sqrt(len(ks))
    assert abs(ks.mean() - K) < 4.5 * se, (ks.mean(), se, K)


def test_steady_cli(built, tmp_path):
    """rtamc2d_gpu runs the steady branch for <gradient> and writes
    steady_<T0>K_run_<i>.csv (rows: T, jx, jy per box)."""
    case = synth.periodic_case(n_particles=2000)
    synth.write_geometry_xml(str(tmp_path / "beam.xml"), case["geom"])
    synth.write_modes_file(str(tmp_path / "modes.bin"), case["modes"])
    (tmp_path / "input.xml").write_text(
        '<RTA_MC2d>\n  <geometry file="beam.xml"/>\n  <time dt="10" maxtime="200"/>\n'
        f'  <material name="synthetic" database="modes.bin" thickness="{case["geom"]["thickness"]!r}"'
        ' T0="300.0"/>\n'
        '  <particles N="2000"/>\n  <gradient x="0.0" y="-0.01"/>\n'
        '  <engine mode="replay" seed="5"/>\n</RTA_MC2d>\n')
    exe = os.path.join(os.path.dirname(built), "rtamc2d_gpu")
    r = subprocess.run([exe, "input.xml", "4"], cwd=tmp_path, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    assert "PERIODIC CASE" in r.stdout
    S = np.loadtxt(tmp_path / "steady_300K_run_0.csv", delimiter=",")
    assert S.shape == (3, case["geom"]["nboxes"])
    o = pyoracle.steady_run(case, (0.0, -0.01), seed=5)
    assert np.allclose(S[0], o["temperature"], rtol=0, atol=6e-4)
    assert np.allclose(S[2], o["jy"], rtol=1e-5, atol=0)


@pytest.mark.parametrize("which", ["bar", "cell"])
def test_steady_polygon_walk_repeats_faithful_kernel(engine, which):
    """The polygon walk draws from each slot's stream in the order the
    evolparticle-faithful kernel does, and its translate skips only
    neighbours the full tests reject: away from corners (a set of measure
    zero) both kernels follow the same trajectories, so their counters agree
    exactly and their tallies to FP64 rounding of the atomics' order."""
    case = synth.periodic_case(n_particles=20000) if which == "bar" else _cell_case(20000)
    grad = (0.0, -0.01) if which == "bar" else (-0.01, 0.004)
    _load(engine, case)
    a = engine.steady_run(300.0, grad, case["N"], seed=17, max_generations=20)
    b = engine.steady_run(300.0, grad, case["N"], seed=17, max_generations=20, flags=btegpu.FLAG_GENERAL)
    for k in ("generations", "events", "translations", "wall_hits", "absorbed", "scattered"):
        assert a[k] == b[k], (k, a[k], b[k])
    # the faithful kernel also counts the step into a reservoir as a crossing
    assert a["crossings"] + a["absorbed"] == b["crossings"]
    assert a["translations"] > 0
    for k in ("gz", "gz_jx", "gz_jy"):
        scale = np.abs(b[k]).max()
        assert np.abs(a[k] - b[k]).max() <= 1e-9 * scale, k
