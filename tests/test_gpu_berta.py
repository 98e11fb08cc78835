"""GPU tests of the beyond-RTA (beRTAMC2D) step loop against the CPU
restatement: per-step energy density and flux agree over independent
replicas (parity_stats: the count of observables above 3 sigma at a 1 %
false-alarm rate, and 4.5 sigma for the family), for propagator scattering
(with sign branching) and for the RTA alternative.  The device loop's
particle order follows its warps' claims, so its runs are not repeatable
draw for draw; every replica is an independent sample."""
import numpy as np
import pytest

import btegpu
import pyoracle
import synth
from parity_stats import check

pytestmark = pytest.mark.gpu


def _case():
    m = synth.mode_table(8, 3, 3, 300.0, config=100)
    g = synth.ribbon_geometry(200.0, 50.0, 5)
    P = synth.propagator(m)
    return m, g, P


def _obs(r):
    # late-time energy density of the 5 interior boxes and the mean x flux
    ed = r["ed"][-10:, :5].mean(axis=0) * 1e-6
    fx = r["flux"][-10:, :5, 0].mean() * 1e-8
    return np.concatenate([ed, [fx]])


@pytest.mark.parametrize("rta", [False, True])
def test_berta_agrees_with_restatement(engine, rta):
    m, g, P = _case()
    engine.load_modes(m)
    engine.load_geometry(g)
    engine.load_propagator(P)
    R = 8
    kw = dict(dt=1.0, maxtime=40.0, Eeff=2e-23, rta=rta)
    gpu = np.array([_obs(engine.berta_run(seed=10 + i, **kw)) for i in range(R)])
    cpu = np.array([_obs(pyoracle.berta_run(m, g, P, seed=20 + i, **kw)) for i in range(R)])
    check(gpu, cpu, [f"ed_box{i}" for i in range(5)] + ["flux_x"], f"beRTA ribbon rta={rta}")


def test_berta_counts_and_branching(engine):
    m, g, P = _case()
    engine.load_modes(m)
    engine.load_geometry(g)
    engine.load_propagator(P)
    r = engine.berta_run(1.0, 20.0, 2e-23, seed=3, histogram=True)
    o = pyoracle.berta_run(m, g, P, 1.0, 20.0, 2e-23, seed=3)
    assert r["nsteps"] == o["nsteps"] == 21
    assert r["branchings"] > 0 and r["particle_steps"] > 0
    # particle numbers follow the same growth within a few percent
    assert abs(r["nparticles"][-1] - o["nparticles"][-1]) < 0.1 * o["nparticles"][-1]
    # the histogram of the last step sums to the signed particle count
    assert r["H"].sum() != 0


def test_bertamc2d_cli_writes_table_and_frames(built, tmp_path):
    import os
    import subprocess
    m, g, P = _case()
    synth.write_geometry_xml(str(tmp_path / "beam.xml"), g)
    synth.write_modes_file(str(tmp_path / "modes.bin"), m)
    synth.write_propagator(str(tmp_path / "p.P.eigen.bin"), P)
    (tmp_path / "input.xml").write_text(
        '<beRTAMC2D>\n  <geometry file="beam.xml"/>\n  <time dt="1.0" maxtime="10"/>\n'
        '  <material name="synthetic" database="modes.bin" thickness="0.335">\n'
        '    <propagator T="300" file="p.P.eigen.bin"/>\n  </material>\n'
        '  <Eeff Ed="2e-23"/>\n</beRTAMC2D>\n')
    exe = os.path.join(os.path.dirname(built), "bertamc2d_gpu")
    r = subprocess.run([exe, "input.xml", "4"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    rows = [ln for ln in r.stdout.splitlines() if ln and ln[0].isdigit()]
    assert len(rows) == 11                      # steps 1..11 for time <= 10
    assert len(rows[0].split("\t")) >= 3 + 3 * g["nboxes"]
    data = (tmp_path / "properties.msgpack.bin").read_bytes()
    assert data.endswith(b"0#")
    assert len(btegpu.split_frames(data)) == 11
    assert "#TIME report:" in r.stdout and " *scattering : " in r.stdout


def _bar_obs(r):
    # late-time energy density of the 10 strips and the mean y flux
    ed = r["ed"][-10:, :10].mean(axis=0) * 1e-6
    fy = r["flux"][-10:, :10, 1].mean() * 1e-8
    return np.concatenate([ed, [fy]])


@pytest.mark.parametrize("rta", [False, True])
def test_berta_periodic_bar_agrees_with_restatement(engine, rta):
    """Boxes that are not a grid, with periodic boxes (the layout of the
    reference's example_bar): the convex-box advection with translations."""
    m = synth.mode_table(8, 3, 3, 300.0, config=100)
    g = synth.periodic_bar_geometry()
    P = synth.propagator(m)
    engine.load_modes(m)
    engine.load_geometry(g)
    engine.load_propagator(P)
    R = 8
    kw = dict(dt=1.0, maxtime=40.0, Eeff=1e-23, rta=rta)
    gpu = np.array([_bar_obs(engine.berta_run(seed=10 + i, **kw)) for i in range(R)])
    cpu = np.array([_bar_obs(pyoracle.berta_run(m, g, P, seed=20 + i, **kw)) for i in range(R)])
    check(gpu, cpu, [f"ed_strip{i}" for i in range(10)] + ["flux_y"], f"beRTA periodic bar rta={rta}")


def test_berta_gradient_source_gives_bulk_kappa(engine):
    """Homogeneous <gradient> source term in an infinite medium (periodic
    boxes on all sides), RTA scattering: the flux follows the bulk
    conductivity with the loop's discrete lifetime at every step."""
    from test_berta_gradient_cpu import DT, GRAD, check_bulk
    m = synth.mode_table(9, 3, 3, 300.0, config=100, even=True)
    g = synth.periodic_cell_geometry(40.0, 40.0, 2, 2)
    engine.load_modes(m)
    engine.load_geometry(g)
    runs = [engine.berta_run(DT, 800.0, 1e-23, seed=40 + k, rta=True, gradient=GRAD) for k in range(10)]
    check_bulk(runs, m, 200, 4.5)


def test_berta_gradient_with_propagator_agrees_with_restatement(engine):
    """The gradient source with propagator scattering (sign branching) on
    the periodic block: energy density and flux against the restatement."""
    m = synth.mode_table(8, 3, 3, 300.0, config=100)
    g = synth.periodic_cell_geometry(40.0, 40.0, 2, 2)
    P = synth.propagator(m)
    engine.load_modes(m)
    engine.load_geometry(g)
    engine.load_propagator(P)
    R = 12
    kw = dict(dt=1.0, maxtime=30.0, Eeff=1e-23, gradient=(0.01, 0.005))

    def obs(r):
        f = r["flux"][-10:, :4].mean(axis=(0, 1)) * 1e-8
        return np.concatenate([f, [r["nparticles"][-1] * 1e-3]])
    gpu = np.array([obs(engine.berta_run(seed=10 + i, **kw)) for i in range(R)])
    cpu = np.array([obs(pyoracle.berta_run(m, g, P, seed=20 + i, **kw)) for i in range(R)])
    check(gpu, cpu, ["flux_x", "flux_y", "particles_end"], "beRTA gradient with propagator")


def test_bertamc2d_cli_gradient_on_periodic_block(built, tmp_path):
    import os
    import subprocess
    m = synth.mode_table(9, 3, 3, 300.0, config=100, even=True)
    g = synth.periodic_cell_geometry(40.0, 40.0, 2, 2)
    synth.write_geometry_xml(str(tmp_path / "block.xml"), g)
    synth.write_modes_file(str(tmp_path / "modes.bin"), m)
    (tmp_path / "input.xml").write_text(
        '<beRTAMC2D>\n  <geometry file="block.xml"/>\n  <time dt="1.0" maxtime="20"/>\n'
        '  <material name="synthetic" database="modes.bin" thickness="0.335"/>\n'
        '  <RTA/>\n  <gradient x="0.01" y="0"/>\n  <Eeff Ed="1e-23"/>\n</beRTAMC2D>\n')
    exe = os.path.join(os.path.dirname(built), "bertamc2d_gpu")
    r = subprocess.run([exe, "input.xml", "4"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    rows = [ln.split("\t") for ln in r.stdout.splitlines() if ln and ln[0].isdigit()]
    assert len(rows) == 21
    assert int(rows[-1][2]) > 0                 # particles from the source term


def test_dist_reader_on_bertamc2d_frames(built, tmp_path):
    """bertamc2d_gpu writes the frames, dist_reader_gpu reads them back: the
    distribution at the dump times against the restatement of dist_reader."""
    import os
    import subprocess
    m, g, P = _case()
    synth.write_geometry_xml(str(tmp_path / "beam.xml"), g)
    synth.write_modes_file(str(tmp_path / "modes.bin"), m)
    synth.write_propagator(str(tmp_path / "p.P.eigen.bin"), P)
    (tmp_path / "input.xml").write_text(
        '<beRTAMC2D>\n  <geometry file="beam.xml"/>\n  <time dt="1.0" maxtime="10"/>\n'
        '  <material name="synthetic" database="modes.bin" thickness="0.335">\n'
        '    <propagator T="300" file="p.P.eigen.bin"/>\n  </material>\n'
        '  <Eeff Ed="2e-24"/>\n'
        '  <spectral>\n    <resolution ticks="30"/>\n    <location bin="0"/>\n'
        '    <location bin="2"/>\n    <time t="5"/>\n    <time t="9"/>\n  </spectral>\n</beRTAMC2D>\n')
    d = os.path.dirname(built)
    r = subprocess.run([os.path.join(d, "bertamc2d_gpu"), "input.xml", "4"], cwd=tmp_path,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([os.path.join(d, "dist_reader_gpu"), "input.xml", "properties.msgpack.bin"],
                       cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    frames = [pyoracle.decode_berta_frame(f)
              for f in btegpu.split_frames((tmp_path / "properties.msgpack.bin").read_bytes())]
    dumps = [f for f in frames if f[0] in (5.0, 9.0)]
    assert len(dumps) == 2
    area = [200.0 / 5 * 50.0] * 5
    assert sum(len(h[3][b]) for h in dumps for b in (0, 2)) > 0
    for b in (0, 2):
        dT = np.loadtxt(tmp_path / f"deltaT_omega_{b}.csv", delimiter=",")
        assert dT.shape == (3, 31)
        for row, (t, E, T, hists) in enumerate(dumps, start=1):
            assert dT[row, 0] == t
            _, out = pyoracle.dist_reader_restated(m, area, 0.335, [0, 2], 30, hists, T, E)
            ref = out[b][0]
            assert np.allclose(dT[row, 1:], ref, rtol=2e-5, atol=1e-5 * np.abs(ref).max())


def test_berta_interpolated_propagator_agrees_with_restatement(engine):
    """Propagators tabulated at 290, 305 and 320 K, a run at 300 K: the
    engine interpolates the signed CDFs (lirp, between 305 and 320 as the
    reference picks them, so extrapolating) and draws from them by the
    reference's lower_bound, whose |values| are not monotone in most
    columns; energy density and flux against the restatement."""
    m, g, _ = _case()
    tab = {T: synth.propagator(m, T=T) for T in (290.0, 305.0, 320.0)}
    engine.load_modes(m)
    engine.load_geometry(g)
    for T, P in tab.items():
        engine.load_propagator(P, T)
    R = 8
    kw = dict(dt=1.0, maxtime=30.0, Eeff=2e-23, T0=300.0)
    gpu = np.array([_obs(engine.berta_run(seed=10 + i, **kw)) for i in range(R)])
    cpu = np.array([_obs(pyoracle.berta_run(m, g, tab, seed=20 + i, **kw)) for i in range(R)])
    check(gpu, cpu, [f"ed_box{i}" for i in range(5)] + ["flux_x"], "beRTA interpolated propagator")
    # with 290 and 305 only, 300 K has one tabulated temperature above it
    e2 = btegpu.Engine(0)
    try:
        e2.load_modes(m)
        e2.load_geometry(g)
        e2.load_propagator(tab[290.0], 290.0)
        e2.load_propagator(tab[305.0], 305.0)
        with pytest.raises(btegpu.BteError, match="Extrapolation"):
            e2.berta_run(1.0, 5.0, 2e-23, T0=300.0)
    finally:
        e2.close()


def test_berta_box_temperatures_agree_with_restatement(engine):
    """Cells at 299.6 ... 300.4 K with propagators tabulated at 299.0,
    300.0, 300.2, 300.6 and 301.0 K: the cells at 300.0 and 300.2 K take
    their tabulated propagators (one alias table each), the other three
    interpolate (lirp drawn on the fly, between the two tabulated
    temperatures above them); the default source term injects the Teq
    profile's least-squares gradients.  Energy density and flux against
    the restatement."""
    from parity_stats import check
    m, g, _ = _case()
    g["Teq"][:5] = [299.6, 299.8, 300.0, 300.2, 300.4]
    g["Tinit"][:5] = g["Teq"][:5]
    tab = {T: synth.propagator(m, T=T) for T in (299.0, 300.0, 300.2, 300.6, 301.0)}
    engine.load_modes(m)
    engine.load_geometry(g)
    for T, P in tab.items():
        engine.load_propagator(P, T)
    R = 6
    kw = dict(dt=1.0, maxtime=30.0, Eeff=2e-23, T0=300.0)
    names = [f"ed_cell{i}" for i in range(5)] + ["flux_x"]
    gpu = np.array([_obs(engine.berta_run(seed=10 + i, **kw)) for i in range(R)])
    cpu = np.array([_obs(pyoracle.berta_run(m, g, tab, seed=20 + i, **kw)) for i in range(R)])
    check(gpu, cpu, names, "beRTA box temperatures")
    # RTA scattering has the mode table's rates at T0 only
    with pytest.raises(btegpu.BteError, match="Teq = T0"):
        engine.berta_run(1.0, 5.0, 2e-23, T0=300.0, rta=True)


def test_berta_phase_times(engine, built, tmp_path):
    """The reference's timer buckets: device time per step phase, which add
    up to no more than the device time of the loop; the CLI prints the
    reference's time report."""
    m, g, P = _case()
    engine.load_modes(m)
    engine.load_geometry(g)
    engine.load_propagator(P)
    r = engine.berta_run(1.0, 20.0, 2e-23, seed=3)
    ph = r["phase_ms"]
    for k in ("advection", "generators", "scattering", "histogram", "properties", "read_data"):
        assert ph[k] > 0.0, k
    device = sum(ph[k] for k in ("advection", "cancelling", "generators", "histogram", "properties", "scattering"))
    assert device <= r["kernel_ms"] * 1.01 + 0.1
    assert ph["saving"] == 0.0  # no on_step hook here



def test_berta_capacity_overflow_is_an_error_and_the_context_stays_usable(engine):
    """A population larger than the particle buffers stops with
    BTE_ERR_LIMIT at the end of the run (the step kernels read no place
    beyond the buffers and drop what does not fit); the next run on the
    same context with room enough is unaffected."""
    m, g, P = _case()
    engine.load_modes(m)
    engine.load_geometry(g)
    engine.load_propagator(P)
    with pytest.raises(btegpu.BteError, match="capacity"):
        engine.berta_run(1.0, 20.0, 2e-23, seed=3, capacity=300)
    r = engine.berta_run(1.0, 20.0, 2e-23, seed=3)
    assert r["nparticles"][-1] > 300 and np.isfinite(r["ed"]).all()
