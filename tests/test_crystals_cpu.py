"""Several crystals joined by diffuse mismatch interfaces (RTAMC2D with boxes
of different materials: change_material_diffuse, src/RTA_MC2D.cpp:871-964,
Diffuse_mismatch_distribution, src/sampling.cpp:437-902), on the CPU:

- the engine's interface tables (host code of libbtegpu.so, through
  bte_interface_table) equal the restatement's entry for entry, whose
  tables tests/test_dmm_pins.py holds to the reference's own code;
- the restatement's multi-crystal run reduces to its one-table run draw for
  draw when there is one crystal;
- with an initial deviation in a closed geometry every particle spends each
  whole bin in some box, across interfaces included;
- a reservoir may inject into its own crystal only."""
import numpy as np
import pytest

import btegpu
import pyoracle
import synth


def _tables():
    return synth.mode_table(8, 3, 3, 300.0, config=100), synth.mode_table(8, 3, 3, 300.0, config=101)


def _same(e, o):
    return all(np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])
               for a, b in zip(e, o))


@pytest.mark.parametrize("normal", [(1.0, 0.0), (0.0, -1.0), (0.6, -0.8)])
def test_engine_interface_tables_equal_the_restatement(built, normal):
    A, B = _tables()
    e = btegpu.interface_table(A, B, normal, 0.335, 300.0)
    o = pyoracle.dmm_table(A, B, normal, 0.335, 300.0)[0]
    assert len(e) == len(o) and _same(e, o)
    assert sum(len(x[0]) for x in e) > 0
    # tables of different sizes (window search over the other crystal)
    A2, B2 = synth.mode_table(12, 3, 3, 300.0, config=100), synth.mode_table(8, 3, 3, 250.0, config=102)
    assert _same(btegpu.interface_table(A2, B2, normal, 0.335, 280.0),
                 pyoracle.dmm_table(A2, B2, normal, 0.335, 280.0)[0])


def test_interface_table_takes_each_crystals_thickness(built):
    """The cell volume of a side enters its table as V thickness / c, so
    B's boxes twice as thick give the table of B with twice its cell
    volume."""
    A, B = _tables()
    B2 = dict(B)
    B2["V"] = 2.0 * B["V"]
    for normal in ((1.0, 0.0), (0.6, -0.8)):
        a = btegpu.interface_table(A, B, normal, (0.335, 0.67), 300.0)
        b = btegpu.interface_table(A, B2, normal, 0.335, 300.0)
        assert _same(a, b)
        assert not _same(a, btegpu.interface_table(A, B, normal, 0.335, 300.0))


def test_restatement_thickness_per_material():
    """Each material's boxes at its own thickness: equal thicknesses repeat
    the run without them draw for draw; another thickness for one crystal
    changes the interface tables (and the boxes' volumes)."""
    A, B = _tables()
    g = _two_crystal_ribbon()
    kw = dict(T0=300.0, dt=10.0, maxtime=100.0, N=3000, seed=4, nthreads=4)
    a = pyoracle.rta_run_multi([A, B], g, **kw)
    b = pyoracle.rta_run_multi([A, B], g, thickness=[0.335, 0.335], **kw)
    assert np.array_equal(a["exact"], b["exact"]) and a["Eeff"] == b["Eeff"]
    c = pyoracle.rta_run_multi([A, B], g, thickness=[0.335, 0.67], **kw)
    # a wall's energy |flux| L t does not depend on t (the flux goes as
    # 1 / t through the unit-cell volume); the interface's tables do
    assert c["Eeff"] == a["Eeff"]
    assert not np.array_equal(a["exact"], c["exact"])


def _two_crystal_ribbon():
    g = synth.ribbon_geometry(200.0, 50.0, 10, T_hot=301.0, T_cold=299.0)
    g["material"] = np.array([0] * 5 + [1] * 5 + [0, 1], dtype=np.int32)
    return g


def _closed_two_crystals():
    """A 200 nm x 50 nm block of 10 x 2 cells closed by void walls, crystal 0
    left of x = 100 nm (initially 0.5 K hot), crystal 1 right of it."""
    g = synth.grid_geometry(200.0, 50.0, 10, 2)
    v = np.asarray(g["vertices"], float).reshape(-1, 4, 2).mean(axis=1)
    g["material"] = (v[:, 0] > 100.0).astype(np.int32)
    g["Tinit"] = np.where(g["material"] == 0, 300.5, 300.0)
    return g


def test_one_crystal_repeats_the_single_table_run():
    A, _ = _tables()
    g = synth.ribbon_geometry(200.0, 50.0, 10)
    g["material"] = np.zeros(12, dtype=np.int32)
    case = {"modes": A, "geom": g, "T0": 300.0, "dt": 10.0, "maxtime": 300.0, "N": 4000}
    a = pyoracle.rta_run(case, seed=5, nthreads=4)
    b = pyoracle.rta_run_multi([A], g, 300.0, 10.0, 300.0, 4000, seed=5, nthreads=4)
    assert np.array_equal(a["gz"], b["gz"]) and a["events"] == b["events"]
    assert np.array_equal(a["temperature"], b["temperature"])
    assert b["interface_hits"] == 0


def test_two_crystals_conserve_particle_time():
    """Without reservoirs no particle is lost: each bin's tally sums to the
    particles times the bin width, while particles cross and bounce back at
    the interface."""
    A, B = _tables()
    g = _closed_two_crystals()
    r = pyoracle.rta_run_multi([A, B], g, 300.0, 10.0, 200.0, 20000, seed=7, nthreads=8,
                               source=btegpu.SOURCE_INITIAL)
    assert r["interface_hits"] > 0 and 0 < r["interface_transmissions"] < r["interface_hits"]
    assert r["absorbed"] == 0
    per_bin = r["gz"].sum(axis=0)
    n = per_bin[0] / 10.0
    assert n > 0 and abs(n - round(n)) < 1e-6
    assert np.allclose(per_bin, per_bin[0], rtol=1e-9, atol=0)


def test_reservoir_injects_into_its_own_crystal_only():
    A, B = _tables()
    g = _two_crystal_ribbon()
    g["material"][10] = 1  # the hot reservoir (touching cell 0 of crystal 0) in crystal 1
    with pytest.raises(btegpu.BteError, match="Injection from material A to B"):
        pyoracle.rta_run_multi([A, B], g, 300.0, 10.0, 100.0, 1000, seed=1, nthreads=2)


# ---------------------------------------------------------------- steady state
# The periodic evolparticle meets a contact between crystals with
# change_material_diffuse and pushes the re-emitted particle into the next
# generation (src/RTA_MC2D.cpp:1672-1689, 1751-1779).


def test_steady_one_crystal_repeats_the_single_table_run():
    A, _ = _tables()
    g = synth.periodic_bar_geometry()
    g["material"] = np.zeros(g["nboxes"], dtype=np.int32)
    a = pyoracle.steady_run({"modes": A, "geom": g, "T0": 300.0, "N": 3000}, (0.0, -0.01), seed=2)
    b = pyoracle.steady_run_multi([A], g, 300.0, (0.0, -0.01), 3000, seed=2)
    assert np.array_equal(a["exact"], b["exact"]) and np.array_equal(a["log"], b["log"])
    assert a["events"] == b["events"] and b["interface_hits"] == 0


def test_steady_two_crystals_bookkeeping_and_threads():
    """Every flight ends one way (an interface re-emission carries the
    particle over like a wall reflection); the run does not depend on the
    thread count."""
    A, B = _tables()
    g = synth.layered_bar_geometry()
    a = pyoracle.steady_run_multi([A, B], g, 300.0, (0.0, -0.01), 3000, seed=3, nthreads=1)
    b = pyoracle.steady_run_multi([A, B], g, 300.0, (0.0, -0.01), 3000, seed=3, nthreads=8)
    assert np.array_equal(a["exact"], b["exact"]) and a["generations"] == b["generations"]
    assert 0 < a["interface_transmissions"] < a["interface_hits"]
    assert a["events"] == a["scattered"] + a["absorbed"] + a["lost"] + a["wall_hits"] + a["interface_hits"]
    assert a["events"] == 3000 + a["births"] + a["interface_hits"]


def test_steady_two_crystals_step_at_the_interface_and_flux_continuity():
    """The interface resists: the temperature steps between strips 4 and 5
    while the flux along the bar stays the same on both sides."""
    A, B = _tables()
    g = synth.layered_bar_geometry()
    R = [pyoracle.steady_run_multi([A, B], g, 300.0, (0.0, -0.01), 4000, seed=10 + i, nthreads=8)
         for i in range(4)]
    T = np.mean([r["temperature"][:10] for r in R], axis=0)
    assert T[4] - T[5] > 3.0 * max(abs(T[3] - T[4]), abs(T[5] - T[6]))
    jy = np.array([[r["jy"][:5].mean(), r["jy"][5:10].mean()] for r in R])
    d = jy[:, 0] - jy[:, 1]
    assert abs(d.mean()) < 4.5 * d.std(ddof=1) / np.sqrt(len(d)) + 1e-3 * abs(jy.mean())
