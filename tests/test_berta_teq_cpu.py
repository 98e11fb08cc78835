"""Boxes at different Teq in the beyond-RTA loop, in the restatement:

- calculate_gradientT (src/geometry_2d.cpp:524-575): per box, the
  minimum-norm least-squares gradient of Teq over its neighbours that are
  neither reservoirs nor periodic (contacts include boxes that touch at a
  corner), checked against numpy's lstsq;
- each box scatters with the propagator of its own Teq (Scattering,
  src/beyondRTA_MC2d.cpp:1130-1165): tabulated, or lirp between the two
  tabulated temperatures above it;
- RTA scattering has rates at T0 only and refuses other temperatures;
- with the default source term (no <gradient>) a Teq profile makes the
  gradient source inject particles."""
import numpy as np
import pytest

import btegpu
import pyoracle
import synth


def _touching(geom):
    """Contacts of axis-aligned rectangles: closed rectangles that meet."""
    v = np.asarray(geom["vertices"], float).reshape(-1, 4, 2)
    lo, hi = v.min(axis=1), v.max(axis=1)
    n = len(v)
    out = []
    for a in range(n):
        nb = [b for b in range(n) if b != a
              and lo[b, 0] <= hi[a, 0] + 1e-9 and lo[a, 0] <= hi[b, 0] + 1e-9
              and lo[b, 1] <= hi[a, 1] + 1e-9 and lo[a, 1] <= hi[b, 1] + 1e-9]
        out.append(nb)
    return out, 0.5 * (lo + hi)


def _lstsq_gradients(geom):
    nbs, c = _touching(geom)
    res = np.asarray(geom["reservoir"]) != 0
    T = np.asarray(geom["Teq"], float)
    out = np.zeros((len(nbs), 2))
    for a, nb in enumerate(nbs):
        if res[a]:
            continue
        nb = [b for b in nb if not res[b]]
        if not nb:
            continue
        H = c[nb] - c[a]
        d = T[nb] - T[a]
        out[a] = np.linalg.lstsq(H, d, rcond=None)[0]
    return out


def test_gradientT_is_the_min_norm_least_squares_gradient():
    m = synth.mode_table(8, 3, 3, 300.0, config=100)
    rng = np.random.default_rng(4)
    # a grid with a pore: 4 to 8 neighbours per cell, corners included
    g = synth.grid_geometry(400.0, 200.0, 20, 10, pore_center=(200.0, 100.0), pore_diameter=80.0)
    g["Teq"] = 300.0 + rng.normal(0.0, 0.5, g["nboxes"])
    got = pyoracle.gradient_T(m, g)
    ref = _lstsq_gradients(g)
    assert np.allclose(got, ref, rtol=1e-10, atol=1e-13), np.abs(got - ref).max()
    # a linear field is reproduced exactly (to rounding) in every cell
    v = np.asarray(g["vertices"], float).reshape(-1, 4, 2).mean(axis=1)
    g["Teq"] = 300.0 + 0.003 * v[:, 0] - 0.002 * v[:, 1]
    got = pyoracle.gradient_T(m, g)
    assert np.allclose(got, [0.003, -0.002], rtol=1e-9, atol=1e-12)


def test_gradientT_of_collinear_neighbours_has_no_normal_component():
    """A ribbon's cells see their neighbours along x only: rank one, the
    minimum-norm solution has no y component; reservoirs take no part."""
    m = synth.mode_table(8, 3, 3, 300.0, config=100)
    g = synth.ribbon_geometry(200.0, 50.0, 5)
    g["Teq"][:5] = [299.6, 299.8, 300.1, 300.2, 300.6]
    got = pyoracle.gradient_T(m, g)
    ref = _lstsq_gradients(g)
    assert np.allclose(got, ref, rtol=1e-12, atol=1e-15)
    assert np.all(got[:, 1] == 0.0) and np.all(got[5:] == 0.0)
    # the end cells have one neighbour each
    assert np.isclose(got[0, 0], 0.2 / 40.0) and np.isclose(got[4, 0], 0.4 / 40.0)


def _teq_case():
    m = synth.mode_table(8, 3, 3, 300.0, config=100)
    g = synth.ribbon_geometry(200.0, 50.0, 5)
    g["Teq"][:5] = [299.6, 299.8, 300.0, 300.2, 300.4]
    g["Tinit"][:5] = g["Teq"][:5]
    return m, g


KW = dict(dt=1.0, maxtime=8.0, Eeff=2e-23, seed=5)


def test_each_box_scatters_with_its_own_table():
    """Every box's table is the same matrix whether it is tabulated at the
    box's Teq or interpolated between two equal matrices above it (the
    lowest tabulated temperature must not be above Teq; its matrix takes no
    part): the runs are identical draw for draw."""
    m, g = _teq_case()
    P = synth.propagator(m)
    a = pyoracle.berta_run(m, g, {T: P for T in g["Teq"][:5]}, **KW)
    b = pyoracle.berta_run(m, g, {299.0: np.eye(P.shape[0]), 310.0: P, 320.0: P}, **KW)
    assert a["nparticles"].max() > 0
    assert np.array_equal(a["ed"], b["ed"]) and np.array_equal(a["H"], b["H"])
    # another matrix in one box changes the run
    c = pyoracle.berta_run(m, g, {**{T: P for T in g["Teq"][:5]}, 300.0: synth.propagator(m, flip=0.1)}, **KW)
    assert not np.array_equal(a["H"], c["H"])


def test_box_temperature_outside_the_table_is_refused():
    m, g = _teq_case()
    P = synth.propagator(m)
    # 300.4 K has only one tabulated temperature above it
    with pytest.raises(btegpu.BteError, match="Extrapolation"):
        pyoracle.berta_run(m, g, {299.0: P, 300.0: P, 300.5: P}, **KW)


def test_rta_scattering_needs_teq_t0():
    m, g = _teq_case()
    with pytest.raises(btegpu.BteError, match="Teq = T0"):
        pyoracle.berta_run(m, g, None, rta=True, **KW)


def test_teq_profile_drives_the_gradient_source():
    """Reservoirs at the neighbouring cells' Teq and no initial deviation:
    only the gradient source of the Teq profile injects particles, and it
    stops when the profile is flat."""
    m, g = _teq_case()
    g["Teq"][5], g["Teq"][6] = g["Teq"][0], g["Teq"][4]   # the left reservoir touches cell 0, the right one cell 4
    g["Tinit"][:] = g["Teq"]
    P = synth.propagator(m)
    tab = {299.0: P, 310.0: P, 320.0: P}
    r = pyoracle.berta_run(m, g, tab, **KW)
    flat = dict(g)
    flat["Teq"] = np.full_like(g["Teq"], 300.0)
    flat["Tinit"] = flat["Teq"].copy()
    r0 = pyoracle.berta_run(m, flat, tab, **KW)
    assert r0["nparticles"].max() == 0
    assert r["nparticles"][-1] > 0
