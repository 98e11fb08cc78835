"""CPU tests of the periodic / gradient steady state (src/RTA_MC2D.cpp:
2544-2842) in the restatement: determinism over threads, bookkeeping of the
generations, and the physics check that pins it independently of the
reference: in an infinite medium (a block closed by periodic boxes on all
sides) the steady flux under a gradient is the bulk RTA conductivity,
J = -kappa grad T with kappa = 1e21 kB / (nq V) sum C v v tau, and in a
ribbon with diffuse walls it is the nanoribbon conductivity of the
reference's analytic model."""
import numpy as np
import pytest

import pyoracle
import synth


def _even_modes():
    # mirror-symmetric table: the gradient source's alternating signs then
    # sample the + and - halves with equal weight, as the analytic forms assume
    return synth.mode_table(9, 3, 3, 300.0, config=100, even=True)


def _cell_case(N=20000):
    return {"modes": _even_modes(),
            "geom": synth.periodic_cell_geometry(40.0, 40.0, 2, 2), "T0": 300.0, "N": N}


def test_steady_restatement_independent_of_threads():
    case = synth.periodic_case(n_particles=1500)
    a = pyoracle.steady_run(case, (0.0, -0.01), seed=4, nthreads=1)
    b = pyoracle.steady_run(case, (0.0, -0.01), seed=4, nthreads=8)
    assert np.array_equal(a["exact"], b["exact"])
    assert np.array_equal(a["log"], b["log"])
    for k in ("generations", "events", "crossings", "absorbed", "translations", "births"):
        assert a[k] == b[k], k


def test_steady_generation_bookkeeping():
    case = synth.periodic_case(n_particles=3000)
    r = pyoracle.steady_run(case, (0.0, -0.01), seed=2)
    assert r["generations"] == len(r["log"]) and r["converged"] == 0
    assert r["log"][-1, 0] == 0            # the loop ends when no particle is left
    assert r["log"][0, 1] == 1.0           # first generation: relative change 1
    # every flight ends in exactly one way; none is reflected in the closed bar
    assert r["events"] == r["scattered"] + r["absorbed"] + r["lost"] + r["wall_hits"]
    assert r["wall_hits"] == 0 and r["translations"] > 0
    assert r["births"] <= r["scattered"]
    assert r["events"] == 3000 + r["births"]


def test_steady_convergence_criterion_stops_early():
    case = synth.periodic_case(n_particles=3000)
    full = pyoracle.steady_run(case, (0.0, -0.01), seed=2)
    early = pyoracle.steady_run(case, (0.0, -0.01), seed=2, eps_energy=0.05, eps_flux=0.05)
    assert early["converged"] == 1 and early["generations"] < full["generations"]
    last = early["log"][-1]
    assert last[1] < 0.05 and last[3] < 0.05   # gradient along y: rgz and rjy


@pytest.mark.parametrize("axis,grad", [(0, (-0.01, 0.0)), (1, (0.0, -0.02))])
def test_steady_infinite_medium_gives_bulk_rta_kappa(axis, grad):
    case = _cell_case()
    K = synth.kappa_rta(case["modes"], 300.0)[axis, axis]
    ks = []
    for seed in range(10):
        r = pyoracle.steady_run(case, grad, seed=300 + seed)
        J = (r["jx"] if axis == 0 else r["jy"])[:4].mean()
        ks.append(-J / (grad[axis] * 1e9))
    ks = np.array(ks)
    se = ks.std(ddof=1) / np.sqrt(len(ks))
    assert abs(ks.mean() - K) < 4.0 * se + 1e-9 * K, (ks.mean(), se, K)
    assert se < 0.05 * K


@pytest.mark.parametrize("width", [50.0, 200.0])
def test_steady_ribbon_gives_diffuse_wall_kappa(width):
    """A ribbon periodic along x with void walls: kappa_xx equals the
    nanoribbon RTA conductivity of scale_tau_nanoribbon (src/nanos.cpp:77-112)."""
    case = {"modes": _even_modes(), "geom": synth.periodic_ribbon_geometry(40.0, width, 2, 2),
            "T0": 300.0, "N": 20000}
    K = synth.kappa_ribbon(case["modes"], 300.0, width)
    ks = np.array([-pyoracle.steady_run(case, (-0.01, 0.0), seed=10 + s)["jx"][:4].mean() / (-0.01e9)
                   for s in range(8)])
    se = ks.std(ddof=1) / np.sqrt(len(ks))
    assert abs(ks.mean() - K) < 4.0 * se, (ks.mean(), se, K)
    assert K < synth.kappa_rta(case["modes"], 300.0)[0, 0]


@pytest.mark.parametrize("p", [0.5, 0.9])
def test_steady_specular_ribbon_gives_fuchs_sondheimer_kappa(p):
    """Walls that reflect specularly with probability p: kappa_xx equals the
    in-plane film conductivity of the reference's analytic1d
    (src/analytic1d.cpp:244-273) on the same modes."""
    case = {"modes": _even_modes(), "geom": synth.periodic_ribbon_geometry(40.0, 100.0, 2, 2),
            "T0": 300.0, "N": 20000}
    K = synth.kappa_ribbon(case["modes"], 300.0, 100.0, p=p)
    ks = np.array([-pyoracle.steady_run(case, (-0.01, 0.0), seed=20 + s, specularity=p)["jx"][:4].mean()
                   / (-0.01e9) for s in range(8)])
    se = ks.std(ddof=1) / np.sqrt(len(ks))
    assert abs(ks.mean() - K) < 4.0 * se, (ks.mean(), se, K)
    assert K > synth.kappa_ribbon(case["modes"], 300.0, 100.0, p=0.0)


def test_steady_needs_a_gradient():
    case = synth.periodic_case(n_particles=10)
    with pytest.raises(Exception):
        pyoracle.steady_run(case, (0.0, 0.0))


def test_even_mode_table_is_mirror_symmetric():
    m = _even_modes()
    n, nb = 9, m["nb"]
    om = m["omega"].reshape(n, n, nb)
    w = m["w"].reshape(n, n, nb)
    v = m["vg"].reshape(n, n, nb, 3)
    flip = (n - np.arange(n)) % n
    assert np.array_equal(om, om[flip]) and np.array_equal(om, om[:, flip])
    assert np.array_equal(w, w[flip]) and np.array_equal(w, w[:, flip])
    assert np.array_equal(v[..., 0], -v[flip][..., 0]) and np.array_equal(v[..., 1], v[flip][..., 1])
