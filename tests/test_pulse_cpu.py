"""Transient physics pin: the single-pulse response of an infinite medium.

A row of cells closed by periodic boxes on all sides, one cell 1 K hot at
t = 0 (source: initial deviation).  The Fourier components of the MC
temperature profile must follow the exact RTA response of the reference's
transient_analytic1d (SPR_calculator_FourierLaplace, src/analytic1d.cpp:
1233-1283, restated with the energy-density weighting in
synth.energy_fourier_laplace and inverted by a fixed Talbot contour)."""
import math

import numpy as np
import pytest

import pyoracle
import synth

NX, LX, DT, TMAX = 40, 400.0, 10.0, 200.0


def pulse_components(runs, ns=(1, 2)):
    x = (np.arange(NX) + 0.5) * (LX / NX) - 0.5 * (LX / NX)
    out = {n: [] for n in ns}
    for r in runs:
        T = r["temperature"][:NX] - 300.0
        for n in ns:
            xi = 2 * math.pi * n / LX
            out[n].append((T * np.cos(xi * x)[:, None]).sum(0) / T.sum(0))
    return {n: np.array(v) for n, v in out.items()}


def analytic_components(modes, n, K=8):
    """What the cosine sum over cell averages of the analytic profile gives:
    the one-cell pulse has every wavenumber m with weight sinc(xi_m dx / 2),
    cell averaging multiplies by it again, and the sum at n collects the
    aliases m = n + k NX:  D_n(t) = sum_k sinc^2(xi_{n+kN} dx/2) G(xi_{n+kN}, t)
    (D_n(0) = 1).  |k| <= K exactly; the aliases beyond K carry the weights
    sum_{|k|>K} sinc^2 (about 2 sin^2(pi n/N) / (pi^2 K)) times the large-xi
    limit of G, which the modes with vx = 0 set."""
    h = 0.5 * LX / NX
    ms = [n + k * NX for k in range(-K, K + 1)]
    xis = [2 * math.pi * m / LX for m in ms] + [math.inf]
    G = synth.pulse_response_bins(modes, 300.0, xis, DT, int(TMAX / DT), h=0.005)
    w = np.array([(math.sin(x * h) / (x * h)) ** 2 for x in xis[:-1]])
    k = np.arange(K + 1, 200000, dtype=float)
    s2 = math.sin(math.pi * n / NX) ** 2
    tail = s2 / math.pi ** 2 * ((1.0 / (k + n / NX) ** 2).sum() + (1.0 / (k - n / NX) ** 2).sum())
    return (w[:, None] * G[:-1]).sum(axis=0) + tail * G[-1]


def test_talbot_inversion_of_known_transforms():
    assert abs(synth.talbot_inverse(lambda s: 1.0 / (s + 0.3), 2.0) - math.exp(-0.6)) < 1e-10
    assert abs(synth.talbot_inverse(lambda s: 1.0 / s ** 2, 3.0) - 3.0) < 1e-10


def test_talbot_and_time_integration_agree_on_the_pulse():
    m = synth.mode_table(9, 3, 3, 300.0, config=100, even=True)
    xi = 2 * math.pi / LX
    b = synth.pulse_response_bins(m, 300.0, [xi], 5.0, 6)[0]     # 6 bins of 5 ps
    tal = np.mean([synth.pulse_response(m, 300.0, xi, t) for t in np.linspace(25.25, 29.75, 10)])
    assert abs(b[5] - tal) < 2e-4


def test_pulse_restatement_follows_the_analytic_response():
    m = synth.mode_table(9, 3, 3, 300.0, config=100, even=True)
    case = {"modes": m, "geom": synth.pulse_geometry(LX, NX), "T0": 300.0, "dt": DT,
            "maxtime": TMAX, "N": 40000, "source": "initial"}
    runs = [pyoracle.rta_run(case, seed=50 + k, nthreads=8) for k in range(10)]
    comps = pulse_components(runs)
    for n, a in comps.items():
        an = analytic_components(m, n)
        mu, se = a.mean(0), a.std(0, ddof=1) / np.sqrt(len(a))
        z = np.abs(mu - an) / se
        assert np.median(z) < 2.0 and z.max() < 6.0, (n, z)
        assert np.abs(mu - an).max() < 0.002
