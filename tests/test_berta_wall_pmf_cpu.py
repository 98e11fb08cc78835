"""The adiabatic walls' re-emission pmf of the beyond-RTA step
(Isothermal_wall_distribution, src/sampling.cpp:189-269:
pmf_k = v_n omega_k |n(omega_k, Tw) - n(omega_k, Te)|) is evaluated in
FP32 on the device (berta.cu, wall_pmf_f): with x = hbar omega / kT,
n_w - n_e = expm1(x_e - x_w) / (expm1(x_e) (-expm1(-x_w))) while
|x_e - x_w| < 1/2, the plain difference otherwise.  This restates that
arithmetic in numpy float32 and holds it to the bound the kernel's comment
states against the FP64 pmf, over wall temperatures from 1e-4 relative of
Te to 100x away."""
import numpy as np

PRE = 1e12 * 1.054571726e-34 / 1.3806488e-23


def pmf_f32(w, vn, Te, Tw):
    ce, q, rr = np.float32(PRE / Te), np.float32(Te / Tw), np.float32((Tw - Te) / Tw)
    wf, vnf = w.astype(np.float32), vn.astype(np.float32)
    with np.errstate(over="ignore", divide="ignore", invalid="ignore"):
        xe = ce * wf
        xw = xe * q
        d = xe * rr
        a = np.where(xe < 80, np.expm1(d) / (np.expm1(xe) * -np.expm1(-xw)), np.float32(0))
        b = np.float32(1) / np.expm1(xw) - np.float32(1) / np.expm1(xe)
        diff = np.where(np.abs(d) < 0.5, a, b)
    return (vnf * wf * np.abs(diff)).astype(np.float64)


def test_fp32_wall_pmf_is_within_its_bound():
    rng = np.random.default_rng(2)
    worst_big = worst_all = 0.0
    for _ in range(300):
        Te = rng.uniform(20.0, 1000.0)
        Tw = [Te * (1 + rng.uniform(-1e-4, 1e-4)), rng.uniform(10.0, 1000.0), Te + rng.uniform(-1.0, 1.0)][
            rng.integers(3)]
        w = np.exp(rng.uniform(np.log(0.01), np.log(300.0), 5000))
        vn = rng.uniform(0.01, 10.0, w.size)
        ref = vn * w * np.abs(1 / np.expm1(PRE * w / Tw) - 1 / np.expm1(PRE * w / Te))
        got = pmf_f32(w, vn, Te, Tw)
        assert np.all(np.isfinite(got))
        rel = np.abs(got - ref) / np.where(ref > 0, ref, 1.0)
        worst_big = max(worst_big, rel[ref > 1e-6 * ref.max()].max())
        worst_all = max(worst_all, rel[ref > 1e-30 * ref.max()].max())
    assert worst_big < 4e-6, worst_big
    assert worst_all < 1e-5, worst_all
