"""Two-sample statistics of the production-mode parity tests.

Each test runs R independent replicas on the GPU and R on the CPU
restatement, forms k observables per replica and compares their means.
For each observable, z = |mean_gpu - mean_cpu| / sqrt(s_gpu^2/R + s_cpu^2/R)
(Welch).  Two bars are applied:

- the per-observable bar of 3 sigma: the number of observables above 3 must
  not exceed what chance allows at a 1 % false-alarm rate for k observables
  (Student t with the Welch-Satterthwaite degrees of freedom);
- the family bound: the largest z must stay below 4.5.

Every z is printed with its observable's name, so a run with -s shows the
per-observable table next to the bound."""
import math

import numpy as np

PER_OBS = 3.0
FAMILY_BOUND = 4.5
FALSE_ALARM = 0.01


def welch(a, b):
    """Per-observable |z| and Welch-Satterthwaite degrees of freedom."""
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    va = a.var(0, ddof=1) / len(a)
    vb = b.var(0, ddof=1) / len(b)
    se = np.sqrt(va + vb)
    z = np.abs(a.mean(0) - b.mean(0)) / np.maximum(se, 1e-300)
    dof = (va + vb) ** 2 / np.maximum(va ** 2 / (len(a) - 1) + vb ** 2 / (len(b) - 1), 1e-300)
    return z, dof


def allowed_above(k, dof):
    """Largest count of observables above 3 sigma that k independent
    observables reach by chance with probability >= FALSE_ALARM."""
    from scipy import stats
    q = float(2.0 * stats.t.sf(PER_OBS, max(float(np.min(dof)), 2.0)))
    tail = 1.0
    for m in range(k + 1):
        # P(count > m)
        tail -= math.comb(k, m) * q ** m * (1.0 - q) ** (k - m)
        if tail < FALSE_ALARM:
            return m
    return k


def check(a, b, names, label):
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    # an observable that never varies on either side (e.g. a region no
    # particle reaches) must be identical on both sides and carries no z
    flat = (a.var(0) == 0) & (b.var(0) == 0)
    assert np.array_equal(a[0, flat], b[0, flat]), (label, [n for n, f in zip(names, flat) if f])
    if flat.any():
        a, b = a[:, ~flat], b[:, ~flat]
        names = [n for n, f in zip(names, flat) if not f]
    z, dof = welch(a, b)
    k = len(z)
    m = allowed_above(k, dof)
    above = int((z > PER_OBS).sum())
    rows = ", ".join(f"{n}={v:.2f}" for n, v in zip(names, z))
    print(f"[{label}] k={k} R={len(a)}/{len(b)} dof>={np.min(dof):.1f} max|z|={z.max():.2f} "
          f"above3={above} (allowed {m}) :: {rows}")
    assert above <= m, (label, above, m, dict(zip(names, np.round(z, 2))))
    assert z.max() < FAMILY_BOUND, (label, dict(zip(names, np.round(z, 2))))
    return z
