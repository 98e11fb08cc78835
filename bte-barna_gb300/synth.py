"""Seeded synthetic inputs for the RTA / beyond-RTA particle loop.

The reference reads almaBTE HDF5 databases (src/bulk_hdf5.cpp:443-686) and
geometry XMLs (src/geometry_2d.cpp:408-522).  No database exists here, so the
workloads run on synthetic 2D-material mode tables with the shapes, sizes and
value distributions of the benchmark configurations:

  * square lattice a = 0.25 nm, out-of-plane c = thickness = 0.335 nm;
  * Gamma-centred n x n q-grid, q index iq = i*n + j, iq = 0 is Gamma;
  * acoustic branches omega = W_b sin(pi s / 2), s = 2|q| (reduced units, s = 1
    at the zone boundary along the axes), W_b ~ 2 pi U[5, 15] THz;
  * flat optical branches 2 pi U[15, 30] THz, each mode x (1 + U[-0.05, 0.05]);
  * group velocity = the analytic gradient (0 for flat branches);
  * tau = A (omega / omega_max,b)^-2 exp(-Theta / 3T) / exp(-Theta / 900),
    A log-uniform in [1, 100] ps per mode, Theta = hbar max(omega) / kB, so
    that tau(300 K) = A at omega = omega_max,b; Gamma acoustic modes get w = 0.

All randomness comes from numpy SeedSequence((master, config, purpose)).
"""
import math
import os

import numpy as np

MASTER_SEED = 20261203
KB = 1.3806488e-23
HBAR = 1.054571726e-34
A_LAT = 0.25
C_LAT = 0.335


def _rng(config: int, purpose: int) -> np.random.Generator:
    return np.random.default_rng(np.random.SeedSequence((MASTER_SEED, config, purpose)))


def mode_table(n: int = 32, n_acoustic: int = 3, n_optical: int = 3, T: float = 300.0,
               config: int = 0, even: bool = False) -> dict:
    """Mode table as a dict of numpy arrays (keys mirror bte_mode_table).

    even=True (odd n) makes every mode quantity symmetric under the mirrors
    q_x -> -q_x and q_y -> -q_y (the random lifetime amplitudes and optical
    frequencies included), so that sources and wall re-emission carry no
    net flux by symmetry: the analytic conductivities hold exactly."""
    rng = _rng(config, 1)
    nb = n_acoustic + n_optical
    idx = np.arange(n)
    qred = ((idx + n // 2) % n - n // 2) / n          # wrapped to [-1/2, 1/2)
    qx = np.repeat(qred, n)                            # iq = i*n + j
    qy = np.tile(qred, n)
    qn = np.sqrt(qx * qx + qy * qy)
    s = 2.0 * qn
    nq = n * n
    omega = np.zeros((nq, nb))
    vg = np.zeros((nq, nb, 3))
    wmax_b = np.zeros(nb)
    W = 2 * math.pi * rng.uniform(5.0, 15.0, n_acoustic)
    with np.errstate(invalid="ignore", divide="ignore"):
        ux = np.where(qn > 0, qx / np.where(qn > 0, qn, 1), 0.0)
        uy = np.where(qn > 0, qy / np.where(qn > 0, qn, 1), 0.0)
    for b in range(n_acoustic):
        omega[:, b] = W[b] * np.sin(math.pi * s / 2)
        dwds = W[b] * np.cos(math.pi * s / 2) * (math.pi / 2)
        # ds/dk = 2 (q/|q|) a / (2 pi) per unit k = (2 pi / a) q
        vg[:, b, 0] = dwds * 2.0 * ux * A_LAT / (2 * math.pi)
        vg[:, b, 1] = dwds * 2.0 * uy * A_LAT / (2 * math.pi)
        wmax_b[b] = W[b]
    omega[0, :n_acoustic] = 0.0
    vg[0, :n_acoustic, :] = 0.0
    Om = 2 * math.pi * rng.uniform(15.0, 30.0, n_optical)
    if even:
        if n % 2 == 0:
            raise ValueError("a mirror-symmetric grid needs an odd n")
        ci = np.minimum(idx, (n - idx) % n)             # mirror representative
        rep = (np.repeat(ci, n) * n + np.tile(ci, n))   # iq -> representative iq
    else:
        rep = np.arange(nq)
    for k in range(n_optical):
        b = n_acoustic + k
        omega[:, b] = (Om[k] * (1.0 + rng.uniform(-0.05, 0.05, nq)))[rep]
        wmax_b[b] = omega[:, b].max()
    A = np.exp(rng.uniform(math.log(1.0), math.log(100.0), (nq, nb)))[rep]
    theta = HBAR * 1e12 * omega.max() / KB
    ratio = np.where(omega > 0, omega / wmax_b[None, :], 1.0)
    tau = A * ratio ** -2 * math.exp(-theta / (3 * T)) / math.exp(-theta / 900.0)
    w = np.where(omega > 0, 1.0 / tau, 0.0)
    dq = np.zeros((3, 3))
    dq[0, 0] = 2 * math.pi / (A_LAT * n)
    dq[1, 1] = 2 * math.pi / (A_LAT * n)
    dq[2, 2] = 2 * math.pi / C_LAT
    return {
        "nq": nq, "nb": nb, "grid": (n, n, 1),
        "omega": np.ascontiguousarray(omega.reshape(-1)),
        "vg": np.ascontiguousarray(vg.reshape(-1)),
        "w": np.ascontiguousarray(w.reshape(-1)),
        "dq": np.ascontiguousarray(dq.reshape(-1, order="F")),
        "V": A_LAT * A_LAT * C_LAT, "c_lat": C_LAT, "T": T,
    }


def _rect(x0, y0, x1, y1):
    # vertex order of the reference's examples: (x0,y0) (x0,y1) (x1,y1) (x1,y0)
    return [(x0, y0), (x0, y1), (x1, y1), (x1, y0)]


def ribbon_geometry(length: float = 1000.0, width: float = 100.0, ncells: int = 50,
                    T_hot: float = 301.0, T_cold: float = 299.0, T0: float = 300.0,
                    thickness: float = C_LAT, reservoir_depth: float = 20.0) -> dict:
    """Ribbon of `ncells` boxes along x between two isothermal reservoirs."""
    boxes, Teq, res = [], [], []
    dx = length / ncells
    for i in range(ncells):
        boxes.append(_rect(i * dx, 0.0, (i + 1) * dx, width))
        Teq.append(T0)
        res.append(0)
    boxes.append(_rect(-reservoir_depth, 0.0, 0.0, width))
    Teq.append(T_hot)
    res.append(1)
    boxes.append(_rect(length, 0.0, length + reservoir_depth, width))
    Teq.append(T_cold)
    res.append(1)
    return _pack(boxes, Teq, list(Teq), res, thickness)


def periodic_bar_geometry(width: float = 20.0, length: float = 40.0, nstrips: int = 10,
                          T_hot: float = 302.0, T_cold: float = 300.0, T0: float = 300.0,
                          thickness: float = C_LAT, side: float = 1.5, cap: float = 2.0) -> dict:
    """A bar along y made of `nstrips` strips spanning the width, closed left
    and right by periodic boxes that map onto each other (the layout of the
    reference's example_bar: box nstrips at the right translates by -width
    to box nstrips+1 at the left and back), with reservoirs below (T_hot) and
    above (T_cold) that span the periodic boxes too."""
    boxes, Teq, res = [], [], []
    dy = length / nstrips
    for j in range(nstrips):
        boxes.append(_rect(0.0, j * dy, width, (j + 1) * dy))
        Teq.append(T0)
        res.append(0)
    right, left = nstrips, nstrips + 1
    boxes.append(_rect(width, 0.0, width + side, length))
    boxes.append(_rect(-side, 0.0, 0.0, length))
    Teq += [T0, T0]
    res += [0, 0]
    boxes.append(_rect(-side, -cap, width + side, 0.0))
    boxes.append(_rect(-side, length, width + side, length + cap))
    Teq += [T_hot, T_cold]
    res += [1, 1]
    g = _pack(boxes, Teq, list(Teq), res, thickness)
    tto = np.full(len(boxes), -1, dtype=np.int32)
    tr = np.zeros((len(boxes), 2))
    tto[right], tr[right] = left, (-width, 0.0)
    tto[left], tr[left] = right, (width, 0.0)
    g["translate_to"] = tto
    g["translation"] = tr
    return g


def layered_bar_geometry(width: float = 20.0, length: float = 40.0, nstrips: int = 10, split: int = 5,
                         T_hot: float = 302.0, T_cold: float = 300.0, T0: float = 300.0,
                         thickness: float = C_LAT, side: float = 1.5, cap: float = 2.0) -> dict:
    """The periodic bar of periodic_bar_geometry made of two crystals: strips
    0..split-1 and the hot reservoir below in crystal 0, the other strips and
    the cold reservoir above in crystal 1 (geom["material"]).  Each crystal
    has its own pair of periodic side boxes (right -> left by -width and
    back), so a flight leaving one side re-enters its own crystal."""
    boxes, Teq, res, mat = [], [], [], []
    dy = length / nstrips
    ys = split * dy
    for j in range(nstrips):
        boxes.append(_rect(0.0, j * dy, width, (j + 1) * dy))
        Teq.append(T0)
        res.append(0)
        mat.append(0 if j < split else 1)
    base = len(boxes)
    for k, (y0, y1) in enumerate(((0.0, ys), (ys, length))):
        boxes.append(_rect(width, y0, width + side, y1))   # right of crystal k
        boxes.append(_rect(-side, y0, 0.0, y1))            # left of crystal k
        Teq += [T0, T0]
        res += [0, 0]
        mat += [k, k]
    boxes.append(_rect(-side, -cap, width + side, 0.0))
    boxes.append(_rect(-side, length, width + side, length + cap))
    Teq += [T_hot, T_cold]
    res += [1, 1]
    mat += [0, 1]
    g = _pack(boxes, Teq, list(Teq), res, thickness)
    tto = np.full(len(boxes), -1, dtype=np.int32)
    tr = np.zeros((len(boxes), 2))
    for k in range(2):
        right, left = base + 2 * k, base + 2 * k + 1
        tto[right], tr[right] = left, (-width, 0.0)
        tto[left], tr[left] = right, (width, 0.0)
    g["translate_to"] = tto
    g["translation"] = tr
    g["material"] = np.array(mat, dtype=np.int32)
    return g


def periodic_cell_geometry(lx: float = 40.0, ly: float = 40.0, nx: int = 2, ny: int = 2,
                           T0: float = 300.0, thickness: float = C_LAT, side: float = 1.0) -> dict:
    """An nx x ny block of cells closed on all four sides by periodic boxes
    (right <-> left, top <-> bottom): an infinite medium for the steady
    state under a gradient.  The corners outside the block are void."""
    boxes, Teq, res = [], [], []
    dx, dy = lx / nx, ly / ny
    for i in range(nx):
        for j in range(ny):
            boxes.append(_rect(i * dx, j * dy, (i + 1) * dx, (j + 1) * dy))
            Teq.append(T0)
            res.append(0)
    nc = len(boxes)
    right, left, top, bottom = nc, nc + 1, nc + 2, nc + 3
    boxes.append(_rect(lx, 0.0, lx + side, ly))
    boxes.append(_rect(-side, 0.0, 0.0, ly))
    boxes.append(_rect(0.0, ly, lx, ly + side))
    boxes.append(_rect(0.0, -side, lx, 0.0))
    Teq += [T0] * 4
    res += [0] * 4
    g = _pack(boxes, Teq, list(Teq), res, thickness)
    tto = np.full(len(boxes), -1, dtype=np.int32)
    tr = np.zeros((len(boxes), 2))
    tto[right], tr[right] = left, (-lx, 0.0)
    tto[left], tr[left] = right, (lx, 0.0)
    tto[top], tr[top] = bottom, (0.0, -ly)
    tto[bottom], tr[bottom] = top, (0.0, ly)
    g["translate_to"] = tto
    g["translation"] = tr
    return g


def kappa_rta(modes: dict, T: float, thickness: float = C_LAT) -> np.ndarray:
    """Bulk RTA conductivity tensor (2x2, W m^-1 K^-1) of a mode table:
    1e21 kB / (nq V_uc) sum C(omega, T) v v tau, with the 2D unit-cell volume
    V thickness / c (the volume the engine's tallies use)."""
    kB = 1.3806488e-23
    om, w = modes["omega"], modes["w"]
    v = modes["vg"].reshape(-1, 3)[:, :2]
    ok = (om > 0) & (w > 0)
    C = be_kernel(om[ok], T)
    tau = 1.0 / w[ok]
    vv = np.einsum("k,ki,kj->ij", C * tau, v[ok], v[ok])
    vuc = modes["V"] * thickness / modes["c_lat"]
    return 1e21 * kB / (modes["nq"] * vuc) * vv


def kappa_berta_steps(modes: dict, T: float, dt: float, steps, thickness: float = C_LAT) -> np.ndarray:
    """Expected conductivity tensor [len(steps), 2, 2] of the beRTAMC2D loop
    with RTA scattering and a
    homogeneous gradient source in an infinite medium, at output rows
    `steps` (row s follows s loop iterations).  A source particle is born
    in an iteration and meets the scattering test 1 - exp(-w dt) at the end
    of that iteration and of every later one; the flux counts it while it
    has not scattered (after scattering the resampled modes carry no net
    flux), so tau_k becomes dt q (1 - q^s) / (1 - q), q = exp(-w_k dt), in
    the bulk formula."""
    om, w = modes["omega"], modes["w"]
    v = modes["vg"].reshape(-1, 3)[:, :2]
    ok = (om > 0) & (w > 0)
    C = be_kernel(om[ok], T)
    q = np.exp(-w[ok] * dt)
    kB = 1.3806488e-23
    vuc = modes["V"] * thickness / modes["c_lat"]
    out = []
    for s_ in np.atleast_1d(steps):
        teff = dt * q * (1 - q ** float(s_)) / (1 - q)
        out.append(1e21 * kB / (modes["nq"] * vuc) * np.einsum("k,ki,kj->ij", C * teff, v[ok], v[ok]))
    return np.array(out)


def periodic_ribbon_geometry(length: float = 40.0, width: float = 100.0, nx: int = 2, ny: int = 2,
                             T0: float = 300.0, thickness: float = C_LAT, side: float = 1.0) -> dict:
    """A ribbon along x, periodic in x (left and right periodic boxes map
    onto each other), with void above and below: the diffuse walls of an
    infinite nanoribbon of the given width."""
    boxes, Teq, res = [], [], []
    dx, dy = length / nx, width / ny
    for i in range(nx):
        for j in range(ny):
            boxes.append(_rect(i * dx, j * dy, (i + 1) * dx, (j + 1) * dy))
            Teq.append(T0)
            res.append(0)
    nc = len(boxes)
    boxes.append(_rect(length, 0.0, length + side, width))
    boxes.append(_rect(-side, 0.0, 0.0, width))
    Teq += [T0, T0]
    res += [0, 0]
    g = _pack(boxes, Teq, list(Teq), res, thickness)
    tto = np.full(len(boxes), -1, dtype=np.int32)
    tr = np.zeros((len(boxes), 2))
    tto[nc], tr[nc] = nc + 1, (-length, 0.0)
    tto[nc + 1], tr[nc + 1] = nc, (length, 0.0)
    g["translate_to"] = tto
    g["translation"] = tr
    return g


def kappa_ribbon(modes: dict, T: float, width: float, thickness: float = C_LAT, p: float = 0.0) -> float:
    """Conductivity along an infinite ribbon whose walls reflect specularly
    with probability p: kappa_xx with each lifetime scaled by the in-plane
    Fuchs-Sondheimer factor of the reference's analytic1d
    (src/analytic1d.cpp:244-273), with K = l / w, l = tau |v_y|:
      (1 - p e^{-1/K} - (1 - p) K (1 - e^{-1/K})) / (1 - p e^{-1/K});
    for p = 0 this is scale_tau_nanoribbon (src/nanos.cpp:77-112)."""
    kB = 1.3806488e-23
    om, w = modes["omega"], modes["w"]
    v = modes["vg"].reshape(-1, 3)
    ok = (om > 0) & (w > 0)
    C = be_kernel(om[ok], T)
    tau = 1.0 / w[ok]
    mfp = np.abs(tau * v[ok, 1])
    K = mfp / width
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        e = np.exp(-1.0 / np.maximum(K, 1e-300))
        f = np.where(K > 1e-12, (1.0 - p * e - (1.0 - p) * K * (1.0 - e)) / (1.0 - p * e), 1.0)
    vuc = modes["V"] * thickness / modes["c_lat"]
    return float(1e21 * kB / (modes["nq"] * vuc) * np.sum(C * tau * f * v[ok, 0] ** 2))


def pulse_geometry(lx: float = 400.0, nx: int = 40, ly: float = 20.0, T0: float = 300.0,
                   dT: float = 1.0, thickness: float = C_LAT) -> dict:
    """A row of nx cells closed on all sides by periodic boxes (an infinite
    medium of period lx along x, uniform along y) whose first cell starts
    dT above T0: the single-pulse experiment of transient_analytic1d."""
    g = periodic_cell_geometry(lx, ly, nx, 1, T0=T0, thickness=thickness)
    g["Tinit"] = g["Tinit"].copy()
    g["Tinit"][0] = T0 + dT
    return g


def spr_fourier_laplace(modes: dict, T: float, xi, s) -> np.ndarray:
    """Exact RTA single-pulse response of the infinite medium along x in
    Fourier-Laplace space (SPR_calculator_FourierLaplace::getSPR,
    src/analytic1d.cpp:1233-1283), in ps and nm:
      P(xi, s) = sum C B / sum (C / tau)(1 - B),
      B = (1 + s tau) / ((1 + s tau)^2 + xi^2 Lambda^2),  Lambda = |v_x tau|.
    Every mode enters (the reference skips the Gamma point, whose optical
    modes the engine does move)."""
    om, w = modes["omega"], modes["w"]
    vx = modes["vg"].reshape(-1, 3)[:, 0]
    ok = (om > 0) & (w > 0)
    C = be_kernel(om[ok], T)
    tau = 1.0 / w[ok]
    lam = np.abs(vx[ok] * tau)
    xi = np.atleast_1d(np.asarray(xi, dtype=float))[:, None, None]
    s = np.atleast_1d(np.asarray(s, dtype=complex))[None, :, None]
    a = 1.0 + s * tau
    B = a / (a * a + (xi * lam) ** 2)
    return (C * B).sum(-1) / ((C / tau) * (1.0 - B)).sum(-1)


def energy_fourier_laplace(modes: dict, T: float, xi, s) -> np.ndarray:
    """Energy density of the same single pulse (thermal, deposited as C_k),
    relative to the total: with g_k = C_k at t = 0 the linearised RTA
    equation gives, per mode, tau (C + C_k P / tau) B, so
      E(xi, s) = (sum tau C B + P sum C B) / sum C,
    where P = spr_fourier_laplace is the scattering-weighted temperature
    sum(g / tau) / sum(C / tau).  E(0, s) = 1 / s."""
    om, w = modes["omega"], modes["w"]
    vx = modes["vg"].reshape(-1, 3)[:, 0]
    ok = (om > 0) & (w > 0)
    C = be_kernel(om[ok], T)
    tau = 1.0 / w[ok]
    lam = np.abs(vx[ok] * tau)
    xi = np.atleast_1d(np.asarray(xi, dtype=float))[:, None, None]
    s = np.atleast_1d(np.asarray(s, dtype=complex))[None, :, None]
    a = 1.0 + s * tau
    B = a / (a * a + (xi * lam) ** 2)
    P = (C * B).sum(-1) / ((C / tau) * (1.0 - B)).sum(-1)
    return ((tau * C * B).sum(-1) + P * (C * B).sum(-1)) / C.sum()


def talbot_inverse(F, t: float, M: int = 32) -> float:
    """Inverse Laplace transform of F at t > 0 by the fixed Talbot contour
    (Abate and Valko 2004): s(theta) = r theta (cot theta + i), r = 2M / (5t)."""
    r = 2.0 * M / (5.0 * t)
    th = np.arange(1, M) * math.pi / M
    cot = 1.0 / np.tan(th)
    sk = r * th * (cot + 1j)
    sig = th + (th * cot - 1.0) * cot
    Fk = F(np.concatenate([[r + 0j], sk]))
    val = 0.5 * np.real(Fk[0] * np.exp(r * t)) + np.sum(np.real(np.exp(t * sk) * Fk[1:] * (1.0 + 1j * sig)))
    return float(r / M * val)


def pulse_response_bins(modes: dict, T: float, xi_list, dt_bin: float, nbins: int,
                        h: float = 0.01) -> np.ndarray:
    """Bin averages of G(xi, t) over [i dt_bin, (i + 1) dt_bin) for each xi,
    from the same linearised RTA equation integrated in time per mode
    (RK4, step h ps): dg_k/dt = -(i xi v_k + 1/tau_k) g_k + C_k dT / tau_k,
    dT = sum(g / tau) / sum(C / tau), g_k(0) = C_k, G = sum g / sum C.
    Exact to the step error; the Talbot inversion of the transform agrees to
    six digits except at late times and large xi.

    xi = inf gives the limit of large xi: every mode with vx != 0 has left
    (its g stays 0), the modes with vx = 0 relax and exchange energy among
    themselves through dT."""
    om, w = modes["omega"], modes["w"]
    vx = modes["vg"].reshape(-1, 3)[:, 0]
    ok = (om > 0) & (w > 0)
    C = be_kernel(om[ok], T)
    tau = 1.0 / w[ok]
    xi = np.asarray(xi_list, dtype=float)[:, None]
    inf = np.isinf(xi)
    keep = ~(inf & (vx[ok][None, :] != 0.0))
    rate = np.where(keep, -(1j * np.where(inf, 0.0, xi) * vx[ok][None, :] + 1.0 / tau[None, :]), 0.0)
    Ct = C / tau
    sCt = Ct.sum()

    def f(g):
        dT = (g / tau).sum(axis=1, keepdims=True) / sCt
        return keep * (rate * g + Ct[None, :] * dT)

    g = keep * C.astype(complex)[None, :]
    steps = int(round(dt_bin / h))
    out = np.zeros((xi.shape[0], nbins))
    Gprev = (g.sum(axis=1) / C.sum()).real
    for b in range(nbins):
        acc = 0.0
        for _ in range(steps):
            k1 = f(g)
            k2 = f(g + 0.5 * h * k1)
            k3 = f(g + 0.5 * h * k2)
            k4 = f(g + h * k3)
            g = g + h / 6.0 * (k1 + 2 * k2 + 2 * k3 + k4)
            Gnew = (g.sum(axis=1) / C.sum()).real
            acc = acc + 0.5 * (Gprev + Gnew) * h   # trapezoid in time
            Gprev = Gnew
        out[:, b] = acc / dt_bin
    return out


def pulse_response(modes: dict, T: float, xi: float, t: float) -> float:
    """G(xi, t): the xi Fourier component of the energy density at time t
    after a thermal pulse, relative to t = 0 (G(0, t) = 1)."""
    return talbot_inverse(lambda s: energy_fourier_laplace(modes, T, [xi], s)[0], t)


def grid_geometry(lx: float, ly: float, nx: int, ny: int, T0: float = 300.0,
                  pore_center=None, pore_diameter: float = 0.0,
                  hot_center=None, hot_sigma: float = 50.0, hot_dT: float = 0.0,
                  thickness: float = C_LAT) -> dict:
    """Rectangle of nx x ny cells; cells whose centre lies inside the pore
    circle are removed (a staircase pore); optional Gaussian initial hot spot
    sets Tinit per cell."""
    boxes, Teq, Tinit, res = [], [], [], []
    dx, dy = lx / nx, ly / ny
    for i in range(nx):
        for j in range(ny):
            cx, cy = (i + 0.5) * dx, (j + 0.5) * dy
            if pore_center is not None:
                if math.hypot(cx - pore_center[0], cy - pore_center[1]) < pore_diameter / 2:
                    continue
            boxes.append(_rect(i * dx, j * dy, (i + 1) * dx, (j + 1) * dy))
            Teq.append(T0)
            if hot_center is not None and hot_dT != 0.0:
                r2 = (cx - hot_center[0]) ** 2 + (cy - hot_center[1]) ** 2
                Tinit.append(T0 + hot_dT * math.exp(-r2 / (2 * hot_sigma ** 2)))
            else:
                Tinit.append(T0)
            res.append(0)
    return _pack(boxes, Teq, Tinit, res, thickness)


def _pack(boxes, Teq, Tinit, res, thickness):
    npts = np.array([len(b) for b in boxes], dtype=np.int32)
    verts = np.array([c for b in boxes for p in b for c in p], dtype=np.float64)
    return {
        "nboxes": len(boxes), "npoints": npts, "vertices": verts,
        "Teq": np.array(Teq, dtype=np.float64), "Tinit": np.array(Tinit, dtype=np.float64),
        "reservoir": np.array(res, dtype=np.int32), "thickness": float(thickness),
    }


def write_geometry_xml(path: str, geom: dict, material: str = "synthetic") -> None:
    """Geometry XML in the schema of read_geometry_XML (src/geometry_2d.cpp:408-522).
    With a "material" array, box b's MaterialID is `material` + its index."""
    lines = ["<Geometry>", f'    <number_of_boxes Ngeom="{geom["nboxes"]}"/>']
    off = 0
    for i in range(geom["nboxes"]):
        n = int(geom["npoints"][i])
        lines.append("    <Box>")
        lines.append(f'        <BoxID id="{i}"/>')
        mname = material + str(int(geom["material"][i])) if geom.get("material") is not None else material
        lines.append(f'        <MaterialID name="{mname}"/>')
        lines.append(f'        <Vertices dim="2" npoints="{n}">')
        for k in range(n):
            x, y = geom["vertices"][2 * (off + k)], geom["vertices"][2 * (off + k) + 1]
            lines.append(f"           {float(x)!r} {float(y)!r}")
        lines.append("        </Vertices>")
        off += n
        teq, tin = float(geom["Teq"][i]), float(geom["Tinit"][i])
        if tin != teq:
            lines.append(f'        <initCnd Teq="{teq!r}" Tinit="{tin!r}"/>')
        else:
            lines.append(f'        <initCnd Teq="{teq!r}"/>')
        if geom["reservoir"][i]:
            lines.append("        <Reservoir/>")
        tto = geom.get("translate_to")
        if tto is not None and int(tto[i]) >= 0:
            tx, ty = (float(v) for v in np.asarray(geom["translation"]).reshape(-1, 2)[i])
            lines.append(f'        <Translate_to id="{int(tto[i])}">')
            lines.append(f"            {tx!r} {ty!r} 0.0")
            lines.append("        </Translate_to>")
        lines.append("    </Box>")
    lines.append("</Geometry>")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


MODES_MAGIC = b"BTEMODE1"


def write_modes_file(path: str, m: dict) -> None:
    """Binary mode table read by the rtamc2d_gpu drop-in in place of the HDF5
    database: magic, int32 nq, nb, grid[3], float64 V, c_lat, dq[9], then
    omega[nq*nb], vg[nq*nb*3], w[nq*nb] (little endian)."""
    with open(path, "wb") as f:
        f.write(MODES_MAGIC)
        np.array([m["nq"], m["nb"], *m["grid"]], dtype="<i4").tofile(f)
        np.array([m["V"], m["c_lat"]], dtype="<f8").tofile(f)
        np.asarray(m["dq"], dtype="<f8").tofile(f)
        np.asarray(m["omega"], dtype="<f8").tofile(f)
        np.asarray(m["vg"], dtype="<f8").tofile(f)
        np.asarray(m["w"], dtype="<f8").tofile(f)


def be_kernel(omega, T):
    """(x / sinh x)^2 with x = hbar omega / 2 kB T (include/utilities.hpp:401-417)."""
    x = 0.5 * 1e12 * HBAR / KB * np.asarray(omega) / T
    out = np.ones_like(x)
    big = x > 300.0
    mid = (x >= 1e-320) & ~big
    out[big] = 0.0
    out[mid] = (x[mid] / np.sinh(x[mid])) ** 2
    return out


def propagator(modes: dict, dt: float = 1.0, T: float = 300.0, nnz_row: int = 64,
               config: int = 2, flip: float = 0.25, use_torch: bool = False) -> np.ndarray:
    """Dense propagator P = exp(B dt) over the non-Gamma modes (3..n-1), in the
    column convention of PropagatorBuilder (src/collision_operator.cpp:1015-1064):
    particle in mode j draws its next mode from column j; columns sum to 1.

    Synthetic operator (symmetrised form, c = C^1/2 the square roots of the
    mode heat capacities): A = A_RTA + L with
      A_RTA = W - (W c)(W c)^T / (c^T W c), W = diag(1/tau): relaxation with
              the energy-conserving resampling of the RTA;
      L     = a seeded symmetric sparse coupling (~nnz_row entries per row)
              with weights s_ij ~ LogNormal(0,1) min(1/tau_i, 1/tau_j) 0.1,
              L_ij = -s_ij, L_ii = sum_j s_ij c_j / c_i; a seeded fraction
              `flip` of the couplings changes sign, which gives P the
              negative entries (and the branching) of real propagators.
    Both parts are symmetric and annihilate c, so A C^1/2 = 0 (energy
    conservation); negative eigenvalues are clipped to make A PSD (c stays
    an eigenvector of eigenvalue 0).  B = -C^1/2 A C^-1/2, so
    P = C^1/2 exp(-A dt) C^-1/2, evaluated through the eigenvectors of A."""
    rng = _rng(config, 2)
    w = np.asarray(modes["w"])[3:]
    om = np.asarray(modes["omega"])[3:]
    n = w.size
    rate = np.where(w > 0, w, 0.0)
    c = np.sqrt(be_kernel(om, T))
    Wc = rate * c
    A = np.diag(rate) - np.outer(Wc, Wc) / float(c @ Wc)
    k = max(1, nnz_row // 2)
    rows = np.repeat(np.arange(n), k)
    cols = rng.integers(0, n, size=n * k)
    keep = rows != cols
    rows, cols = rows[keep], cols[keep]
    wgt = rng.lognormal(0.0, 1.0, rows.size) * np.minimum(rate[rows], rate[cols]) * 0.1
    wgt *= np.where(rng.random(rows.size) < flip, -1.0, 1.0)
    S = np.zeros((n, n))
    np.add.at(S, (rows, cols), wgt)
    S = S + S.T
    A -= S
    A[np.diag_indices(n)] += (S @ c) / c
    A = 0.5 * (A + A.T)
    E = exp_neg_psd(A, dt, use_torch)
    P = (c[:, None] * E) / c[None, :]
    return np.asfortranarray(P)


def exp_neg_psd(A: np.ndarray, dt: float, use_torch: bool = False) -> np.ndarray:
    """exp(-A dt) of a symmetric A through its eigenvectors, with negative
    eigenvalues clipped to 0 (A made positive semi-definite): V e^{-lambda dt}
    V^T.  The propagator builder of the reference (build_P,
    src/collision_operator.cpp:1015-1064) computes the same exponential by
    Arnoldi iterations and a dense exponential of the Krylov matrix."""
    if use_torch:
        import torch
        dev = "cuda" if torch.cuda.is_available() else "cpu"
        lam, V = torch.linalg.eigh(torch.from_numpy(A).to(dev))
        lam = torch.clamp(lam, min=0.0)
        E = (V * torch.exp(-lam * dt)) @ V.T
        return E.cpu().numpy()
    lam, V = np.linalg.eigh(A)
    lam = np.clip(lam, 0.0, None)
    return (V * np.exp(-lam * dt)) @ V.T


def write_propagator(path: str, P: np.ndarray) -> None:
    """*.P.eigen.bin of save_P (src/collision_operator.cpp:931-970): int64
    number of rows, then the matrix in column-major FP64."""
    P = np.asfortranarray(P, dtype="<f8")
    with open(path, "wb") as f:
        np.array([P.shape[0]], dtype="<i8").tofile(f)
        f.write(P.tobytes(order="F"))


def read_propagator(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        n = int(np.fromfile(f, dtype="<i8", count=1)[0])
        data = np.fromfile(f, dtype="<f8", count=n * n)
    return data.reshape((n, n), order="F")


# ------------------------------------------------------------------ sweep
def sweep_cases(n_widths: int = 16, temps=(100.0, 200.0, 300.0, 500.0), w_min: float = 20.0,
                w_max: float = 2000.0, n0: float = 1e5) -> list:
    """The batched-sweep cases: n_widths ribbon widths log-spaced over
    [w_min, w_max] at each temperature, budgets N_w = n0 * 100^(k/15)."""
    widths = np.geomspace(w_min, w_max, n_widths)
    budgets = [int(round(n0 * 100.0 ** (k / max(n_widths - 1, 1)))) for k in range(n_widths)]
    return [{"T": float(T), "width": float(w), "budget": int(N)}
            for T in temps for w, N in zip(widths, budgets)]


def sweep_ribbon(width: float, T: float, length: float = 1000.0, ncells: int = 50, dT: float = 1.0,
                 thickness: float = C_LAT) -> dict:
    """One sweep case alone: the plain ribbon at temperature T with its
    reservoirs at T + dT and T - dT."""
    return ribbon_geometry(length, width, ncells, T_hot=T + dT, T_cold=T - dT, T0=T,
                           thickness=thickness)


def sweep_union_geometry(cases: list, length: float = 1000.0, ncells: int = 50, dT: float = 1.0,
                         gap: float = 10.0, reservoir_depth: float = 20.0,
                         thickness: float = C_LAT) -> dict:
    """Every case's ribbon in one geometry: ribbons stacked along y with a
    void gap between them (so no particle changes ribbon), each with its own
    reservoirs at T +- dT; box material = case index.  The boxes tile one
    axis-aligned grid (shared x lines), so the union runs on the grid path."""
    boxes, Teq, res, mat = [], [], [], []
    dx = length / ncells
    y0 = 0.0
    for ci, cs in enumerate(cases):
        w, T = cs["width"], cs["T"]
        for i in range(ncells):
            boxes.append(_rect(i * dx, y0, (i + 1) * dx, y0 + w))
            Teq.append(T)
            res.append(0)
            mat.append(ci)
        boxes.append(_rect(-reservoir_depth, y0, 0.0, y0 + w))
        boxes.append(_rect(length, y0, length + reservoir_depth, y0 + w))
        Teq += [T + dT, T - dT]
        res += [1, 1]
        mat += [ci, ci]
        y0 += w + gap
    g = _pack(boxes, Teq, list(Teq), res, thickness)
    g["material"] = np.array(mat, dtype=np.int32)
    g["ncells"] = ncells
    return g


def sweep_kappa(jx: np.ndarray, cells, length: float = 1000.0, dT: float = 1.0, last: int = 10) -> float:
    """kappa_eff = J_x L / Delta T (W m^-1 K^-1) from the flux of the given
    cells averaged over the last time bins (the step response has reached
    its steady state there)."""
    J = float(np.mean(jx[cells, -last:]))
    return J * length * 1e-9 / (2.0 * dT)


# ------------------------------------------------------------------ configs
def config0(n_particles: int = 1_000_000) -> dict:
    """Plain RTA ribbon: 32x32x6 modes, 1 um x 100 nm, 50 cells, 301/299 K
    reservoirs, diffuse walls, 100 bins of 10 ps."""
    return {"modes": mode_table(32, 3, 3, 300.0, config=0),
            "geom": ribbon_geometry(1000.0, 100.0, 50),
            "T0": 300.0, "dt": 10.0, "maxtime": 1000.0, "N": n_particles,
            "specularity": 0.0, "source": "walls"}


def config1(n_particles: int = 100_000_000) -> dict:
    """Transient RTA at scale: 64x64x9 modes, 2 um x 500 nm, 100x25 cells of
    20 nm, 200 nm-diameter staircase pore at the centre, p = 0.3, 1 K Gaussian
    hot spot (sigma 50 nm) at (500, 250) nm, 200 bins to 10 ns."""
    return {"modes": mode_table(64, 3, 6, 300.0, config=1),
            "geom": grid_geometry(2000.0, 500.0, 100, 25, 300.0,
                                  pore_center=(1000.0, 250.0), pore_diameter=200.0,
                                  hot_center=(500.0, 250.0), hot_sigma=50.0, hot_dT=1.0),
            "T0": 300.0, "dt": 50.0, "maxtime": 10000.0, "N": n_particles,
            "specularity": 0.3, "source": "initial"}


def periodic_case(n: int = 8, n_particles: int = 2000, maxtime: float = 200.0,
                  dt: float = 10.0) -> dict:
    """Parity-sized periodic bar (transient, walls source)."""
    return {"modes": mode_table(n, 3, 3, 300.0, config=100),
            "geom": periodic_bar_geometry(),
            "T0": 300.0, "dt": dt, "maxtime": maxtime, "N": n_particles,
            "specularity": 0.0, "source": "walls"}


def small_case(n: int = 8, ncells: int = 5, n_particles: int = 2000, maxtime: float = 200.0,
               dt: float = 10.0, width: float = 50.0, length: float = 200.0) -> dict:
    """A parity-sized ribbon the oracle finishes in well under a second."""
    return {"modes": mode_table(n, 3, 3, 300.0, config=100),
            "geom": ribbon_geometry(length, width, ncells),
            "T0": 300.0, "dt": dt, "maxtime": maxtime, "N": n_particles,
            "specularity": 0.0, "source": "walls"}


if __name__ == "__main__":
    m = mode_table()
    print(m["nq"], m["nb"], float(np.max(np.abs(m["vg"]))), float(np.max(m["omega"])))
    w = m["w"][m["w"] > 0]
    print("tau range ps", 1 / w.max(), 1 / w.min())
    os.makedirs("/tmp/bte", exist_ok=True)
