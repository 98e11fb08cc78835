"""ctypes binding of the CPU restatement (oracle/rta_oracle.cpp).

Test infrastructure: used by tests/, __graft_entry__.smoke() and the
cpu_baseline leg of bench.py only.
"""
import ctypes as C
import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)

if "btegpu" in sys.modules:
    _bt = sys.modules["btegpu"]
else:  # share the struct definitions of the engine's host module
    _spec = importlib.util.spec_from_file_location(
        "btegpu", os.path.join(REPO, "bte-barna_gb300", "btegpu.py"))
    _bt = importlib.util.module_from_spec(_spec)
    sys.modules["btegpu"] = _bt
    _spec.loader.exec_module(_bt)

_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    bspec = importlib.util.spec_from_file_location("bte_oracle_build", os.path.join(HERE, "build.py"))
    bmod = importlib.util.module_from_spec(bspec)
    bspec.loader.exec_module(bmod)
    path = bmod.build_oracle()
    lib = C.CDLL(path)
    lib.oracle_last_error.restype = C.c_char_p
    lib.oracle_rta_run.argtypes = [C.POINTER(_bt.ModeTable), C.POINTER(_bt.Geometry),
                                   C.POINTER(_bt.RtaParams), C.c_int, C.c_int,
                                   C.POINTER(_bt.RtaResult), C.POINTER(C.c_int64)]
    lib.oracle_rta_run.restype = C.c_int
    lib.oracle_rta_run_mat.argtypes = [C.POINTER(_bt.ModeTable), C.POINTER(_bt.Geometry), C.c_int,
                                       C.POINTER(C.c_double), C.POINTER(C.c_double),
                                       C.POINTER(C.c_double),
                                       C.POINTER(_bt.RtaParams), C.c_int, C.c_int,
                                       C.POINTER(_bt.RtaResult), C.POINTER(C.c_int64)]
    lib.oracle_rta_run_mat.restype = C.c_int
    lib.oracle_geometry_dump.argtypes = [C.c_void_p, C.POINTER(_bt.Geometry),
                                         C.POINTER(C.c_double), C.c_longlong]
    lib.oracle_geometry_dump.restype = C.c_longlong
    lib.oracle_inter_side.argtypes = [C.POINTER(_bt.Geometry), C.c_int] + [C.c_double] * 5 + [
        C.POINTER(C.c_double)]
    lib.oracle_inter_side.restype = C.c_int
    lib.oracle_translate.argtypes = [C.POINTER(_bt.Geometry), C.c_int] + [C.c_double] * 4 + [
        C.c_uint64, C.c_uint64, C.POINTER(C.c_int), C.POINTER(C.c_double)]
    lib.oracle_translate.restype = C.c_int
    lib.oracle_set_spectral.argtypes = [C.c_int, C.POINTER(C.c_int)]
    lib.oracle_berta_run_tab.restype = C.c_int
    lib.oracle_kat_segment.argtypes = [C.POINTER(C.c_double), C.c_int, C.c_double, C.c_double, C.c_int,
                                       C.POINTER(C.c_double)]
    lib.oracle_kat_cdf_sample.argtypes = [C.POINTER(C.c_double), C.c_int, C.c_double]
    lib.oracle_kat_cdf_sample.restype = C.c_longlong
    lib.oracle_kat_propagator.argtypes = [C.POINTER(C.c_double), C.c_int, C.c_int, C.c_double,
                                          C.POINTER(C.c_int)]
    lib.oracle_kat_propagator.restype = C.c_int
    lib.oracle_spectral_raw.argtypes = [C.POINTER(C.c_int64), C.c_longlong]
    lib.oracle_spectral_raw.restype = C.c_longlong
    lib.oracle_spectral_counts.argtypes = [C.POINTER(C.c_int64), C.c_longlong]
    lib.oracle_spectral_counts.restype = C.c_longlong
    lib.oracle_steady_run.argtypes = [C.POINTER(_bt.ModeTable), C.POINTER(_bt.Geometry),
                                      C.POINTER(_bt.SteadyParams), C.c_int, C.POINTER(_bt.SteadyResult)]
    lib.oracle_steady_run.restype = C.c_int
    lib.oracle_steady_run_multi.argtypes = [C.POINTER(_bt.ModeTable), C.c_int, C.POINTER(_bt.Geometry),
                                            C.POINTER(_bt.SteadyParams), C.c_int, C.POINTER(_bt.SteadyResult),
                                            C.POINTER(C.c_double)]
    lib.oracle_steady_run_multi.restype = C.c_int
    lib.oracle_pcg64.argtypes = [C.c_uint64, C.c_uint64, C.c_int, C.POINTER(C.c_uint64),
                                 C.POINTER(C.c_double), C.POINTER(C.c_int), C.c_int]
    lib.oracle_log.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_longlong, C.c_int]
    lib.oracle_be.argtypes = [C.POINTER(C.c_double), C.c_longlong, C.c_double,
                              C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.oracle_lambert_nnz.argtypes = [C.POINTER(_bt.ModeTable), C.POINTER(_bt.Geometry),
                                       C.POINTER(C.c_longlong)]
    lib.oracle_berta_run.argtypes = [C.POINTER(_bt.ModeTable), C.POINTER(_bt.Geometry),
                                     C.POINTER(C.c_double), C.c_int, C.POINTER(_bt.BertaParams),
                                     C.POINTER(C.c_double), C.POINTER(C.c_double),
                                     C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.POINTER(C.c_int64)]
    lib.oracle_berta_run.restype = C.c_int
    lib.oracle_timegrid.argtypes = [C.c_double, C.c_double, C.POINTER(C.c_double), C.c_int]
    lib.oracle_timegrid.restype = C.c_int
    # hooks compared with the reference's own code (tests/golden/ref_pins.json)
    dp, lp, ip = C.POINTER(C.c_double), C.POINTER(C.c_longlong), C.POINTER(C.c_int)
    mtp = C.POINTER(_bt.ModeTable)
    lib.oracle_uniform_int_seq.argtypes = [C.c_uint64, C.c_uint64, ip, C.c_int, ip]
    lib.oracle_kat_almost_equal.argtypes = [C.c_double, C.c_double]
    lib.oracle_kat_almost_equal.restype = C.c_int
    lib.oracle_kat_bin_index.argtypes = [dp, C.c_int, C.c_double]
    lib.oracle_kat_bin_index.restype = C.c_longlong
    lib.oracle_kat_segment3.argtypes = [dp, C.c_int, C.c_double, C.c_double, C.c_int, C.c_double, C.c_double,
                                        dp, dp, dp]
    lib.oracle_kat_steady_terms.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, dp]
    lib.oracle_kat_get_v.argtypes = [mtp, dp, dp]
    lib.oracle_kat_random_dt.argtypes = [C.c_uint64, C.c_uint64, dp, C.c_int, C.c_int, C.c_int, dp]
    lib.oracle_kat_random_dt.restype = C.c_int
    lib.oracle_kat_distribution.argtypes = [mtp, C.c_int, dp, dp, ip, dp]
    lib.oracle_kat_distribution.restype = C.c_int
    lib.oracle_kat_ntogen.argtypes = [C.c_int, dp, C.c_int, C.c_double, C.c_double, C.c_uint64, C.c_uint64, lp]
    lib.oracle_kat_be_samples.argtypes = [mtp, C.c_double, C.c_uint64, C.c_uint64, C.c_int, lp]
    lib.oracle_kat_lambert.argtypes = [mtp, lp, lp, dp, C.c_longlong]
    lib.oracle_kat_lambert.restype = C.c_longlong
    lib.oracle_kat_bounce.argtypes = [mtp, C.c_double, C.c_double, C.c_int, C.c_uint64, C.c_uint64, C.c_int, lp]
    lib.oracle_kat_bounce.restype = C.c_int
    lib.oracle_kat_prop_cumm.argtypes = [dp, C.c_int, C.c_int, dp]
    lib.oracle_kat_lirp.argtypes = [dp, dp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, dp]
    lib.oracle_kat_gradientT.argtypes = [mtp, C.POINTER(_bt.Geometry), dp]
    lib.oracle_kat_gradientT.restype = C.c_int
    lib.oracle_rta_run_multi.argtypes = [mtp, C.c_int, C.POINTER(_bt.Geometry), C.POINTER(_bt.RtaParams), C.c_int,
                                         C.POINTER(_bt.RtaResult), lp, dp]
    lib.oracle_rta_run_multi.restype = C.c_int
    lib.oracle_kat_dmm.argtypes = [mtp, mtp, C.c_double, C.c_double, C.c_double, C.c_double, lp, lp, lp,
                                   ip, lp, dp]
    lib.oracle_kat_dmm.restype = C.c_int
    lib.oracle_kat_dmm_reemit.argtypes = [mtp, mtp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_uint64,
                                          C.c_uint64, C.c_int, lp, ip, lp]
    lib.oracle_kat_dmm_reemit.restype = C.c_int
    _lib = lib
    return lib


def gradient_T(modes, geom):
    """calculate_gradientT of the restatement: [box, 2] K/nm."""
    lib = load()
    ms, k1 = _bt.mode_struct(modes)
    gs, k2 = _bt.geom_struct(geom)
    out = np.zeros((int(geom["nboxes"]), 2))
    st = lib.oracle_kat_gradientT(C.byref(ms), C.byref(gs), out.ctypes.data_as(C.POINTER(C.c_double)))
    if st != 0:
        raise _bt.BteError(st, lib.oracle_last_error().decode())
    return out


def timegrid(dt, maxtime):
    lib = load()
    n = lib.oracle_timegrid(dt, maxtime, None, 0)
    out = np.zeros(n)
    lib.oracle_timegrid(dt, maxtime, out.ctypes.data_as(C.POINTER(C.c_double)), n)
    return out


def translate(geom: dict, ibox: int, x: float, y: float, vx: float, vy: float, seed=1, stream=0):
    """One periodic jump of the restatement: (new box, (x, y))."""
    lib = load()
    gs, keep = _bt.geom_struct(geom)
    nb = C.c_int()
    xy = np.zeros(2)
    st = lib.oracle_translate(C.byref(gs), int(ibox), float(x), float(y), float(vx), float(vy),
                              C.c_uint64(seed), C.c_uint64(stream), C.byref(nb),
                              xy.ctypes.data_as(C.POINTER(C.c_double)))
    if st != 0:
        raise _bt.BteError(st, lib.oracle_last_error().decode())
    return nb.value, (float(xy[0]), float(xy[1]))


def steady_run(case: dict, gradient, N=None, seed=1, nthreads=8, eps_energy=-42.0, eps_flux=-42.0,
               max_generations=0, specularity=0.0):
    """Steady state of the restatement (replay draws) on a synth case dict."""
    lib = load()
    ms, k1 = _bt.mode_struct(case["modes"])
    gs, k2 = _bt.geom_struct(case["geom"])
    N = case["N"] if N is None else N

    def call(p, r):
        st = lib.oracle_steady_run(C.byref(ms), C.byref(gs), C.byref(p), int(nthreads), C.byref(r))
        if st != 0:
            raise _bt.BteError(st, lib.oracle_last_error().decode())
    return _bt.steady_call(call, int(case["geom"]["nboxes"]), case["T0"], gradient, N, seed,
                           _bt.MODE_REPLAY, eps_energy, eps_flux, max_generations,
                           specularity=specularity)


def steady_run_multi(tables, geom, T0, gradient, N, seed=1, nthreads=8, eps_energy=-42.0, eps_flux=-42.0,
                     max_generations=0, specularity=0.0, thickness=None):
    """Steady state of a geometry of several crystals with their own mode
    tables (box b in crystal geom["material"][b]), diffuse mismatch at their
    contacts."""
    lib = load()
    keep = []
    arr = (_bt.ModeTable * len(tables))()
    for i, t in enumerate(tables):
        ms, k = _bt.mode_struct(t)
        arr[i] = ms
        keep.append(k)
    gs, k2 = _bt.geom_struct(geom)

    th, thp = _thickness_arg(thickness, len(tables))

    def call(p, r):
        st = lib.oracle_steady_run_multi(arr, len(tables), C.byref(gs), C.byref(p), int(nthreads), C.byref(r),
                                         thp)
        if st != 0:
            raise _bt.BteError(st, lib.oracle_last_error().decode())
    return _bt.steady_call(call, int(geom["nboxes"]), T0, gradient, N, seed, _bt.MODE_REPLAY, eps_energy,
                           eps_flux, max_generations, specularity=specularity)


def set_spectral(boxes):
    """Spectral locations of the following rta_run calls ([] switches off)."""
    lib = load()
    b = np.ascontiguousarray(np.asarray(boxes, dtype=np.int32))
    lib.oracle_set_spectral(len(b), b.ctypes.data_as(C.POINTER(C.c_int)) if len(b) else None)


def spectral_raw(shape):
    """The last run's per-mode time at the locations: (hi, lo) fixed-point
    pairs [loc, bin, mode, 2] and their values in ps."""
    lib = load()
    n = int(np.prod(shape))
    out = np.zeros(tuple(shape) + (2,), dtype=np.int64)
    got = lib.oracle_spectral_raw(out.ctypes.data_as(C.POINTER(C.c_int64)), n)
    if got != n:
        raise ValueError(f"spectral tally has {got} values, expected {n}")
    hi = out[..., 0].reshape(-1).tolist()
    lo = out[..., 1].astype(np.uint64).reshape(-1).tolist()
    val = np.array([float((h << 64) | l) for h, l in zip(hi, lo)]).reshape(shape) / 2.0 ** 44
    return out, val


def mode_sigmas(modes):
    """Broadening of every mode, Gamma_grid::base_sigma
    (include/qpoint_grid.hpp:179-181), |v^T dq| / sqrt(12), with the low
    outliers raised to exp(p25 - 1.5 (p75 - p25)) of the log-percentiles
    (src/RTA_MC2D.cpp:573-576, :2038-2040)."""
    v = np.asarray(modes["vg"], dtype=float).reshape(-1, 3)
    dq = np.asarray(modes["dq"], dtype=float).reshape(3, 3, order="F")
    sig = np.sqrt(((v @ dq) ** 2).sum(axis=1)) / np.sqrt(12.0)
    n = sig.size
    with np.errstate(divide="ignore", over="ignore"):
        ls = np.sort(np.where(sig == 0.0, -np.finfo(float).max, np.log(np.where(sig == 0.0, 1.0, sig))))
        p25, p75 = ls[25 * n // 100], ls[75 * n // 100]
        lbound = np.exp(p25 - 1.5 * (p75 - p25))
    return np.maximum(sig, lbound)


def spectral_post(modes, raw, nomega, counts=None):
    """Post-processing of the per-mode time tally raw[loc, bin, mode]
    (src/RTA_MC2D.cpp:2041-2045, :719-766, :2386-2413) before the constant
    scalings: the omega ticks, and the time integrals of sum_k t_k g_k(w),
    sum_k vx_k t_k g_k(w), sum_k vy_k t_k g_k(w) and of t_k / w_k per q
    point, g_k the Gamma pdf of shape w_k^2 / sigma_k and scale
    sigma_k / w_k."""
    from math import lgamma
    om = np.asarray(modes["omega"], dtype=float)
    v = np.asarray(modes["vg"], dtype=float).reshape(-1, 3)
    nb = int(modes["nb"])
    maxw = om.max()
    grid = maxw * np.arange(nomega) / max(nomega - 1, 1) + 0.5 * maxw / nomega
    sig = mode_sigmas(modes)
    W = np.zeros((om.size, nomega))
    for k in np.nonzero((om > 0) & (sig > 0))[0]:   # sigma = 0: no omega weight
        kk, th = om[k] ** 2 / sig[k], sig[k] / om[k]
        x = grid / th
        lp = (kk - 1.0) * np.log(x) - x - lgamma(kk) - np.log(th)
        W[k] = np.where(lp > -700.0, np.exp(np.maximum(lp, -700.0)), 0.0)
    inv = np.where(om > 0, 1.0 / np.where(om > 0, om, 1.0), 0.0)
    fq = np.zeros(raw.shape[:2] + (om.size // nb,))
    if counts is not None:
        # steady state (:2729-2830): one bin, no time integration, and
        # fd_qmesh from the signed segment counts (sign / omega per segment)
        np.add.at(fq, (slice(None), slice(None), np.arange(om.size) // nb), counts[:, None, :] * inv)
        return grid, raw @ W, (raw * v[:, 0]) @ W, (raw * v[:, 1]) @ W, fq
    dT = np.cumsum(raw @ W, axis=1)
    jx = np.cumsum((raw * v[:, 0]) @ W, axis=1)
    jy = np.cumsum((raw * v[:, 1]) @ W, axis=1)
    np.add.at(fq, (slice(None), slice(None), np.arange(om.size) // nb), raw * inv)
    return grid, dT, jx, jy, np.cumsum(fq, axis=1)


def spectral_counts(shape):
    """The last steady run's signed segment counts per mode [loc, mode]."""
    lib = load()
    n = int(np.prod(shape))
    out = np.zeros(tuple(shape), dtype=np.int64)
    got = lib.oracle_spectral_counts(out.ctypes.data_as(C.POINTER(C.c_int64)), n)
    if got != n:
        raise ValueError(f"spectral counts have {got} values, expected {n}")
    return out


def kat_segment(grid, t0, t1, sign):
    g = np.ascontiguousarray(grid, dtype=float)
    out = np.zeros(g.size - 1)
    load().oracle_kat_segment(g.ctypes.data_as(C.POINTER(C.c_double)), g.size, t0, t1, sign,
                              out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def kat_cdf_sample(pmf, u):
    p = np.ascontiguousarray(pmf, dtype=float)
    return int(load().oracle_kat_cdf_sample(p.ctypes.data_as(C.POINTER(C.c_double)), p.size, u))


def kat_propagator(P, col, u):
    """(outgoing mode, sign) of propagator_H::get on column `col` of P."""
    a = np.ascontiguousarray(np.asarray(P, dtype=float).ravel(order="F"))
    s = C.c_int(0)
    m = load().oracle_kat_propagator(a.ctypes.data_as(C.POINTER(C.c_double)), int(np.asarray(P).shape[0]),
                                     col, u, C.byref(s))
    return m, s.value


def decode_berta_frame(body: bytes):
    """One properties.msgpack.bin frame body (src/beyondRTA_MC2d.cpp:
    1604-1769): (time, Eeff, temperatures, [{mode: count} per box]).  Reads
    the msgpack subset the frames use (arrays, float64/32, integers)."""
    import struct
    pos = [0]

    def byte():
        c = body[pos[0]]
        pos[0] += 1
        return c

    def be(n):
        v = int.from_bytes(body[pos[0]:pos[0] + n], "big")
        pos[0] += n
        return v

    def array():
        c = byte()
        if c & 0xF0 == 0x90:
            return c & 0x0F
        return be(2) if c == 0xDC else be(4)

    def number():
        c = byte()
        if c <= 0x7F:
            return c
        if c >= 0xE0:
            return c - 256
        if c == 0xCB:
            v = struct.unpack(">d", body[pos[0]:pos[0] + 8])[0]
            pos[0] += 8
            return v
        if c == 0xCA:
            v = struct.unpack(">f", body[pos[0]:pos[0] + 4])[0]
            pos[0] += 4
            return v
        if 0xCC <= c <= 0xCF:
            return be(1 << (c - 0xCC))
        n = 1 << (c - 0xD0)
        v = be(n)
        return v - (1 << (8 * n)) if v >> (8 * n - 1) else v

    top = array()
    time, Eeff = number(), number()
    temps = [number() for _ in range(array())]
    hists = []
    for _ in range((top - 3) // 2):
        nel = int(number())
        vals = [number() for _ in range(array())]
        hists.append({int(vals[2 * j]): vals[2 * j + 1] for j in range(nel // 2)})
    return time, Eeff, temps, hists


def dist_reader_restated(modes, area, thickness, boxes, nbins, hists, temps, Eeff):
    """print_distribution of dist_reader (src/dist_reader.cpp:270-508) for one
    frame: per listed box (d, dvx, dvy) on the omega mesh and dfd per q
    point, plus the mesh.  `hists` is [{mode: count} per box]."""
    from math import lgamma
    om = np.asarray(modes["omega"], dtype=float)
    v = np.asarray(modes["vg"], dtype=float).reshape(-1, 3)
    dq = np.asarray(modes["dq"], dtype=float).reshape(3, 3, order="F")
    nb, nq = int(modes["nb"]), int(modes["nq"])
    zero = np.abs(om) < 1e-8 + 1e-5 * np.abs(om)       # almost_equal(omega, 0)
    sig = np.where(zero, 0.0, np.sqrt(((v @ dq) ** 2).sum(axis=1)) / np.sqrt(12.0))
    n = sig.size
    with np.errstate(divide="ignore", over="ignore"):
        ls = np.sort(np.where(sig == 0.0, -np.finfo(float).max, np.log(np.where(sig == 0.0, 1.0, sig))))
        p25, p75 = ls[25 * n // 100], ls[75 * n // 100]
        sig = np.maximum(sig, np.exp(p25 - 1.5 * (p75 - p25)))
    mesh = np.linspace(0.0, om.max(), nbins)
    mesh = mesh + mesh[1] / 2.0
    kB, hbar = 1.3806488e-23, 1.054571726e-34
    T = temps[boxes[0]]
    vuc = modes["V"] * thickness / modes["c_lat"]
    import synth
    Cv = kB / vuc / nq * synth.be_kernel(om[~zero], T).sum()
    out = {}
    for b in boxes:
        d, dx, dy, fd = np.zeros(nbins), np.zeros(nbins), np.zeros(nbins), np.zeros(nq)
        vol = area[b] * thickness
        for k, val in hists[b].items():
            if val == 0:
                continue
            fd[k // nb] += val / om[k]
            if zero[k] or abs(sig[k]) < 1e-8:
                continue
            kk, th = om[k] ** 2 / sig[k], sig[k] / om[k]
            z = mesh / th
            g = np.exp((kk - 1.0) * np.log(z) - z - lgamma(kk) - np.log(th))
            d += val * g
            dx += val * g * 1e3 * v[k, 0]
            dy += val * g * 1e3 * v[k, 1]
        out[b] = (d * Eeff / (vol * Cv), dx * Eeff * 1e27 / vol, dy * Eeff * 1e27 / vol,
                  fd * Eeff * vuc * nq / (1e12 * vol * hbar))
    return mesh, out


def rta_run(case: dict, N=None, seed=1, nthreads=1, log_impl=0, begin=0, end=0, ballistic=False,
            source=None, specularity=None, materials=None):
    """`materials`: optional (list of per-mode rate arrays, list of T0[,
    shares]) for geometries whose boxes carry a `material` index."""
    """Run the restatement on a synth case dict; returns arrays and counters."""
    if source is None:
        source = _bt.SOURCE_INITIAL if case.get("source") == "initial" else _bt.SOURCE_WALLS
    if specularity is None:
        specularity = case.get("specularity", 0.0)
    lib = load()
    ms, k1 = _bt.mode_struct(case["modes"])
    gs, k2 = _bt.geom_struct(case["geom"])
    N = case["N"] if N is None else N
    p = _bt.params_struct(case["T0"], case["dt"], case["maxtime"], N, seed, _bt.MODE_REPLAY,
                          source, ballistic, specularity, begin, end)
    nbins = int(np.floor(case["maxtime"] / case["dt"] + 1e-6))
    shape = (int(case["geom"]["nboxes"]), nbins)
    out = {k: np.zeros(shape) for k in ("gz", "gz_jx", "gz_jy", "temperature", "jx", "jy")}
    out["exact"] = np.zeros(shape + (3, 2), dtype=np.int64)
    r = _bt.RtaResult()
    for k in ("gz", "gz_jx", "gz_jy", "temperature", "jx", "jy"):
        setattr(r, k, out[k].ctypes.data_as(C.POINTER(C.c_double)))
    r.exact = out["exact"].ctypes.data_as(C.POINTER(C.c_int64))
    cnt = np.zeros(7, dtype=np.int64)
    if materials:
        W = np.ascontiguousarray(np.stack([np.asarray(w, dtype=np.float64) for w in materials[0]]))
        T = np.ascontiguousarray(np.asarray(materials[1], dtype=np.float64))
        Sh = None
        if len(materials) > 2 and materials[2] is not None:
            Sh = np.ascontiguousarray(np.asarray(materials[2], dtype=np.float64))
        st = lib.oracle_rta_run_mat(C.byref(ms), C.byref(gs), len(materials[0]),
                                    W.ctypes.data_as(C.POINTER(C.c_double)),
                                    T.ctypes.data_as(C.POINTER(C.c_double)),
                                    None if Sh is None else Sh.ctypes.data_as(C.POINTER(C.c_double)),
                                    C.byref(p), int(nthreads),
                                    int(log_impl), C.byref(r), cnt.ctypes.data_as(C.POINTER(C.c_int64)))
    else:
        st = lib.oracle_rta_run(C.byref(ms), C.byref(gs), C.byref(p), int(nthreads), int(log_impl),
                                C.byref(r), cnt.ctypes.data_as(C.POINTER(C.c_int64)))
    if st != 0:
        raise _bt.BteError(st, lib.oracle_last_error().decode())
    out.update(Eeff=r.Eeff, energy_rate=r.energy_rate, events=int(cnt[0]), wall_hits=int(cnt[1]),
               crossings=int(cnt[2]), absorbed=int(cnt[3]), nudges=int(cnt[4]), quirks=int(cnt[5]),
               specular_hits=int(r.specular_hits), translations=int(r.translations),
               loop_seconds=float(cnt[6]) * 1e-6)
    return out


def _thickness_arg(thickness, n):
    if thickness is None:
        return None, None
    th = np.ascontiguousarray(np.asarray(thickness, dtype=float))
    if th.size != n:
        raise ValueError("one thickness per mode table")
    return th, th.ctypes.data_as(C.POINTER(C.c_double))


def rta_run_multi(tables, geom, T0, dt, maxtime, N, seed=1, nthreads=8, source=None, specularity=0.0,
                  ballistic=False, begin=0, end=0, thickness=None):
    """A geometry of several materials with their own mode tables (box b in
    material geom["material"][b]), diffuse mismatch at their contacts.
    `thickness`: each material's thickness (None: the geometry's)."""
    if source is None:
        source = _bt.SOURCE_WALLS
    lib = load()
    keep = []
    arr = (_bt.ModeTable * len(tables))()
    for i, t in enumerate(tables):
        ms, k = _bt.mode_struct(t)
        arr[i] = ms
        keep.append(k)
    gs, k2 = _bt.geom_struct(geom)
    p = _bt.params_struct(T0, dt, maxtime, N, seed, _bt.MODE_PRODUCTION, source, ballistic, specularity, begin, end)
    nbins = int(np.floor(maxtime / dt + 1e-6))
    shape = (int(geom["nboxes"]), nbins)
    out = {k: np.zeros(shape) for k in ("gz", "gz_jx", "gz_jy", "temperature", "jx", "jy")}
    r = _bt.RtaResult()
    for k in out:
        setattr(r, k, out[k].ctypes.data_as(C.POINTER(C.c_double)))
    out["exact"] = np.zeros(shape + (3, 2), dtype=np.int64)
    r.exact = out["exact"].ctypes.data_as(C.POINTER(C.c_int64))
    cnt = np.zeros(9, dtype=np.int64)
    th, thp = _thickness_arg(thickness, len(tables))
    st = lib.oracle_rta_run_multi(arr, len(tables), C.byref(gs), C.byref(p), int(nthreads), C.byref(r),
                                  cnt.ctypes.data_as(C.POINTER(C.c_longlong)), thp)
    if st != 0:
        raise _bt.BteError(st, lib.oracle_last_error().decode())
    out.update(Eeff=r.Eeff, energy_rate=r.energy_rate, events=int(cnt[0]), wall_hits=int(cnt[1]),
               crossings=int(cnt[2]), absorbed=int(cnt[3]), nudges=int(cnt[4]), quirks=int(cnt[5]),
               loop_seconds=float(cnt[6]) * 1e-6, interface_hits=int(cnt[7]),
               interface_transmissions=int(cnt[8]), translations=int(r.translations))
    return out


def dmm_table(A, B, normal, thickness, Tref):
    """The restatement's diffuse mismatch table of mode tables A and B
    (normal from A to B): per side s a list over incident modes of arrays
    (side_out, mode_out, cumulative)."""
    lib = load()
    ma, k1 = _bt.mode_struct(A)
    mb, k2 = _bt.mode_struct(B)
    ne = np.zeros(2, dtype=np.int64)
    lp_ = C.POINTER(C.c_longlong)
    args = (C.byref(ma), C.byref(mb), float(normal[0]), float(normal[1]), float(thickness), float(Tref))
    st = lib.oracle_kat_dmm(*args, ne.ctypes.data_as(lp_), None, None, None, None, None)
    if st != 0:
        raise _bt.BteError(st, lib.oracle_last_error().decode())
    nA, nB = int(A["omega"].size), int(B["omega"].size)
    fa = np.zeros(nA + 1, dtype=np.int64)
    fb = np.zeros(nB + 1, dtype=np.int64)
    tot = int(ne.sum())
    side = np.zeros(tot, dtype=np.int32)
    idx = np.zeros(tot, dtype=np.int64)
    cum = np.zeros(tot)
    st = lib.oracle_kat_dmm(*args, ne.ctypes.data_as(lp_), fa.ctypes.data_as(lp_), fb.ctypes.data_as(lp_),
                            side.ctypes.data_as(C.POINTER(C.c_int)), idx.ctypes.data_as(lp_),
                            cum.ctypes.data_as(C.POINTER(C.c_double)))
    if st != 0:
        raise _bt.BteError(st, lib.oracle_last_error().decode())
    out = []
    base = 0
    for f, n in ((fa, nA), (fb, nB)):
        lists = [(side[base + f[i]:base + f[i + 1]], idx[base + f[i]:base + f[i + 1]], cum[base + f[i]:base + f[i + 1]])
                 for i in range(n)]
        out.append(lists)
        base += int(f[n])
    return out


def dmm_reemit(A, B, normal, thickness, Tref, seed, stream, idx_in):
    """Draws of the restatement's diffuse mismatch re-emission, incident
    modes idx_in of side A in turn from one pcg64(seed, stream): (side out,
    mode out) per draw."""
    lib = load()
    ma, k1 = _bt.mode_struct(A)
    mb, k2 = _bt.mode_struct(B)
    ii = np.ascontiguousarray(idx_in, dtype=np.int64)
    side = np.zeros(ii.size, dtype=np.int32)
    io = np.zeros(ii.size, dtype=np.int64)
    lp_ = C.POINTER(C.c_longlong)
    st = lib.oracle_kat_dmm_reemit(C.byref(ma), C.byref(mb), float(normal[0]), float(normal[1]), float(thickness),
                                   float(Tref), int(seed), int(stream), int(ii.size), ii.ctypes.data_as(lp_),
                                   side.ctypes.data_as(C.POINTER(C.c_int)), io.ctypes.data_as(lp_))
    if st != 0:
        raise _bt.BteError(st, lib.oracle_last_error().decode())
    return side, io


def geometry_dump(g: dict) -> np.ndarray:
    lib = load()
    gs, keep = _bt.geom_struct(g)
    n = lib.oracle_geometry_dump(None, C.byref(gs), None, 0)
    if n < 0:
        raise _bt.BteError(3, lib.oracle_last_error().decode())
    out = np.zeros(n)
    lib.oracle_geometry_dump(None, C.byref(gs), out.ctypes.data_as(C.POINTER(C.c_double)), n)
    return out


def inter_side(g: dict, box, x, y, vx, vy, dt):
    lib = load()
    gs, keep = _bt.geom_struct(g)
    out = np.zeros(12)
    st = lib.oracle_inter_side(C.byref(gs), box, x, y, vx, vy, dt,
                               out.ctypes.data_as(C.POINTER(C.c_double)))
    if st != 0:
        return None
    nb = int(out[3])
    return out[0], (out[1], out[2]), [int(b) for b in out[4:4 + nb]]


def pcg64(seed, stream, n, int_hi=6):
    lib = load()
    raw = np.zeros(n, dtype=np.uint64)
    can = np.zeros(n)
    ints = np.zeros(n, dtype=np.int32)
    lib.oracle_pcg64(seed, stream, n, raw.ctypes.data_as(C.POINTER(C.c_uint64)),
                     can.ctypes.data_as(C.POINTER(C.c_double)),
                     ints.ctypes.data_as(C.POINTER(C.c_int)), int_hi)
    return raw, can, ints


def log(x, impl=0):
    lib = load()
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros_like(x)
    lib.oracle_log(x.ctypes.data_as(C.POINTER(C.c_double)), y.ctypes.data_as(C.POINTER(C.c_double)),
                   x.size, impl)
    return y


def lambert_nnz(case: dict) -> np.ndarray:
    lib = load()
    ms, k1 = _bt.mode_struct(case["modes"])
    gs, k2 = _bt.geom_struct(case["geom"])
    n = int(case["modes"]["nq"]) * int(case["modes"]["nb"])
    out = np.zeros(n, dtype=np.int64)
    st = lib.oracle_lambert_nnz(C.byref(ms), C.byref(gs), out.ctypes.data_as(C.POINTER(C.c_longlong)))
    if st != 0:
        raise _bt.BteError(st, lib.oracle_last_error().decode())
    return out


def berta_run(modes, geom, P, dt, maxtime, Eeff, T0=300.0, seed=1, rta=False, gradient=None):
    """beRTAMC2D restatement: per-step ed [s, box], flux [s, box, 2], N [s].
    `gradient` (K/nm): the homogeneous <gradient x y> source term."""
    lib = load()
    ms, k1 = _bt.mode_struct(modes)
    gs, k2 = _bt.geom_struct(geom)
    nsteps = _bt.berta_steps(dt, maxtime)
    nbx = int(geom["nboxes"])
    n = int(modes["nq"]) * int(modes["nb"])
    ed = np.zeros((nsteps + 1, nbx))
    flux = np.zeros((nsteps + 1, nbx, 2))
    npart = np.zeros(nsteps + 1, dtype=np.int64)
    H = np.zeros((nbx, n), dtype=np.int32)
    cnt = np.zeros(3, dtype=np.int64)
    # P: one matrix (taken at T0) or {T: matrix}, the propagator tabulated in temperature
    tab = P if isinstance(P, dict) else ({T0: P} if P is not None else {})
    Ts = np.array(sorted(tab), dtype=float)
    Pa = (np.concatenate([np.asfortranarray(tab[t]).ravel(order="F") for t in Ts]) if len(tab)
          else np.zeros(1))
    Pa = np.ascontiguousarray(Pa, dtype=float)
    nmP = int(next(iter(tab.values())).shape[0]) if tab else 0
    bp = _bt.berta_params(dt, maxtime, Eeff, T0, seed, rta, gradient=gradient)
    dp = C.POINTER(C.c_double)
    st = lib.oracle_berta_run_tab(C.byref(ms), C.byref(gs), Pa.ctypes.data_as(dp),
                                  Ts.ctypes.data_as(dp) if len(Ts) else None, len(Ts), nmP,
                                  C.byref(bp), ed.ctypes.data_as(dp), flux.ctypes.data_as(dp),
                                  npart.ctypes.data_as(C.POINTER(C.c_int64)),
                                  H.ctypes.data_as(C.POINTER(C.c_int32)),
                                  cnt.ctypes.data_as(C.POINTER(C.c_int64)))
    if st != 0:
        raise _bt.BteError(st, lib.oracle_last_error().decode())
    return {"ed": ed, "flux": flux, "nparticles": npart, "H": H, "particle_steps": int(cnt[0]),
            "branchings": int(cnt[1]), "nsteps": int(cnt[2]) - 1}
