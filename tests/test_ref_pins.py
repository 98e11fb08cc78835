"""The CPU restatement against the reference's own code on the same inputs.

tests/golden/ref_pins.json holds the outputs of reference functions that
oracle/build_ref.py compiled from their cited line ranges (with small
stand-ins for Boost, TBB and MPI, oracle/ref_pins.cpp) on a seeded 6x6x6
mode table.  Each test below feeds the same inputs to the restatement
(oracle/rta_oracle.cpp, through the same helpers its runs use) and requires
the same result, bit for bit unless a test says otherwise:

- utilities: almost_equal, bose_einstein and its kernel, my_jobs;
- the transient loop: get_bin_index, process_segment (transient and
  periodic), get_v, random_dt;
- the distributions: BE_derivative (CDF and draws), Isothermal_wall (CDF,
  cumulsum, flux, Ntogenerate), outTref and Nabla_T (CDF, signs,
  cumulsum, get_energy, Ntogenerate);
- diffusive_bouncing: every entry of the Lambert table and the bounce draws;
- propagator_H (signed CDF and get), lirp, the save_P file layout, and the
  propagator builder build_P (Arnoldi + matrix exponential) against the
  eigen-form exponential of the synthetic propagators."""
import ctypes as C
import json
import os

import numpy as np
import pytest

import btegpu
import pyoracle
import replicas
import synth

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "ref_pins.json")))
dp = C.POINTER(C.c_double)
lp = C.POINTER(C.c_longlong)


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


@pytest.fixture(scope="module")
def lib():
    return pyoracle.load()


@pytest.fixture(scope="module")
def modes():
    m = dict(GOLD["modes"])
    m["grid"] = (6, 6, 1)
    for k in ("omega", "vg", "w", "dq"):
        m[k] = _d(m[k])
    s, keep = btegpu.mode_struct(m)
    return m, s, keep


def test_almost_equal(lib):
    for a, b, r in GOLD["almost_equal"]:
        assert lib.oracle_kat_almost_equal(a, b) == r, (a, b)


def test_bose_einstein_and_kernel(lib):
    g = GOLD["bose"]
    om, T = _d(g["omega"]), np.array(g["T"])
    for t in np.unique(T):
        sel = T == t
        o = _d(om[sel])
        be, ke = np.zeros(o.size), np.zeros(o.size)
        lib.oracle_be(o.ctypes.data_as(dp), o.size, float(t), be.ctypes.data_as(dp), ke.ctypes.data_as(dp))
        assert np.array_equal(be, np.array(g["be"])[sel])
        assert np.array_equal(ke, np.array(g["kernel"])[sel])


def test_my_jobs_slices():
    rows = np.array(GOLD["my_jobs"]).reshape(-1, 5)
    for nj, np_, i, b, e in rows:
        assert replicas.my_jobs(int(nj), int(np_), int(i)) == (b, e)


def test_bin_index(lib):
    g = GOLD["bin_index"]
    grid = _d(g["grid"])
    for t, idx in zip(g["t"], g["index"]):
        assert lib.oracle_kat_bin_index(grid.ctypes.data_as(dp), grid.size, t) == idx, t


def test_process_segment_transient(lib):
    grid = _d(GOLD["bin_index"]["grid"])
    nb = grid.size - 1
    for c in GOLD["segment"]:
        out = [np.zeros(nb) for _ in range(3)]
        lib.oracle_kat_segment3(grid.ctypes.data_as(dp), grid.size, c["t0"], c["t1"], int(c["sign"]),
                                c["v"][0], c["v"][1], *(o.ctypes.data_as(dp) for o in out))
        for o, key in zip(out, ("gz", "jx", "jy")):
            assert np.array_equal(o, np.array(c[key])), (c["t0"], c["t1"], key)


def test_process_segment_periodic(lib):
    for c in GOLD["segment_periodic"]:
        out = np.zeros(3)
        lib.oracle_kat_steady_terms(int(c["sign"]), c["dt"], c["v"][0], c["v"][1], out.ctypes.data_as(dp))
        b = c["box"]
        assert out[0] == c["gz"][b] and out[1] == c["jx"][b] and out[2] == c["jy"][b]
        # phi(box) += sign only when evaluated
        assert c["phi"][b] == (c["sign"] if c["evalphi"] else 0)


def test_get_v(lib, modes):
    m, s, _ = modes
    n = int(m["nq"]) * int(m["nb"])
    vx, vy = np.zeros(n), np.zeros(n)
    lib.oracle_kat_get_v(C.byref(s), vx.ctypes.data_as(dp), vy.ctypes.data_as(dp))
    assert np.array_equal(vx, np.array(GOLD["get_v"]["vx"]))
    assert np.array_equal(vy, np.array(GOLD["get_v"]["vy"]))


def test_random_dt(lib):
    g = GOLD["random_dt"]
    w = _d(g["w"])
    K = len(g["dt"])
    out = np.zeros(K)
    assert lib.oracle_kat_random_dt(g["seed"], g["stream"], w.ctypes.data_as(dp), w.size, K, 1,
                                    out.ctypes.data_as(dp)) == 0
    assert np.array_equal(out, np.array(g["dt"]))  # glibc log: bit for bit
    own = np.zeros(K)
    lib.oracle_kat_random_dt(g["seed"], g["stream"], w.ctypes.data_as(dp), w.size, K, 0, own.ctypes.data_as(dp))
    ulp = np.abs(own - out) / np.spacing(np.abs(out))
    assert ulp.max() <= 4.0  # the restatement's own log (bte_log) within 4 ulp


def _dist(lib, s, n, kind, args):
    cum, sign, scal = np.zeros(n), np.zeros(n, dtype=np.int32), np.zeros(2)
    a = _d(args)
    st = lib.oracle_kat_distribution(C.byref(s), kind, a.ctypes.data_as(dp), cum.ctypes.data_as(dp),
                                     sign.ctypes.data_as(C.POINTER(C.c_int)), scal.ctypes.data_as(dp))
    assert st == 0
    return cum, sign, scal


def test_be_derivative_distribution(lib, modes):
    m, s, _ = modes
    g = GOLD["be_derivative"]
    n = int(m["nq"]) * int(m["nb"])
    cum, _, _ = _dist(lib, s, n, 0, [g["T"]])
    assert np.array_equal(cum, np.array(g["cumulative"]))
    out = np.zeros(len(g["samples"]), dtype=np.int64)
    lib.oracle_kat_be_samples(C.byref(s), g["T"], g["seed"], g["stream"], out.size, out.ctypes.data_as(lp))
    assert list(out) == g["samples"]


def _ntogen(lib, kind, args, cumulsum, nq, seed, stream):
    a = _d(np.asarray(args, float).reshape(-1))
    K = a.size // 3
    out = np.zeros(K, dtype=np.int64)
    lib.oracle_kat_ntogen(kind, a.ctypes.data_as(dp), K, cumulsum, float(nq), seed, stream, out.ctypes.data_as(lp))
    return list(out)


def test_isothermal_wall_distribution(lib, modes):
    m, s, _ = modes
    n = int(m["nq"]) * int(m["nb"])
    for g in GOLD["isothermal_wall"]:
        nrm = g["normal"]
        cum, sign, scal = _dist(lib, s, n, 1, [g["Tw"], g["Teq"], nrm[0], nrm[1], g["vuc"]])
        assert np.array_equal(cum, np.array(g["cumulative"])), nrm
        assert scal[0] == g["cumulsum"] and scal[1] == g["flux"]
        assert sign[0] == g["sign"]
        args = [[1.0 + 0.25 * i, 37.5, 2.5e-22] for i in range(16)]
        assert _ntogen(lib, 1, args, g["cumulsum"], m["nq"], 7, g["stream"]) == g["ntogen"]


def test_out_tref_distribution(lib, modes):
    m, s, _ = modes
    n = int(m["nq"]) * int(m["nb"])
    g = GOLD["out_tref"]
    cum, sign, scal = _dist(lib, s, n, 2, [g["Tinit"], g["Tref"], 400.0])
    assert np.array_equal(cum, np.array(g["cumulative"]))
    assert scal[0] == g["cumulsum"] and scal[1] == g["energy"] and sign[0] == g["sign"]
    args = [[400.0 + 37.0 * i, 3e-21, 0.0] for i in range(16)]
    assert _ntogen(lib, 2, args, g["cumulsum"], m["nq"], g["seed"], g["stream"]) == g["ntogen"]


def test_nabla_t_distribution(lib, modes):
    m, s, _ = modes
    n = int(m["nq"]) * int(m["nb"])
    g = GOLD["nabla_t"]
    cum, sign, scal = _dist(lib, s, n, 3, [g["gradient"][0], g["gradient"][1], g["T"], 400.0])
    assert np.array_equal(cum, np.array(g["cumulative"]))
    # the reference leaves the sign of zero-frequency modes (probability 0)
    # value-initialised; every mode that can be drawn has the same sign
    ref_sign = np.array(g["signs"])
    live = np.diff(np.concatenate([[0.0], cum])) > 0
    assert np.array_equal(sign[live], ref_sign[live])
    assert scal[0] == g["cumulsum"] and scal[1] == g["energy"]
    args = [[1.0, 400.0 + 37.0 * i, 3e-22] for i in range(16)]
    assert _ntogen(lib, 3, args, g["cumulsum"], m["nq"], g["seed"], g["stream"]) == g["ntogen"]


def test_lambert_table(lib, modes):
    m, s, _ = modes
    n = int(m["nq"]) * int(m["nb"])
    g = GOLD["lambert"]
    nnz = int(sum(g["nnz"]))
    rowptr, idx, val = np.zeros(n + 1, dtype=np.int64), np.zeros(nnz, dtype=np.int64), np.zeros(nnz)
    assert lib.oracle_kat_lambert(C.byref(s), rowptr.ctypes.data_as(lp), idx.ctypes.data_as(lp),
                                  val.ctypes.data_as(dp), nnz) == nnz
    assert list(np.diff(rowptr)) == g["nnz"]
    for k in range(n):
        a, b = rowptr[k], rowptr[k + 1]
        order = np.argsort(idx[a:b], kind="stable")
        total = 0.0
        for v in val[a:b][order]:  # ascending outgoing mode, as the golden sums
            total += float(v)
        # NaN on both sides for a row that pairs two zero-broadening modes
        # (zero velocity: sigma = 0, the Gaussian is 0/0); bounce never
        # reaches those entries, it skips outgoing modes without velocity
        assert total == g["sum"][k] or (np.isnan(total) and np.isnan(g["sum"][k])), k
    for r in g["rows"]:
        a, b = rowptr[r["mode"]], rowptr[r["mode"] + 1]
        order = np.argsort(idx[a:b], kind="stable")
        assert list(idx[a:b][order]) == r["index"]
        assert np.array_equal(val[a:b][order], np.array(r["value"]), equal_nan=True)


def test_bounce_draws(lib, modes):
    m, s, _ = modes
    for c in GOLD["bounce"]:
        out = np.zeros(len(c["out"]), dtype=np.int64)
        st = lib.oracle_kat_bounce(C.byref(s), c["npout"][0], c["npout"][1], c["mode"], c["seed"], c["stream"],
                                   out.size, out.ctypes.data_as(lp))
        assert st == 0
        assert list(out) == c["out"], (c["npout"], c["mode"])


def test_propagator_signed_cdf_and_draws(lib):
    g = GOLD["propagator"]
    n = g["n"]
    P = _d(g["P"])  # column-major
    for c in g["columns"]:
        out = np.zeros(n)
        lib.oracle_kat_prop_cumm(P.ctypes.data_as(dp), n, c["col"], out.ctypes.data_as(dp))
        assert np.array_equal(out, np.array(c["signed_cumm"])), c["col"]
        gets = np.array(c["get"]).reshape(-1, 2)
        for R, (sg, mode) in zip(c["R"], gets):
            sign = C.c_int()
            got = lib.oracle_kat_propagator(P.ctypes.data_as(dp), n, c["col"], R, C.byref(sign))
            assert (sign.value, got) == (sg, mode), (c["col"], R)


def test_lirp(lib):
    g = GOLD["propagator"]
    n = g["n"]
    P, Q = _d(g["P"]), _d(g["Q"])
    for c in g["lirp"]:
        out = np.zeros(n)
        lib.oracle_kat_lirp(P.ctypes.data_as(dp), Q.ctypes.data_as(dp), n, 1, c["T1"], c["T2"], c["Tx"],
                            out.ctypes.data_as(dp))
        assert np.array_equal(out, np.array(c["signed_cumm"])), c["Tx"]


def test_save_p_layout(tmp_path):
    g = GOLD["save_P"]
    M = np.array(g["matrix"]).reshape(3, 3, order="F")
    path = str(tmp_path / "x.P.eigen.bin")
    synth.write_propagator(path, M)
    assert open(path, "rb").read().hex() == g["hex"]
    back = synth.read_propagator(path)
    assert np.array_equal(back.ravel(order="F"), np.array(g["loaded"]))


def test_build_p_matches_eigen_form_exponential():
    """build_P (Krylov subspace of the order error_bound picks, H.exp())
    against the eigen-form exponential that builds the synthetic
    propagators: P = V exp(lambda t) V^T of the symmetric energy-form
    operator.  Two algorithms for exp(B t), so agreement is to the Krylov
    tolerance the reference asks for (1e-8 per element on average)."""
    g = GOLD["build_P"]
    n = g["n"]
    B = np.array(g["B"]).reshape(n, n, order="F")
    Pref = np.array(g["P"]).reshape(n, n, order="F")
    P = synth.exp_neg_psd(-B, g["t"])  # B = -A: negative semi-definite, columns summing to 0
    assert np.abs(P - Pref).max() < 1e-8 * n * n
    # energy conservation of both: columns of exp(B t) sum to 1 when B's sum to 0
    assert np.allclose(Pref.sum(axis=0), 1.0, atol=1e-8 * n)
