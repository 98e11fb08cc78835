"""CPU tests: the C-ABI library loads and exports every entry point of
include/btegpu.h, its host-side tables equal the CPU restatement's, geometry
known-answer cases, and properties of the restatement itself."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import btegpu
import pyoracle
import synth

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    text = open(os.path.join(REPO, "include", "btegpu.h")).read()
    return sorted(set(re.findall(r"^\s*(?:bte_status|int32_t)\s+(bte_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol(built):
    lib = C.CDLL(built)
    names = header_functions()
    assert set(names) == set(btegpu.PUBLIC_SYMBOLS)
    for n in names:
        assert hasattr(lib, n), n
    assert lib.bte_version() == 1


def test_create_without_gpu_fails_cleanly(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(btegpu.BteError) as e:
        btegpu.Engine(0)
    assert e.value.code == btegpu.BTE_ERR_CUDA


@pytest.mark.parametrize("which", ["small", "c0", "pore"])
def test_geometry_tables_equal_restatement(built, which):
    if which == "small":
        g = synth.small_case()["geom"]
    elif which == "c0":
        g = synth.ribbon_geometry(1000.0, 100.0, 50)
    else:
        g = synth.grid_geometry(400.0, 200.0, 20, 10, pore_center=(200.0, 100.0), pore_diameter=80.0)
    a = btegpu.debug_geometry(g)
    b = pyoracle.geometry_dump(g)
    assert np.array_equal(a, b)


def test_grid_detection(built):
    assert btegpu.debug_grid(synth.ribbon_geometry(1000.0, 100.0, 50)) == (1, 52, 1)
    g = synth.grid_geometry(400.0, 200.0, 20, 10, pore_center=(200.0, 100.0), pore_diameter=80.0)
    assert btegpu.debug_grid(g) == (1, 20, 10)
    tri = {"nboxes": 2, "npoints": np.array([3, 3], np.int32),
           "vertices": np.array([0, 0, 10, 0, 0, 10, 10, 0, 10, 10, 0, 10], float),
           "Teq": np.array([300.0, 300.0]), "Tinit": np.array([300.0, 300.0]),
           "reservoir": np.array([0, 0], np.int32), "thickness": 0.3}
    assert btegpu.debug_grid(tri)[0] == 0


def test_host_log_bits_equal_restatement(built):
    x = np.random.default_rng(3).uniform(0, 1, 50000)
    assert np.array_equal(btegpu.debug_log(x).view(np.int64), pyoracle.log(x, 0).view(np.int64))


def test_lambert_rows_nonempty_for_moving_modes(built):
    case = synth.small_case()
    tot, nnz = btegpu.debug_lambert(case["modes"], case["geom"])
    assert tot == nnz[:4].sum() and tot > 0
    raw = pyoracle.lambert_nnz(case)
    # every class keeps only outgoing modes: at most the raw row size per class
    assert nnz[:4].max() <= raw.sum()


# --------------------------------------------------------- geometry KATs
def _box(x0, y0, x1, y1):
    return [(x0, y0), (x0, y1), (x1, y1), (x1, y0)]


def _geom(boxes, res=None):
    res = res or [0] * len(boxes)
    return {"nboxes": len(boxes), "npoints": np.array([len(b) for b in boxes], np.int32),
            "vertices": np.array([c for b in boxes for p in b for c in p], float),
            "Teq": np.full(len(boxes), 300.0), "Tinit": np.full(len(boxes), 300.0),
            "reservoir": np.array(res, np.int32), "thickness": 0.3}


def test_get_inter_side_straight_and_corner():
    g = _geom([_box(0, 0, 10, 10), _box(10, 0, 20, 10)])
    # vertices (x0,y0) (x0,y1) (x1,y1) (x1,y0): get_sides pairs give the
    # borders in the order left, bottom, top, right
    t, r, b = pyoracle.inter_side(g, 0, 5.0, 5.0, 1.0, 0.0, 100.0)
    assert t == 5.0 and r == (10.0, 5.0) and b == [3]
    t, r, b = pyoracle.inter_side(g, 0, 5.0, 5.0, 0.0, -2.0, 100.0)
    assert t == 2.5 and r == (5.0, 0.0) and b == [1]
    # exactly through the corner: both borders reported
    t, r, b = pyoracle.inter_side(g, 0, 5.0, 5.0, 1.0, 1.0, 100.0)
    assert t == 5.0 and sorted(b) == [2, 3]


def test_get_inter_side_from_border_uses_fallback():
    g = _geom([_box(0, 0, 10, 10)])
    # a point on the right border moving out: the first pass skips borders
    # that contain the start point; the fallback finds it at time 0
    t, r, b = pyoracle.inter_side(g, 0, 10.0, 5.0, 1.0, 0.0, 1.0)
    assert t == 0.0 and b == [3]
    # no border ahead at all: geometry error
    assert pyoracle.inter_side(g, 0, 5.0, 5.0, 0.0, 0.0, 1.0) is None


def test_contacts_of_a_row_and_corner_touch():
    g = _geom([_box(0, 0, 10, 10), _box(10, 0, 20, 10), _box(10, 10, 20, 20)])
    d = pyoracle.geometry_dump(g)
    # box 0: 4 borders, then contacts: box 1 (edge, normal +x) and box 2 (corner point)
    nb = int(d[0])
    off = 1 + 6 * nb
    nc = int(d[off])
    contacts = d[off + 1: off + 1 + 3 * nc].reshape(nc, 3)
    assert nc == 2
    assert contacts[0].tolist() == [1.0, 1.0, 0.0]
    assert contacts[1][0] == 2.0


# --------------------------------------------------------- restatement properties
def test_restatement_log_choice_is_immaterial():
    case = synth.small_case(n_particles=400)
    a = pyoracle.rta_run(case, log_impl=0)
    b = pyoracle.rta_run(case, log_impl=1)
    scale = np.abs(a["gz"]).max()
    assert np.abs(a["gz"] - b["gz"]).max() <= 1e-12 * scale


def test_restatement_exact_sums_independent_of_threading():
    case = synth.small_case(n_particles=600)
    a = pyoracle.rta_run(case, nthreads=1)
    b = pyoracle.rta_run(case, nthreads=4)
    assert np.array_equal(a["exact"], b["exact"])
    assert a["events"] == b["events"]
    scale = np.abs(a["gz"]).max()
    assert np.abs(a["gz"] - b["gz"]).max() <= 1e-12 * scale


def test_restatement_particle_ranges_add_up():
    case = synth.small_case(n_particles=500)
    full = pyoracle.rta_run(case)
    lo = pyoracle.rta_run(case, begin=0, end=200)
    hi = pyoracle.rta_run(case, begin=200, end=500)
    s = (lo["exact"][..., 0].astype(object) * 2 ** 64 + (lo["exact"][..., 1].astype(np.uint64)).astype(object)
         + hi["exact"][..., 0].astype(object) * 2 ** 64 + (hi["exact"][..., 1].astype(np.uint64)).astype(object))
    f = full["exact"][..., 0].astype(object) * 2 ** 64 + (full["exact"][..., 1].astype(np.uint64)).astype(object)
    assert np.all(s == f)
    assert lo["events"] + hi["events"] == full["events"]


def test_restatement_steady_profile_is_monotone():
    case = synth.small_case(n_particles=4000, maxtime=400.0)
    r = pyoracle.rta_run(case, nthreads=4)
    T = r["temperature"][:5, -5:].mean(axis=1)  # interior boxes, late bins
    assert np.all(np.diff(T) < 0)               # hot (301 K) side to cold (299 K)
    assert 299.0 < T.min() < T.max() < 301.0
    assert r["absorbed"] > 0 and r["wall_hits"] > 0


def test_restatement_rejects_zero_rate_mode():
    case = synth.small_case(n_particles=50)
    m = dict(case["modes"])
    w = m["w"].copy()
    w[w > 0] = 0.0
    m["w"] = w
    with pytest.raises(btegpu.BteError) as e:
        pyoracle.rta_run({**case, "modes": m})
    assert e.value.code == btegpu.BTE_ERR_VALUE


def test_berta_frame_layout(built):
    """properties.msgpack.bin frames (src/beyondRTA_MC2d.cpp:1604-1769)."""
    msgpack = pytest.importorskip("msgpack")
    H = np.array([[0, 3, 0, -2, 0], [0, 0, 0, 0, 0], [200, 0, -70000, 0, 1]], dtype=np.int32)
    raw = btegpu.debug_frame(12.5, 3e-24, [300.0, 301.0, 299.0], H)
    head, _, body = raw.partition(b"#")
    assert int(head) == len(body)
    frame = msgpack.unpackb(body, strict_map_key=False)
    assert frame[0] == 12.5 and frame[1] == 3e-24 and frame[2] == [300.0, 301.0, 299.0]
    assert frame[3] == 4 and frame[4] == [1, 3, 3, -2]
    assert frame[5] == 0 and frame[6] == [42.0]
    assert frame[7] == 6 and frame[8] == [0, 200, 2, -70000, 4, 1]
    assert len(frame) == 3 + 2 * 3
    assert btegpu.split_frames(raw + b"0#") == [body]
