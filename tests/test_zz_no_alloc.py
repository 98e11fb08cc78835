"""bte_rta_run_noalloc, the allocation-free entry point, against bte_rta_run.

Callers that cannot allocate device memory at run time (a framework that
owns every device allocation through its own pool, or a loop that must not
reach the driver's allocator) pass their own device buffer for the tallies;
the entry point keeps its scratch in a fixed device array of the library.
Both entry points carry the same particles with the same counter-based
streams, so their tallies agree to FP64 atomic ordering (1e-12 of the
largest tally, the tolerance of the other GPU tests) and their event
counters agree exactly.  Two calls in a row check that the
shared scratch starts clean on every call; the device's free memory must not
change across the second call, and the context's own entry point must give
its result unchanged after the allocation-free calls.
"""
import ctypes as C

import numpy as np
import pytest

import btegpu
import synth

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12


def _check_against(ref, got, nev):
    for q, key in enumerate(("gz", "gz_jx", "gz_jy")):
        scale = np.abs(ref[key]).max()
        assert scale > 0
        assert np.abs(got[..., q] - ref[key]).max() <= REL_TOL * scale, key
    assert nev == ref["events"]


@pytest.mark.parametrize("which", ["walls", "initial"])
def test_noalloc_matches_bte_rta_run(built, which):
    import torch
    eng = btegpu.Engine(0)
    try:
        if which == "walls":
            case = synth.small_case(n_particles=20000)
            src, p = btegpu.SOURCE_WALLS, 0.0
        else:
            g = synth.grid_geometry(400.0, 200.0, 20, 10, pore_center=(200.0, 100.0),
                                   pore_diameter=80.0, hot_center=(100.0, 100.0),
                                   hot_sigma=30.0, hot_dT=1.0)
            case = {"modes": synth.mode_table(8, 3, 3, 300.0, config=100), "geom": g,
                    "T0": 300.0, "dt": 10.0, "maxtime": 200.0, "N": 20000}
            src, p = btegpu.SOURCE_INITIAL, 0.3
        eng.load_modes(case["modes"])
        eng.load_geometry(case["geom"])
        # the existing entry point prepares the context and gives the reference tallies
        ref = eng.rta_run(case["T0"], case["dt"], case["maxtime"], case["N"], seed=21,
                          mode=btegpu.MODE_PRODUCTION, source=src, specularity=p)
        nboxes, nbins = ref["gz"].shape
        params = btegpu.params_struct(case["T0"], case["dt"], case["maxtime"], case["N"], 21,
                                      btegpu.MODE_PRODUCTION, src, False, p)
        dev = torch.empty((nboxes, nbins, 3), dtype=torch.float64, device="cuda:0")
        for call in range(2):
            dev.fill_(123.0)  # stale contents must not leak into the result
            torch.cuda.synchronize()
            free_before = torch.cuda.mem_get_info(0)[0]
            r = btegpu.RtaResult()
            st = eng.lib.bte_rta_run_noalloc(eng.ctx, C.byref(params), C.c_void_p(dev.data_ptr()),
                                             C.byref(r))
            assert st == btegpu.BTE_OK, st
            torch.cuda.synchronize()
            free_after = torch.cuda.mem_get_info(0)[0]
            if call == 1:  # the first call may load the module; the second allocates nothing
                assert free_after == free_before, (free_before, free_after)
            got = dev.cpu().numpy()
            _check_against(ref, got, r.events)
            assert (r.nboxes, r.nbins) == (nboxes, nbins)
            assert r.Eeff == ref["Eeff"]
        # the context's own tables and buffers are untouched by the calls above
        again = eng.rta_run(case["T0"], case["dt"], case["maxtime"], case["N"], seed=21,
                            mode=btegpu.MODE_PRODUCTION, source=src, specularity=p)
        assert again["events"] == ref["events"]
        for key in ("gz", "gz_jx", "gz_jy"):
            scale = np.abs(ref[key]).max()
            assert np.abs(again[key] - ref[key]).max() <= REL_TOL * scale, key
    finally:
        eng.close()


def test_noalloc_rejects_unprepared_and_oversized(built):
    import torch
    eng = btegpu.Engine(0)
    try:
        case = synth.small_case(n_particles=1000)
        eng.load_modes(case["modes"])
        eng.load_geometry(case["geom"])
        dev = torch.zeros(16, dtype=torch.float64, device="cuda:0")
        params = btegpu.params_struct(case["T0"], case["dt"], case["maxtime"], case["N"], 1)
        r = btegpu.RtaResult()
        st = eng.lib.bte_rta_run_noalloc(eng.ctx, C.byref(params), C.c_void_p(dev.data_ptr()), C.byref(r))
        assert st == btegpu.BTE_ERR_STATE  # tables not built for these parameters yet
        eng.rta_run(case["T0"], case["dt"], case["maxtime"], case["N"], seed=1)
        big = btegpu.params_struct(case["T0"], 0.01, 100.0, case["N"], 1)  # 10000 bins
        st = eng.lib.bte_rta_run_noalloc(eng.ctx, C.byref(big), C.c_void_p(dev.data_ptr()), C.byref(r))
        assert st == btegpu.BTE_ERR_INPUT
        buf = C.create_string_buffer(256)
        eng.lib.bte_last_error(eng.ctx, buf, 256)
        assert b"allocation-free limit" in buf.value
    finally:
        eng.close()
