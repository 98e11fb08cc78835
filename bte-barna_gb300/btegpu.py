"""Python host interface of the GB300 engine (ctypes over libbtegpu.so).

Mirrors the reference's run interface for the RTA particle loop: load a mode
table and a geometry, then run with the <RTA_MC2d> parameters (T0, dt,
maxtime, N, ballistic) and read back the temperature / jx / jy arrays that
RTAMC2D writes to temperature_*.csv, jx_*.csv and jy_*.csv
(src/RTA_MC2D.cpp:2437-2471).  Errors raise BteError carrying the status code
that maps to the reference's exception types (include/exceptions.hpp).

The CUDA library is the only compute path: if it cannot be loaded this module
raises instead of falling back to anything else.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libbtegpu.so")

(BTE_OK, BTE_ERR_INPUT, BTE_ERR_VALUE, BTE_ERR_GEOMETRY, BTE_ERR_LIMIT, BTE_ERR_CUDA, BTE_ERR_STATE,
 BTE_ERR_CHECK) = range(8)
FLAG_CHECKS = 1
FLAG_GENERAL = 2
STATUS_NAMES = {0: "ok", 1: "input_error", 2: "value_error", 3: "geometry_error",
                4: "limit", 5: "cuda_error", 6: "state_error"}
MODE_REPLAY, MODE_PRODUCTION = 0, 1
SOURCE_WALLS, SOURCE_INITIAL = 0, 1

# Exported symbols declared in include/btegpu.h.
PUBLIC_SYMBOLS = ["bte_create", "bte_destroy", "bte_last_error", "bte_load_modes",
                  "bte_load_geometry", "bte_rta_run", "bte_set_tuning", "bte_query_sizes",
                  "bte_version", "bte_rta_run_noalloc", "bte_load_propagator", "bte_berta_run",
                  "bte_steady_run", "bte_load_materials", "bte_rta_adjoint", "bte_set_spectral",
                  "bte_get_spectral", "bte_set_groups", "bte_get_group_result", "bte_load_mode_tables",
                  "bte_interface_table"]


class BteError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code



class DeviceOpts(C.Structure):
    _fields_ = [("device", C.c_int32), ("verbose", C.c_int32)]


class ModeTable(C.Structure):
    _fields_ = [("nq", C.c_int32), ("nb", C.c_int32), ("grid", C.c_int32 * 3),
                ("omega", C.POINTER(C.c_double)), ("vg", C.POINTER(C.c_double)),
                ("w", C.POINTER(C.c_double)), ("dq", C.POINTER(C.c_double)),
                ("V", C.c_double), ("c_lat", C.c_double)]


class Geometry(C.Structure):
    _fields_ = [("nboxes", C.c_int32), ("npoints", C.POINTER(C.c_int32)),
                ("vertices", C.POINTER(C.c_double)), ("Teq", C.POINTER(C.c_double)),
                ("Tinit", C.POINTER(C.c_double)), ("reservoir", C.POINTER(C.c_int32)),
                ("thickness", C.c_double), ("translate_to", C.POINTER(C.c_int32)),
                ("translation", C.POINTER(C.c_double)), ("material", C.POINTER(C.c_int32))]


class RtaParams(C.Structure):
    _fields_ = [("T0", C.c_double), ("dt", C.c_double), ("maxtime", C.c_double),
                ("nparticles", C.c_int64), ("seed", C.c_uint64), ("mode", C.c_int32),
                ("source", C.c_int32), ("ballistic", C.c_int32), ("flags", C.c_int32),
                ("specularity", C.c_double), ("particle_begin", C.c_int64),
                ("particle_end", C.c_int64), ("flight_cap", C.c_int64)]


class RtaResult(C.Structure):
    _fields_ = [("nboxes", C.c_int32), ("nbins", C.c_int32),
                ("gz", C.POINTER(C.c_double)), ("gz_jx", C.POINTER(C.c_double)),
                ("gz_jy", C.POINTER(C.c_double)), ("temperature", C.POINTER(C.c_double)),
                ("jx", C.POINTER(C.c_double)), ("jy", C.POINTER(C.c_double)),
                ("exact", C.POINTER(C.c_int64)), ("Eeff", C.c_double),
                ("energy_rate", C.c_double), ("events", C.c_int64), ("wall_hits", C.c_int64),
                ("crossings", C.c_int64), ("absorbed", C.c_int64),
                ("specular_hits", C.c_int64), ("tally_updates", C.c_int64),
                ("kernel_ms", C.c_double), ("translations", C.c_int64),
                ("interface_hits", C.c_int64), ("interface_transmissions", C.c_int64)]


class Propagator(C.Structure):
    _fields_ = [("nmodes", C.c_int32), ("T", C.c_double), ("P", C.POINTER(C.c_double))]


class BertaParams(C.Structure):
    _fields_ = [("dt", C.c_double), ("maxtime", C.c_double), ("Eeff", C.c_double),
                ("T0", C.c_double), ("seed", C.c_uint64), ("mode", C.c_int32),
                ("rta", C.c_int32), ("cancel_every", C.c_int32), ("gradient_mode", C.c_int32),
                ("capacity", C.c_int64), ("on_step", C.c_void_p), ("user", C.c_void_p),
                ("gradient", C.c_double * 2)]


class BertaResult(C.Structure):
    _fields_ = [("nboxes", C.c_int32), ("nsteps", C.c_int32), ("ed", C.POINTER(C.c_double)),
                ("flux", C.POINTER(C.c_double)), ("nparticles", C.POINTER(C.c_int64)),
                ("histogram", C.POINTER(C.c_int32)), ("particle_steps", C.c_int64),
                ("branchings", C.c_int64), ("kernel_ms", C.c_double), ("phase_ms", C.c_double * 8),
                ("advance_in", C.c_int64), ("advance_out", C.c_int64)]

# the reference's beRTA timer buckets, in the order of bte_berta_result.phase_ms
BERTA_PHASES = ("advection", "cancelling", "generators", "histogram", "properties", "read_data",
                "saving", "scattering")


class SpectralResult(C.Structure):
    _fields_ = [("nloc", C.c_int32), ("nbins", C.c_int32), ("nomega", C.c_int32), ("nq", C.c_int32),
                ("omega", C.POINTER(C.c_double)), ("dT_omega", C.POINTER(C.c_double)),
                ("jx_omega", C.POINTER(C.c_double)), ("jy_omega", C.POINTER(C.c_double)),
                ("fd_q", C.POINTER(C.c_double)), ("q1bz", C.POINTER(C.c_double)),
                ("raw", C.POINTER(C.c_double)), ("steady", C.c_int32), ("reserved0", C.c_int32),
                ("counts", C.POINTER(C.c_double))]


class AdjointResult(C.Structure):
    _fields_ = [("phi", C.c_double), ("dphi_dtau", C.POINTER(C.c_double)), ("dphi_dp", C.c_double),
                ("events", C.c_int64), ("kernel_ms", C.c_double)]


class SteadyParams(C.Structure):
    _fields_ = [("T0", C.c_double), ("gradient", C.c_double * 2), ("eps_energy", C.c_double),
                ("eps_flux", C.c_double), ("nparticles", C.c_int64), ("seed", C.c_uint64),
                ("mode", C.c_int32), ("max_generations", C.c_int32), ("specularity", C.c_double),
                ("flags", C.c_int32), ("reserved0", C.c_int32)]


class SteadyResult(C.Structure):
    _fields_ = [("nboxes", C.c_int32), ("generations", C.c_int32), ("converged", C.c_int32),
                ("log_cap", C.c_int32), ("gz", C.POINTER(C.c_double)),
                ("gz_jx", C.POINTER(C.c_double)), ("gz_jy", C.POINTER(C.c_double)),
                ("temperature", C.POINTER(C.c_double)), ("jx", C.POINTER(C.c_double)),
                ("jy", C.POINTER(C.c_double)), ("exact", C.POINTER(C.c_int64)),
                ("log", C.POINTER(C.c_double)), ("Eeff", C.c_double), ("energy_rate", C.c_double),
                ("events", C.c_int64), ("wall_hits", C.c_int64), ("crossings", C.c_int64),
                ("absorbed", C.c_int64), ("translations", C.c_int64), ("scattered", C.c_int64),
                ("births", C.c_int64), ("lost", C.c_int64), ("kernel_ms", C.c_double),
                ("interface_hits", C.c_int64), ("interface_transmissions", C.c_int64)]


STEADY_KEYS = ("generations", "converged", "Eeff", "energy_rate", "events", "wall_hits", "crossings",
               "absorbed", "translations", "scattered", "births", "lost", "kernel_ms", "interface_hits",
               "interface_transmissions")


def steady_call(fn, nboxes, T0, gradient, N, seed=1, mode=MODE_PRODUCTION, eps_energy=-42.0,
                eps_flux=-42.0, max_generations=0, log_cap=100000, specularity=0.0, flags=0):
    """Fill SteadyParams / SteadyResult, call fn(params, result), return a dict.
    `flags`: FLAG_GENERAL for the evolparticle-faithful kernel."""
    p = SteadyParams()
    p.T0 = float(T0)
    p.gradient[0], p.gradient[1] = float(gradient[0]), float(gradient[1])
    p.eps_energy, p.eps_flux = float(eps_energy), float(eps_flux)
    p.nparticles, p.seed, p.mode = int(N), int(seed), int(mode)
    p.max_generations = int(max_generations)
    p.specularity = float(specularity)
    p.flags = int(flags)
    out = {k: np.zeros(nboxes) for k in ("gz", "gz_jx", "gz_jy", "temperature", "jx", "jy")}
    out["exact"] = np.zeros((nboxes, 3, 2), dtype=np.int64)
    out["log"] = np.zeros((log_cap, 4))
    r = SteadyResult()
    for k in ("gz", "gz_jx", "gz_jy", "temperature", "jx", "jy", "log"):
        setattr(r, k, _dptr(out[k]))
    r.exact = out["exact"].ctypes.data_as(C.POINTER(C.c_int64))
    r.log_cap = log_cap
    fn(p, r)
    for k in STEADY_KEYS:
        out[k] = getattr(r, k)
    out["log"] = out["log"][:min(r.generations, log_cap)].copy()
    return out


def berta_steps(dt: float, maxtime: float) -> int:
    """Iterations of `while (time <= maxtime) { ...; time += dt; }`."""
    t, n = 0.0, 0
    while t <= maxtime:
        n += 1
        t += dt
    return n


def berta_params(dt, maxtime, Eeff, T0=300.0, seed=1, rta=False, mode=MODE_PRODUCTION,
                 cancel_every=4, capacity=0, gradient=None):
    """`gradient`: None for the gradients of the boxes' Teq (the reference's
    default), or (gx, gy) in K/nm, the homogeneous <gradient x y>."""
    p = BertaParams()
    p.dt, p.maxtime, p.Eeff, p.T0, p.seed = float(dt), float(maxtime), float(Eeff), float(T0), int(seed)
    p.mode, p.rta, p.cancel_every, p.capacity = int(mode), int(bool(rta)), int(cancel_every), int(capacity)
    if gradient is not None:
        p.gradient_mode = 1
        p.gradient[0], p.gradient[1] = float(gradient[0]), float(gradient[1])
    return p


class Tuning(C.Structure):
    _fields_ = [("block_threads", C.c_int32), ("blocks_per_sm", C.c_int32),
                ("smem_tally", C.c_int32), ("particles_per_thread", C.c_int32)]


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def mode_struct(m: dict):
    """ModeTable over the arrays of a synth.mode_table dict (keeps refs)."""
    keep = {k: np.ascontiguousarray(m[k], dtype=np.float64) for k in ("omega", "vg", "w", "dq")}
    s = ModeTable()
    s.nq, s.nb = int(m["nq"]), int(m["nb"])
    for i in range(3):
        s.grid[i] = int(m["grid"][i])
    s.omega, s.vg, s.w, s.dq = (_dptr(keep[k]) for k in ("omega", "vg", "w", "dq"))
    s.V, s.c_lat = float(m["V"]), float(m["c_lat"])
    return s, keep


def geom_struct(g: dict):
    keep = {"npoints": np.ascontiguousarray(g["npoints"], dtype=np.int32),
            "vertices": np.ascontiguousarray(g["vertices"], dtype=np.float64),
            "Teq": np.ascontiguousarray(g["Teq"], dtype=np.float64),
            "Tinit": np.ascontiguousarray(g.get("Tinit", g["Teq"]), dtype=np.float64),
            "reservoir": np.ascontiguousarray(g["reservoir"], dtype=np.int32)}
    s = Geometry()
    s.nboxes = int(g["nboxes"])
    s.npoints = _iptr(keep["npoints"])
    s.vertices = _dptr(keep["vertices"])
    s.Teq = _dptr(keep["Teq"])
    s.Tinit = _dptr(keep["Tinit"])
    s.reservoir = _iptr(keep["reservoir"])
    s.thickness = float(g["thickness"])
    if g.get("translate_to") is not None:
        keep["translate_to"] = np.ascontiguousarray(g["translate_to"], dtype=np.int32)
        keep["translation"] = np.ascontiguousarray(g["translation"], dtype=np.float64).reshape(-1)
        s.translate_to = _iptr(keep["translate_to"])
        s.translation = _dptr(keep["translation"])
    if g.get("material") is not None:
        keep["material"] = np.ascontiguousarray(g["material"], dtype=np.int32)
        s.material = _iptr(keep["material"])
    return s, keep


def params_struct(T0, dt, maxtime, N, seed=1, mode=MODE_PRODUCTION, source=SOURCE_WALLS,
                  ballistic=False, specularity=0.0, begin=0, end=0, flags=0, flight_cap=0):
    """`flags`: FLAG_CHECKS for the checked grid kernel, FLAG_GENERAL for the
    evolparticle-faithful kernel on boxes off a grid; `flight_cap`: free
    flights per particle before BTE_ERR_LIMIT (0: the default)."""
    p = RtaParams()
    p.T0, p.dt, p.maxtime, p.nparticles, p.seed = float(T0), float(dt), float(maxtime), int(N), int(seed)
    p.mode, p.source, p.ballistic = int(mode), int(source), int(bool(ballistic))
    p.specularity, p.particle_begin, p.particle_end = float(specularity), int(begin), int(end)
    p.flags, p.flight_cap = int(flags), int(flight_cap)
    return p


_lib = None


def load_library(path: str = LIB_PATH):
    """Load libbtegpu.so (raises OSError when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OSError(f"{path} is missing: run __graft_entry__.build() first")
    lib = C.CDLL(path)
    vp = C.c_void_p
    lib.bte_create.argtypes = [C.POINTER(vp), C.POINTER(DeviceOpts)]
    lib.bte_destroy.argtypes = [vp]
    lib.bte_last_error.argtypes = [vp, C.c_char_p, C.c_size_t]
    lib.bte_load_modes.argtypes = [vp, C.POINTER(ModeTable)]
    lib.bte_load_geometry.argtypes = [vp, C.POINTER(Geometry)]
    lib.bte_rta_run.argtypes = [vp, C.POINTER(RtaParams), C.POINTER(RtaResult)]
    lib.bte_set_tuning.argtypes = [vp, C.POINTER(Tuning)]
    lib.bte_query_sizes.argtypes = [vp, C.POINTER(RtaParams), C.POINTER(C.c_int32),
                                    C.POINTER(C.c_int32), C.POINTER(C.c_int64)]
    lib.bte_version.restype = C.c_int32
    lib.bte_load_propagator.argtypes = [vp, C.POINTER(Propagator)]
    lib.bte_load_propagator.restype = C.c_int
    lib.bte_berta_run.argtypes = [vp, C.POINTER(BertaParams), C.POINTER(BertaResult)]
    lib.bte_berta_run.restype = C.c_int
    lib.bte_load_materials.argtypes = [vp, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                       C.POINTER(C.c_double)]
    lib.bte_load_materials.restype = C.c_int
    lib.bte_load_mode_tables.argtypes = [vp, C.c_int32, C.POINTER(ModeTable), C.POINTER(C.c_double)]
    lib.bte_load_mode_tables.restype = C.c_int
    lib.bte_interface_table.argtypes = [C.POINTER(ModeTable), C.POINTER(ModeTable), C.c_double, C.c_double,
                                        C.c_double, C.c_double, C.c_double, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                        C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_double)]
    lib.bte_interface_table.restype = C.c_int
    lib.bte_set_spectral.argtypes = [vp, C.c_int32, C.POINTER(C.c_int32), C.c_int32]
    lib.bte_set_spectral.restype = C.c_int
    lib.bte_get_spectral.argtypes = [vp, C.POINTER(SpectralResult)]
    lib.bte_get_spectral.restype = C.c_int
    lib.bte_rta_adjoint.argtypes = [vp, C.POINTER(RtaParams), C.POINTER(C.c_double),
                                    C.POINTER(AdjointResult)]
    lib.bte_rta_adjoint.restype = C.c_int
    lib.bte_steady_run.argtypes = [vp, C.POINTER(SteadyParams), C.POINTER(SteadyResult)]
    lib.bte_steady_run.restype = C.c_int
    lib.bte_rta_run_noalloc.argtypes = [vp, C.POINTER(RtaParams), C.c_void_p, C.POINTER(RtaResult)]
    lib.bte_rta_run_noalloc.restype = C.c_int
    lib.bte_set_groups.argtypes = [vp, C.c_int32]
    lib.bte_set_groups.restype = C.c_int
    lib.bte_get_group_result.argtypes = [vp, C.c_int32, C.POINTER(RtaResult)]
    lib.bte_get_group_result.restype = C.c_int
    for f in ("bte_create", "bte_destroy", "bte_last_error", "bte_load_modes",
              "bte_load_geometry", "bte_rta_run", "bte_set_tuning", "bte_query_sizes"):
        getattr(lib, f).restype = C.c_int
    lib.btegpu_debug_geometry.argtypes = [C.POINTER(Geometry), C.POINTER(C.c_double), C.c_longlong]
    lib.btegpu_debug_geometry.restype = C.c_longlong
    lib.btegpu_debug_grid.argtypes = [C.POINTER(Geometry), C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.btegpu_debug_lambert.argtypes = [C.POINTER(ModeTable), C.POINTER(Geometry),
                                         C.POINTER(C.c_longlong), C.c_int]
    lib.btegpu_debug_lambert.restype = C.c_longlong
    lib.btegpu_debug_log.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_longlong]
    lib.btegpu_debug_frame.argtypes = [C.c_double, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_int),
                                       C.c_int, C.c_int, C.c_char_p, C.c_longlong]
    lib.btegpu_debug_frame.restype = C.c_longlong
    _lib = lib
    return lib


class Engine:
    """One engine context on one CUDA device."""

    def __init__(self, device: int = 0, verbose: bool = False):
        self.lib = load_library()
        self.ctx = C.c_void_p()
        opts = DeviceOpts(device, int(verbose))
        st = self.lib.bte_create(C.byref(self.ctx), C.byref(opts))
        if st != BTE_OK:
            buf = C.create_string_buffer(512)
            self.lib.bte_last_error(None, buf, 512)
            raise BteError(st, buf.value.decode())
        self._keep = {}

    def close(self):
        if self.ctx:
            self.lib.bte_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != BTE_OK:
            buf = C.create_string_buffer(1024)
            self.lib.bte_last_error(self.ctx, buf, 1024)
            raise BteError(st, buf.value.decode())

    def load_modes(self, m: dict):
        s, keep = mode_struct(m)
        self._check(self.lib.bte_load_modes(self.ctx, C.byref(s)))
        self._keep["modes"] = keep

    def load_mode_tables(self, tables, thickness=None):
        """Several crystals: mode table k for the boxes of material k
        (geometry "material"), diffuse mismatch at their contacts.
        `thickness`: each crystal's thickness in nm (None: the geometry's)."""
        arr = (ModeTable * len(tables))()
        keep = []
        for i, t in enumerate(tables):
            s, k = mode_struct(t)
            arr[i] = s
            keep.append(k)
        th = None if thickness is None else np.ascontiguousarray(np.asarray(thickness, dtype=float))
        if th is not None and th.size != len(tables):
            raise ValueError("one thickness per mode table")
        self._check(self.lib.bte_load_mode_tables(self.ctx, len(tables), arr,
                                                  _dptr(th) if th is not None else None))
        keep.append(th)
        self._keep["modes"] = {"omega": np.concatenate([np.asarray(t["omega"], float) for t in tables])}
        self._keep["crystals"] = (arr, keep)

    def load_geometry(self, g: dict):
        s, keep = geom_struct(g)
        self._check(self.lib.bte_load_geometry(self.ctx, C.byref(s)))
        self._keep["geom"] = keep
        self.nboxes = int(g["nboxes"])

    def set_tuning(self, block_threads=0, blocks_per_sm=0, smem_tally=1, particles_per_thread=0):
        t = Tuning(block_threads, blocks_per_sm, smem_tally, particles_per_thread)
        self._check(self.lib.bte_set_tuning(self.ctx, C.byref(t)))

    def rta_run(self, T0, dt, maxtime, N, seed=1, mode=MODE_PRODUCTION, source=SOURCE_WALLS,
                ballistic=False, specularity=0.0, begin=0, end=0, raw=True, exact=False, flags=0,
                flight_cap=0):
        p = params_struct(T0, dt, maxtime, N, seed, mode, source, ballistic, specularity, begin, end,
                          flags, flight_cap)
        nbx, nbn, nm = C.c_int32(), C.c_int32(), C.c_int64()
        self._check(self.lib.bte_query_sizes(self.ctx, C.byref(p), C.byref(nbx), C.byref(nbn), C.byref(nm)))
        shape = (nbx.value, nbn.value)
        out = {k: np.zeros(shape) for k in ("temperature", "jx", "jy")}
        r = RtaResult()
        r.temperature, r.jx, r.jy = (_dptr(out[k]) for k in ("temperature", "jx", "jy"))
        if raw:
            for k in ("gz", "gz_jx", "gz_jy"):
                out[k] = np.zeros(shape)
            r.gz, r.gz_jx, r.gz_jy = (_dptr(out[k]) for k in ("gz", "gz_jx", "gz_jy"))
        if exact:
            out["exact"] = np.zeros(shape + (3, 2), dtype=np.int64)
            r.exact = out["exact"].ctypes.data_as(C.POINTER(C.c_int64))
        self._check(self.lib.bte_rta_run(self.ctx, C.byref(p), C.byref(r)))
        for k in ("Eeff", "energy_rate", "events", "wall_hits", "crossings", "absorbed",
                  "specular_hits", "tally_updates", "kernel_ms", "translations", "interface_hits",
                  "interface_transmissions"):
            out[k] = getattr(r, k)
        return out


def _engine_load_propagator(self, P: np.ndarray, T: float = 300.0):
    """Propagator over modes 3..n-1, column j = outgoing distribution of mode j + 3."""
    Pf = np.asfortranarray(P, dtype=np.float64)
    flat = np.ascontiguousarray(Pf.ravel(order="F"))
    s = Propagator(int(P.shape[0]), float(T), _dptr(flat))
    self._check(self.lib.bte_load_propagator(self.ctx, C.byref(s)))


def _engine_berta_run(self, dt, maxtime, Eeff, T0=300.0, seed=1, rta=False, cancel_every=4,
                      capacity=0, histogram=False, gradient=None):
    """beRTAMC2D loop: per step ed [s, box] (J m^-3), flux [s, box, 2], N [s].
    `gradient` (K/nm): the homogeneous <gradient x y> source term."""
    p = berta_params(dt, maxtime, Eeff, T0, seed, rta, MODE_PRODUCTION, cancel_every, capacity,
                     gradient)
    nsteps = berta_steps(dt, maxtime)
    nbx = self.nboxes
    ed = np.zeros((nsteps + 1, nbx))
    flux = np.zeros((nsteps + 1, nbx, 2))
    npart = np.zeros(nsteps + 1, dtype=np.int64)
    r = BertaResult()
    r.ed, r.flux = _dptr(ed), _dptr(flux)
    r.nparticles = npart.ctypes.data_as(C.POINTER(C.c_int64))
    H = None
    if histogram:
        n = int(self._keep["modes"]["omega"].size)
        H = np.zeros((nbx, n), dtype=np.int32)
        r.histogram = H.ctypes.data_as(C.POINTER(C.c_int32))
    self._check(self.lib.bte_berta_run(self.ctx, C.byref(p), C.byref(r)))
    return {"ed": ed, "flux": flux, "nparticles": npart, "H": H, "nsteps": r.nsteps,
            "particle_steps": r.particle_steps, "branchings": r.branchings, "kernel_ms": r.kernel_ms,
            "phase_ms": dict(zip(BERTA_PHASES, list(r.phase_ms))),
            "advance_in": r.advance_in, "advance_out": r.advance_out}


def _engine_steady_run(self, T0, gradient, N, seed=1, mode=MODE_PRODUCTION, eps_energy=-42.0,
                       eps_flux=-42.0, max_generations=0, log_cap=100000, specularity=0.0, flags=0):
    """Steady state of a periodic structure under `gradient` (K/nm)."""
    def call(p, r):
        self._check(self.lib.bte_steady_run(self.ctx, C.byref(p), C.byref(r)))
    return steady_call(call, self.nboxes, T0, gradient, N, seed, mode, eps_energy, eps_flux,
                       max_generations, log_cap, specularity, flags)


def _engine_load_materials(self, w_list, T0_list, share=None):
    """Materials for batched runs: rates w_list[m] (per mode) at T0_list[m];
    optional particle share per material (walls source)."""
    if not w_list:
        self._check(self.lib.bte_load_materials(self.ctx, 0, None, None, None))
        return
    W = np.ascontiguousarray(np.stack([np.asarray(w, dtype=np.float64) for w in w_list]))
    T = np.ascontiguousarray(np.asarray(T0_list, dtype=np.float64))
    S = None if share is None else np.ascontiguousarray(np.asarray(share, dtype=np.float64))
    self._keep["materials"] = (W, T, S)
    self._check(self.lib.bte_load_materials(self.ctx, len(w_list), _dptr(W), _dptr(T),
                                            None if S is None else _dptr(S)))


def _engine_rta_adjoint(self, weights, T0, dt, maxtime, N, seed=1, source=SOURCE_WALLS,
                       specularity=0.0, ballistic=False, begin=0, end=0):
    """dPhi/dtau per mode and dPhi/dp of Phi = sum(weights * raw tallies),
    weights shaped [nboxes, nbins, 3] (gz, gz_jx, gz_jy)."""
    p = params_struct(T0, dt, maxtime, N, seed, MODE_PRODUCTION, source, ballistic, specularity,
                      begin, end)
    W = np.ascontiguousarray(weights, dtype=np.float64)
    n = int(self._keep["modes"]["omega"].size)
    g = np.zeros(n)
    r = AdjointResult()
    r.dphi_dtau = _dptr(g)
    self._check(self.lib.bte_rta_adjoint(self.ctx, C.byref(p), _dptr(W), C.byref(r)))
    return {"phi": r.phi, "dphi_dtau": g, "dphi_dp": r.dphi_dp, "events": r.events,
            "kernel_ms": r.kernel_ms}


def _engine_set_spectral(self, boxes, nomega=500):
    """Spectral decomposition at the given boxes for the following runs."""
    b = np.ascontiguousarray(np.asarray(boxes, dtype=np.int32))
    self._keep["spectral"] = b
    self._check(self.lib.bte_set_spectral(self.ctx, len(b), _iptr(b) if len(b) else None, int(nomega)))
    self._spec_nomega = int(nomega)


def _engine_get_spectral(self, nbins=1):
    """The last run's spectral outputs (arrays [nloc, nbins, ...]; a steady
    run has one bin and also returns `counts` [nloc, nmodes], the signed
    segments per mode)."""
    nloc = len(self._keep["spectral"])
    nw = self._spec_nomega
    n = int(self._keep["modes"]["omega"].size)
    out = {"omega": np.zeros((nloc, nw)), "dT_omega": np.zeros((nloc, nbins, nw)),
           "jx_omega": np.zeros((nloc, nbins, nw)), "jy_omega": np.zeros((nloc, nbins, nw)),
           "raw": np.zeros((nloc, nbins, n)), "counts": np.zeros((nloc, n))}
    r = SpectralResult()
    self._check(self.lib.bte_get_spectral(self.ctx, C.byref(r)))
    if r.nbins != nbins:
        raise ValueError(f"the last run has {r.nbins} spectral bins, not {nbins}")
    for k in ("omega", "dT_omega", "jx_omega", "jy_omega", "raw", "counts"):
        setattr(r, k, _dptr(out[k]))
    out["fd_q"] = np.zeros((nloc, nbins, r.nq))
    out["q1bz"] = np.zeros((r.nq, 2))
    r.fd_q, r.q1bz = _dptr(out["fd_q"]), _dptr(out["q1bz"])
    self._check(self.lib.bte_get_spectral(self.ctx, C.byref(r)))
    out["steady"] = bool(r.steady)
    return out


def _engine_set_groups(self, ngroups: int):
    """Replica groups of the following production grid runs (0 or 1: off)."""
    self._check(self.lib.bte_set_groups(self.ctx, int(ngroups)))


def _engine_group_result(self, group: int, shape, raw: bool = False, keys=("temperature", "jx", "jy")):
    """Outputs of one replica group of the last run, scaled to the whole run
    (`keys`: which of temperature, jx, jy to form)."""
    out = {k: np.zeros(shape) for k in keys}
    r = RtaResult()
    for k in keys:
        setattr(r, k, _dptr(out[k]))
    if raw:
        for k in ("gz", "gz_jx", "gz_jy"):
            out[k] = np.zeros(shape)
        r.gz, r.gz_jx, r.gz_jy = (_dptr(out[k]) for k in ("gz", "gz_jx", "gz_jy"))
    self._check(self.lib.bte_get_group_result(self.ctx, int(group), C.byref(r)))
    out["Eeff"] = r.Eeff
    return out


Engine.set_groups = _engine_set_groups
Engine.group_result = _engine_group_result
Engine.set_spectral = _engine_set_spectral
Engine.get_spectral = _engine_get_spectral
Engine.rta_adjoint = _engine_rta_adjoint
Engine.load_materials = _engine_load_materials
Engine.steady_run = _engine_steady_run
Engine.load_propagator = _engine_load_propagator
Engine.berta_run = _engine_berta_run


def interface_table(A: dict, B: dict, normal, thickness, Tref: float):
    """The engine's diffuse mismatch table from mode table A to B (host
    code, no device): per incident mode of A, arrays (side out, mode out,
    cumulative).  `thickness`: one value for both crystals' boxes, or the
    pair (A's, B's)."""
    lib = load_library()
    sa, ka = mode_struct(A)
    sb, kb = mode_struct(B)
    na = int(np.asarray(A["omega"]).size)
    first = np.zeros(na + 1, dtype=np.int64)
    ne = np.zeros(1, dtype=np.int64)
    ta, tb = (thickness, thickness) if np.isscalar(thickness) else thickness
    args = (C.byref(sa), C.byref(sb), float(normal[0]), float(normal[1]), float(ta), float(tb), float(Tref))
    lp = C.POINTER(C.c_int64)
    st = lib.bte_interface_table(*args, first.ctypes.data_as(lp), ne.ctypes.data_as(lp), None, None, None)
    if st != 0:
        raise BteError(st, _host_error(lib))
    side = np.zeros(int(ne[0]), dtype=np.int32)
    mode = np.zeros(int(ne[0]), dtype=np.int32)
    cum = np.zeros(int(ne[0]))
    st = lib.bte_interface_table(*args, first.ctypes.data_as(lp), ne.ctypes.data_as(lp),
                                 side.ctypes.data_as(C.POINTER(C.c_int32)), mode.ctypes.data_as(C.POINTER(C.c_int32)),
                                 cum.ctypes.data_as(C.POINTER(C.c_double)))
    if st != 0:
        raise BteError(st, _host_error(lib))
    return [(side[first[i]:first[i + 1]], mode[first[i]:first[i + 1]], cum[first[i]:first[i + 1]]) for i in range(na)]


def _host_error(lib) -> str:
    buf = C.create_string_buffer(512)
    lib.bte_last_error(None, buf, 512)
    return buf.value.decode()

def debug_geometry(g: dict) -> np.ndarray:
    lib = load_library()
    s, keep = geom_struct(g)
    n = lib.btegpu_debug_geometry(C.byref(s), None, 0)
    if n < 0:
        raise BteError(BTE_ERR_GEOMETRY, "geometry build failed")
    out = np.zeros(n)
    lib.btegpu_debug_geometry(C.byref(s), _dptr(out), n)
    return out


def debug_grid(g: dict):
    lib = load_library()
    s, keep = geom_struct(g)
    nx, ny = C.c_int(), C.c_int()
    r = lib.btegpu_debug_grid(C.byref(s), C.byref(nx), C.byref(ny))
    return r, nx.value, ny.value


def debug_lambert(m: dict, g: dict, maxclass: int = 16):
    lib = load_library()
    ms, k1 = mode_struct(m)
    gs, k2 = geom_struct(g)
    nnz = np.zeros(maxclass, dtype=np.int64)
    tot = lib.btegpu_debug_lambert(C.byref(ms), C.byref(gs),
                                   nnz.ctypes.data_as(C.POINTER(C.c_longlong)), maxclass)
    return tot, nnz


def debug_frame(time: float, Eeff: float, temps, H: np.ndarray) -> bytes:
    lib = load_library()
    t = np.ascontiguousarray(temps, dtype=np.float64)
    Hc = np.ascontiguousarray(H, dtype=np.int32)
    n = lib.btegpu_debug_frame(time, Eeff, _dptr(t), Hc.ctypes.data_as(C.POINTER(C.c_int)),
                               Hc.shape[0], Hc.shape[1], None, 0)
    buf = C.create_string_buffer(int(n))
    lib.btegpu_debug_frame(time, Eeff, _dptr(t), Hc.ctypes.data_as(C.POINTER(C.c_int)),
                           Hc.shape[0], Hc.shape[1], buf, n)
    return buf.raw[:n]


def split_frames(data: bytes):
    """Frames of a properties.msgpack.bin file ("<size>#<msgpack>" ..., "0#")."""
    out, i = [], 0
    while i < len(data):
        j = data.index(b"#", i)
        size = int(data[i:j])
        if size == 0:
            break
        out.append(data[j + 1:j + 1 + size])
        i = j + 1 + size
    return out


def debug_log(x: np.ndarray) -> np.ndarray:
    lib = load_library()
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros_like(x)
    lib.btegpu_debug_log(_dptr(x), _dptr(y), x.size)
    return y
