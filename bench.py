"""Throughput benchmark of the RTA particle loop on GB300.

Metric: particle-flight events per second (one event = one free-flight draw,
random_dt in src/RTA_MC2D.cpp:2271-2274, with its cell crossings, tally
updates and the closing scatter, wall reflection or absorption).

Workload (default "c1"): the transient benchmark configuration at scale:
64x64 q-grid x 9 branches (36864 modes), 2 um x 500 nm rectangle of 100x25
cells of 20 nm, a 200 nm-diameter staircase pore, specular fraction 0.3,
1 K Gaussian hot spot (sigma 50 nm), 200 time bins to 10 ns, N = 1e8
particles.  One step = one batch of the run's particles (a contiguous slice
of the 1e8, --per-step particles) carried through their whole 10 ns life.
Inputs are seeded synthetic mode tables (no material database exists here).

  value  events / device time of the kernel (CUDA events on the launching
         stream, tables resident in HBM, L2 flushed between steps)
  e2e    events / wall time of the C-ABI call bte_rta_run with host output
         buffers (tally D2H and post-processing inside the timed region)

--impl reference times the CPU restatement of the reference loop (oracle/)
on the host cores on bounded samples of the same workload.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "bte-barna_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

import numpy as np  # noqa: E402

METRIC = "particle-flight events/s"
UNIT = "events/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c1", choices=["c1", "c0", "c2", "c3", "c4", "bar"])
    ap.add_argument("--sweep-tol", type=float, default=0.01, help="3 sigma / kappa target (c3)")
    ap.add_argument("--sweep-seconds", type=float, default=240.0, help="time cap per arm (c3)")
    ap.add_argument("--per-step", type=int, default=0, help="particles per step")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the time-to-1%% summaries of the sweep and the gradient")
    ap.add_argument("--extra-seconds", type=float, default=30.0,
                    help="time cap of each arm of those summaries")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--berta-eeff", type=float, default=0.0,
                    help="c2: this Eeff (J) instead of the calibration towards 1e7 particles alive; "
                         "the line then lists the particles alive at every step of the first timed run")
    return ap.parse_args()


def workload(name):
    import synth
    if name == "c1":
        c = synth.config1()
        c["label"] = ("transient RTA at scale: 64x64 q x 9 branches (36864 modes), 2um x 500nm, "
                      "100x25 cells of 20nm, 200nm staircase pore, p=0.3, 1K hot spot sigma 50nm, "
                      "200 bins to 10ns, N=1e8")
        c["per_step"] = 2_000_000
    elif name == "bar":
        # boxes off a grid (periodic boxes): the convex-polygon kernel
        c = synth.config0()
        c["geom"] = synth.periodic_bar_geometry()
        c["dt"], c["maxtime"], c["N"] = 10.0, 1000.0, 10_000_000
        c["label"] = ("periodic bar, convex-polygon kernel: 32x32 q x 6 branches (6144 modes), "
                      "20nm x 40nm bar of 10 strips between periodic side boxes, 302/300K "
                      "reservoirs below and above, 100 bins of 10ps, N=1e7, a step is the whole run")
        c["per_step"] = 10_000_000
    else:
        c = synth.config0()
        c["label"] = ("plain RTA ribbon: 32x32 q x 6 branches (6144 modes), 1um x 100nm, 50 cells, "
                      "301/299K reservoirs, diffuse walls, 100 bins of 10ps, N=1e6")
        c["per_step"] = 1_000_000
    return c


def source_of(c):
    import btegpu
    return btegpu.SOURCE_INITIAL if c["source"] == "initial" else btegpu.SOURCE_WALLS


# ----------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------- roofline
def algorithmic_bytes(events, tallies, particles):
    # per event: mode record (vx, vy, tau: 24 B) + one alias/CDF probe (12 B);
    # per tally update: 3 FP64 read-modify-writes (48 B); per particle: state
    # load + store (144 B)
    return 36.0 * events + 48.0 * tallies + 144.0 * particles


def measured_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def nsm_of_device():
    import torch
    return torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count


def profile_figures():
    """ncu figures of the grid kernel from the committed capture summary:
    DRAM bytes per launch = fixed (tables, first touch) + per event, and the
    FP64 thread operations per event."""
    p = os.path.join(REPO, "profiles", "rta_prod_grid_c1.json")
    if os.path.exists(p):
        try:
            return json.load(open(p))
        except (ValueError, OSError):
            return {}
    return {}


# be_advance: a particle read is x, y (FP64), mode, box, sign (int32): 28 B;
# a particle written is the same 28 B plus the propagator column entry (or
# resampling alias entry) drawn for it, 8 B.  The histogram's atomics hit
# a 1.3 MB array that stays in L2.
BE_IN_BYTES = 28
BE_OUT_BYTES = 36


def berta_profile_figures():
    """ncu figures of be_advance from the committed capture summary: DRAM
    bytes of one existing-particle launch per particle it read."""
    p = os.path.join(REPO, "profiles", "be_advance_c2.json")
    if os.path.exists(p):
        try:
            return json.load(open(p))
        except (ValueError, OSError):
            return {}
    return {}


# ----------------------------------------------------------------- CPU leg
def cpu_sample(c, seconds, nthreads, seed=7, offset=0):
    """Time the restatement on a bounded slice of the workload's particles."""
    import pyoracle
    # calibrate on a small slice, then size the sample to ~`seconds` of the
    # particle loop (the restatement times its loop without table set-up)
    probe = 64 * nthreads
    r = pyoracle.rta_run(c, N=c["N"], seed=seed, nthreads=nthreads, begin=offset, end=offset + probe)
    dt = r["loop_seconds"]
    n = int(max(probe, min(probe * seconds / max(dt, 1e-3), 50_000_000)))
    r = pyoracle.rta_run(c, N=c["N"], seed=seed, nthreads=nthreads, begin=offset, end=offset + n)
    return r["events"], r["loop_seconds"], n


def reference_arm(args, c, rank, world):
    if rank != 0:
        return 0
    import pyoracle
    nthreads = os.cpu_count() or 1
    pyoracle.load()
    per_step = max(1, args.per_step) if args.per_step else None
    # W warm-up + K timed samples; each step a bounded slice sized to ~cpu_seconds / steps
    secs = max(2.0, args.cpu_seconds / max(args.steps, 1))
    ev_tot, t_tot, n_tot = 0, 0.0, 0
    off = 0
    for i in range(args.warmup + args.steps):
        if per_step:
            r = pyoracle.rta_run(c, N=c["N"], seed=11, nthreads=nthreads, begin=off, end=off + per_step)
            ev, dt, n = r["events"], r["loop_seconds"], per_step
        else:
            ev, dt, n = cpu_sample(c, secs, nthreads, seed=11, offset=off)
        off += n
        if i >= args.warmup:
            ev_tot += ev
            t_tot += dt
            n_tot += n
    v = ev_tot / t_tot
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_tot / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": c["label"], "particles_per_step": n_tot // args.steps},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": nthreads, "kind": "port",
                             "sample": f"{n_tot} particles of the workload over {args.steps} steps"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ----------------------------------------------------------------- GPU leg
def run_berta(args, rank, world, local):
    """beRTAMC2D on the plain ribbon (6144 modes, 50 cells, 301/299 K
    reservoirs) with a synthetic 6141 x 6141 propagator exp(B dt), dt = 1 ps,
    100 steps; Eeff calibrated so that about 1e7 particles are alive at the
    last step.  A step of this line is one whole 100-step run; the metric is
    particle-steps (advect + scatter draw) per second."""
    import torch
    import btegpu
    import synth
    if world > 1 and rank != 0:
        return 0  # one replica is enough for this extra workload line
    torch.cuda.set_device(local)
    c = synth.config0()
    eng = btegpu.Engine(local)
    eng.load_modes(c["modes"])
    eng.load_geometry(c["geom"])
    t0 = time.perf_counter()
    P = synth.propagator(c["modes"], dt=1.0, T=300.0, use_torch=True)
    eng.load_propagator(P, 300.0)
    build_s = time.perf_counter() - t0
    dt, maxtime, target = 1.0, 99.0, 10_000_000
    E = args.berta_eeff if args.berta_eeff > 0 else 1e-21
    for _ in range(0 if args.berta_eeff > 0 else 8):  # about 1 / Eeff, less where cancellation bites: iterate
        r = eng.berta_run(dt, maxtime, E, seed=7)
        n_end = int(r["nparticles"][-1])
        if n_end < 10_000:
            E = E / 100.0
            continue
        if abs(n_end / target - 1.0) < 0.15:
            break
        E = E * (n_end / target) ** 1.5
    for w in range(args.warmup):
        eng.berta_run(dt, maxtime, E, seed=100 + w)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    ps = 0
    kern_ms = 0.0
    e2e_s = 0.0
    alive = []
    adv_ms = 0.0
    adv_bytes = 0.0
    adv_in = 0
    phase_sum = {}
    by_step = None
    for k in range(args.steps):
        flush.fill_(float(k))
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        r = eng.berta_run(dt, maxtime, E, seed=200 + k)
        e2e_s += time.perf_counter() - t1
        ps += int(r["particle_steps"])
        kern_ms += float(r["kernel_ms"])
        alive.append(int(r["nparticles"][-1]))
        # be_advance: the advection and scattering phases (two launches a step)
        adv_ms += r["phase_ms"]["advection"] + r["phase_ms"]["scattering"]
        adv_bytes += BE_IN_BYTES * r["advance_in"] + BE_OUT_BYTES * r["advance_out"]
        adv_in += int(r["advance_in"])
        for ph, v in r["phase_ms"].items():
            phase_sum[ph] = phase_sum.get(ph, 0.0) + v
        if by_step is None:
            by_step = [int(v) for v in r["nparticles"]]
    torch.cuda.synchronize()
    clk = clocks.stop()
    nbx = int(c["geom"]["nboxes"])
    nsteps = btegpu.berta_steps(dt, maxtime)
    launches = 2 * nsteps * args.steps
    peak, peak_kind = measured_peaks()
    achieved = adv_bytes / (adv_ms * 1e-3) / 1e9
    prof = berta_profile_figures()
    traffic = (prof["dram_bytes_per_particle_in"] * adv_in / launches
               if prof.get("dram_bytes_per_particle_in") else None)
    line = {
        "metric": "beRTA particle-steps/s", "value": ps / (kern_ms * 1e-3), "unit": "particle-steps/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * e2e_s / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded mode table and propagator, no database)",
        "config": {"workload": "beRTAMC2D on the plain ribbon: 32x32 q x 6 branches (6144 modes), "
                               "6141x6141 propagator exp(B dt), dt=1 ps, 100 steps, 1 um x 100 nm, "
                               "50 cells, 301/299K reservoirs, ~1e7 particles alive",
                   "Eeff_J": E, "alive_at_end": int(np.mean(alive)),
                   "particle_steps_per_run": ps // args.steps, "propagator_build_s": build_s,
                   "l2": "flushed between runs (256 MB write)", "parallelism": "replicas x1"},
        "e2e": {"value": ps / e2e_s, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": (nsteps + 1) * (nbx * 3 + 1) * 8},
        "kernel_ms_per_step": kern_ms / args.steps,
        # device time of the reference's timer buckets per 100-step run
        # (CUDA events at the phase borders of every step)
        "phase_ms_per_step": {ph: v / args.steps for ph, v in phase_sum.items()},
        "roofline": {"bound": "hbm", "kernel": "be_advance", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind + " (copy burst)",
                     "traffic": traffic,
                     "algorithmic_bytes_per_launch": adv_bytes / launches,
                     "launch_ms": adv_ms / launches,
                     "per_unit": f"{BE_IN_BYTES} B per particle read + {BE_OUT_BYTES} B per particle written"},
        "clocks": clk,
    }
    if args.berta_eeff > 0:
        line["nparticles_by_step"] = by_step
    print(json.dumps(line))
    eng.close()
    return 0


class SweepStats:
    """Batch means of kappa_eff per case: replicas are independent runs."""

    def __init__(self, n):
        self.k = [[] for _ in range(n)]

    def add(self, i, kappa):
        self.k[i].append(kappa)

    def rel3(self, i):
        v = np.asarray(self.k[i])
        if len(v) < 4:
            return float("inf")
        return 3.0 * v.std(ddof=1) / np.sqrt(len(v)) / abs(v.mean())

    def mean(self, i):
        return float(np.mean(self.k[i])) if self.k[i] else float("nan")


class AdaptiveShares:
    """Particle allocation from measured variances, for runs whose launches
    deal their particles to G replica groups.  A case starts with a fraction
    of its budget; each round adds its (particles, variance of the round's
    mean) and the particle-weighted kappa mean; the next round gives it what
    its pooled per-particle variance still asks for, with margin, and at
    least a quarter of what it has used (an estimate from few groups may say
    a case is nearly there while it is not)."""

    def __init__(self, budgets, first_frac, nmin, tol, groups):
        n = len(budgets)
        self.G = groups
        self.tol = tol
        self.nmin = nmin
        self.need = np.maximum(np.asarray(budgets, float) * first_frac, nmin)
        self.w_sum = np.zeros(n)
        self.wk_sum = np.zeros(n)
        self.rounds = [[] for _ in range(n)]
        self.kappa = np.full(n, np.nan)
        self.rel = np.full(n, np.inf)

    def alloc(self, i):
        return max(self.need[i], self.nmin)

    def add(self, i, n_i, kg):
        """Adds one round of case i (n_i particles, per-group kappa kg);
        returns True once 3 sigma / kappa <= tol."""
        kg = np.asarray(kg, float)
        self.rounds[i].append((n_i, kg.var(ddof=1) / self.G))
        self.w_sum[i] += n_i
        self.wk_sum[i] += n_i * kg.mean()
        self.kappa[i] = self.wk_sum[i] / self.w_sum[i]
        var = sum((n / self.w_sum[i]) ** 2 * v for n, v in self.rounds[i])
        self.rel[i] = 3.0 * np.sqrt(var) / abs(self.kappa[i])
        if self.rel[i] <= self.tol:
            return True
        s2 = np.mean([v * n for n, v in self.rounds[i]])
        total = 9.0 * s2 / (self.tol * self.kappa[i]) ** 2
        self.need[i] = max(1.3 * (total - self.w_sum[i]), 0.25 * self.w_sum[i], self.nmin)
        return False


def run_sweep(args, rank, world, local):
    """The C3 workload line (see sweep_arms)."""
    import torch
    if world > 1 and rank != 0:
        return 0
    torch.cuda.set_device(local)
    print(json.dumps(sweep_arms(local, args.sweep_tol, args.sweep_seconds)))
    return 0


def kappa_agreement(kap_b, rel_b, sp):
    """Largest |z| between the batched and the per-case kappa_eff over the
    cases both arms converged (sigma of each from its own batch means)."""
    zs = []
    for i in range(len(kap_b)):
        v = np.asarray(sp.k[i])
        if len(v) < 4 or not np.isfinite(rel_b[i]):
            continue
        sb = rel_b[i] * abs(kap_b[i]) / 3.0
        spl = v.std(ddof=1) / np.sqrt(len(v))
        zs.append(abs(kap_b[i] - v.mean()) / np.sqrt(sb ** 2 + spl ** 2))
    return float(max(zs)) if zs else None


def sweep_arms(local, tol, cap, first_frac=0.25, groups=8, plain=True):
    """The batched sweep: 64 ribbons (16 widths 20 nm - 2 um x 4 temperatures,
    1 um long, p = 0, reservoirs at T +- 1 K) with budgets N_w = 1e5 100^(k/15).
    Each arm runs until every case's kappa_eff has 3 sigma / kappa <= tol.
    Plain: each case alone, one context per temperature, independent
    replicas of N_w particles (batch means over at least four).  Batched:
    every unconverged case in one grid-kernel launch per round (union
    geometry, one material per case); each launch deals its particles to 8
    replica groups, so batch means exist after one launch, and each round
    gives each case, through its particle share, what its measured variance
    still asks for (a fraction of a budget in the first round); converged cases
    drop out.  Plain adaptive: each case alone in per-case launches with the
    batched arm's groups and allocation.  Table construction is outside
    these clocks.  Returns the line."""
    import torch
    import btegpu
    import synth
    L, ncells, dt, maxtime = 1000.0, 50, 10.0, 1000.0
    cases = synth.sweep_cases()
    temps = sorted({c["T"] for c in cases})
    tabs = {T: synth.mode_table(32, 3, 3, T, config=0) for T in temps}
    nc = len(cases)
    budgets = np.array([c["budget"] for c in cases], dtype=np.int64)
    clocks = ClockSampler(local)
    clocks.start()

    # ---- batched: every unconverged case in one launch per round; the
    # launch deals its particles to G replica groups (batch means inside
    # the launch) and each round gives each case the particles its measured
    # variance still asks for
    G = groups
    g = synth.sweep_union_geometry(cases, length=L, ncells=ncells)
    eng = btegpu.Engine(local)
    eng.load_modes(tabs[300.0])
    eng.load_geometry(g)
    rates = [tabs[c["T"]]["w"] for c in cases]
    Ts = [c["T"] for c in cases]
    eng.load_materials(rates, Ts, budgets / budgets.sum())
    eng.rta_run(300.0, dt, maxtime, 100000, seed=1)          # builds the tables
    eng.set_groups(G)
    per = ncells + 2
    active = np.ones(nc, dtype=bool)
    nmin = 2000.0 * G
    ab = AdaptiveShares(budgets, first_frac, nmin, tol, G)
    ev_b = 0
    reps_b = 0
    parts_b = 0
    round_log = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    while active.any() and time.perf_counter() - t0 < cap:
        alloc = np.array([ab.alloc(i) if active[i] else 0.0 for i in range(nc)])
        N = int(alloc.sum())
        ta = time.perf_counter()
        eng.load_materials(rates, Ts, alloc / alloc.sum())
        tb = time.perf_counter()
        r = eng.rta_run(300.0, dt, maxtime, N, seed=1000 + reps_b, raw=False)
        tc = time.perf_counter()
        grs = [eng.group_result(k, r["jx"].shape, keys=("jx",)) for k in range(G)]
        td = time.perf_counter()
        ev_b += int(r["events"])
        reps_b += 1
        parts_b += N
        # active cases, particles, kernel ms, and host ms of the share
        # update, the run call and the group results
        round_log.append([int(active.sum()), N, round(float(r["kernel_ms"]), 2), round(1e3 * (tb - ta), 1),
                          round(1e3 * (tc - tb), 1), round(1e3 * (td - tc), 1)])
        for i in np.flatnonzero(active):
            sl = slice(per * i, per * i + ncells)
            kg = [synth.sweep_kappa(x["jx"], sl, length=L) for x in grs]
            if ab.add(i, alloc[i], kg):
                active[i] = False
    t_b = time.perf_counter() - t0
    conv_b = int((~active).sum())
    eng.set_groups(0)
    eng.close()

    sp = SweepStats(nc)
    t_p = 0.0
    ev_p = 0
    reps_p = 0
    parts_p = 0
    conv_p = 0
    t_f = 0.0
    conv_f = 0
    cases_iter = list(enumerate(cases)) if plain else []
    # ---- plain
    engs = {}
    for T in (temps if plain else []):
        e = btegpu.Engine(local)
        e.load_modes(tabs[T])
        engs[T] = e
    for i, cs in cases_iter:
        e = engs[cs["T"]]
        e.load_geometry(synth.sweep_ribbon(cs["width"], cs["T"], length=L, ncells=ncells))
        e.rta_run(cs["T"], dt, maxtime, 1000, seed=2)         # tables for this geometry
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        k = 0
        while t_p + (time.perf_counter() - t1) < cap:
            r = e.rta_run(cs["T"], dt, maxtime, int(cs["budget"]), seed=5000 + k, raw=False)
            ev_p += int(r["events"])
            parts_p += int(cs["budget"])
            k += 1
            sp.add(i, synth.sweep_kappa(r["jx"], slice(0, ncells), length=L))
            if sp.rel3(i) <= tol:
                conv_p += 1
                break
        t_p += time.perf_counter() - t1
        reps_p += k
        if t_p >= cap:
            break
    # ---- plain, adaptive: each case alone in per-case launches, with the
    # batched arm's replica groups and allocation, so that the comparison
    # shows what one launch over all cases adds to the allocation
    ad = AdaptiveShares(budgets, first_frac, nmin, tol, G)
    t_a = 0.0
    ev_a = 0
    reps_a = 0
    parts_a = 0
    conv_a = 0
    for i, cs in cases_iter:
        e = engs[cs["T"]]
        e.load_geometry(synth.sweep_ribbon(cs["width"], cs["T"], length=L, ncells=ncells))
        e.rta_run(cs["T"], dt, maxtime, 1000, seed=2)         # tables for this geometry
        e.set_groups(G)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        while t_a + (time.perf_counter() - t1) < cap:
            n_i = int(ad.alloc(i))
            r = e.rta_run(cs["T"], dt, maxtime, n_i, seed=7000 + reps_a, raw=False)
            grs = [e.group_result(k, r["jx"].shape, keys=("jx",)) for k in range(G)]
            ev_a += int(r["events"])
            parts_a += n_i
            reps_a += 1
            if ad.add(i, n_i, [synth.sweep_kappa(x["jx"], slice(0, ncells), length=L) for x in grs]):
                conv_a += 1
                break
        t_a += time.perf_counter() - t1
        e.set_groups(0)
        if t_a >= cap:
            break
    for e in engs.values():
        e.close()

    # ---- plain, one fresh context per case (tables built per case, as one
    # process per case would)
    sf = SweepStats(nc)
    t2 = time.perf_counter()
    for i, cs in cases_iter:
        if time.perf_counter() - t2 >= cap:
            break
        e = btegpu.Engine(local)
        e.load_modes(tabs[cs["T"]])
        e.load_geometry(synth.sweep_ribbon(cs["width"], cs["T"], length=L, ncells=ncells))
        k = 0
        while time.perf_counter() - t2 < cap:
            r = e.rta_run(cs["T"], dt, maxtime, int(cs["budget"]), seed=5000 + k, raw=False)
            k += 1
            sf.add(i, synth.sweep_kappa(r["jx"], slice(0, ncells), length=L))
            if sf.rel3(i) <= tol:
                conv_f += 1
                break
        e.close()
    t_f = time.perf_counter() - t2 if plain else 0.0
    # ---- batched with its table construction on the clock
    t3 = time.perf_counter()
    eng = btegpu.Engine(local)
    eng.load_modes(tabs[300.0])
    eng.load_geometry(g)
    eng.load_materials(rates, Ts, budgets / budgets.sum())
    eng.rta_run(300.0, dt, maxtime, 1000, seed=1)
    t_setup_b = time.perf_counter() - t3
    eng.close()
    clk = clocks.stop()
    kap_b, rel_b = ab.kappa, ab.rel
    worst_b = float(np.max(rel_b))
    line = {
        "metric": "seconds to 1% kappa_eff (3 sigma) over the 64-case sweep, batched",
        "value": t_b, "unit": "s", "n_gpus": 1, "steps": reps_b, "warmup": 1,
        "ms_per_step": 1e3 * t_b / max(reps_b, 1), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded mode tables, no database)",
        "config": {"workload": "64-case ribbon sweep: 16 widths 20nm-2um x T in {100,200,300,500} K, "
                               "1 um long, p=0, 32x32x6 modes with tau at T, reservoirs T+-1 K, "
                               "budgets 1e5*100^(k/15), 100 bins of 10 ps",
                   "tol_3sigma": tol, "time_cap_s": cap, "parallelism": "replicas x1"},
        "batched": {"seconds": t_b, "launches": reps_b, "replica_groups": G, "particles": parts_b,
                    "first_round_fraction": first_frac, "rounds": round_log,
                    "cases_converged": conv_b, "events": ev_b,
                    "events_per_s": ev_b / max(t_b, 1e-9), "worst_3sigma_rel": worst_b},
        "plain": {"seconds": t_p, "launches": reps_p, "particles": parts_p, "cases_converged": conv_p,
                  "events": ev_p,
                  "events_per_s": ev_p / max(t_p, 1e-9)},
        "speedup_plain_over_batched": (t_p / t_b) if (conv_b == nc and conv_p == nc) else None,
        "plain_adaptive": {"seconds": t_a, "launches": reps_a, "particles": parts_a, "cases_converged": conv_a,
                           "events": ev_a, "events_per_s": ev_a / max(t_a, 1e-9),
                           "worst_3sigma_rel": float(np.max(ad.rel)) if conv_a else None},
        "speedup_plain_adaptive_over_batched": (t_a / t_b) if (conv_b == nc and conv_a == nc) else None,
        "with_table_setup": {"batched_seconds": t_b + t_setup_b, "batched_setup_s": t_setup_b,
                             "plain_fresh_contexts_seconds": t_f, "plain_fresh_cases_converged": conv_f,
                             "speedup": (t_f / (t_b + t_setup_b)) if (conv_b == nc and conv_f == nc)
                             else None},
        "kappa_eff_W_mK": {f"{c['T']:.0f}K_{c['width']:.0f}nm": round(float(kap_b[i]), 4)
                           for i, c in enumerate(cases)},
        "kappa_batched_vs_plain_max_z": kappa_agreement(kap_b, rel_b, sp),
        "clocks": clk,
    }
    return line


def kappa_weights(c, Eeff):
    """Weights W[box][bin][q] of kappa_eff = J_x L / dT as a linear functional
    of the raw tallies: the mean over the interior cells and the last 10
    bins of the cumulative flux (/ V_box, x Eeff x 1e30)."""
    nb = int(math.floor(c["maxtime"] / c["dt"] + 1e-6))
    nbx = int(c["geom"]["nboxes"])
    ncell = nbx - 2
    last = 10
    cnt = np.array([(nb - b) if b >= nb - last else last for b in range(nb)], float) / last
    verts = np.asarray(c["geom"]["vertices"]).reshape(-1, 4, 2)
    W = np.zeros((nbx, nb, 3))
    L = float(verts[:ncell, :, 0].max() - verts[:ncell, :, 0].min())
    for b in range(ncell):
        xs, ys = verts[b, :, 0], verts[b, :, 1]
        vbox = (xs.max() - xs.min()) * (ys.max() - ys.min()) * c["geom"]["thickness"]
        W[b, :, 1] = cnt * Eeff * 1e30 / vbox / ncell * L * 1e-9 / 2.0
    return W


def run_adjoint(args, rank, world, local):
    """The C4 workload line (see adjoint_arms)."""
    import torch
    if world > 1 and rank != 0:
        return 0
    torch.cuda.set_device(local)
    print(json.dumps(adjoint_arms(local, args.sweep_seconds)))
    return 0


def adjoint_arms(local, cap, replay_particles=1_000_000):
    """Gradient of kappa_eff of the plain ribbon at p = 0.2 (6144 modes,
    N = 1e7) with respect to 32 seeded mode lifetimes and p, to 1% (3 sigma,
    L2 over the 33 components): the adjoint against central differences
    with common random numbers (dtau/tau = 1e-3, dp = 1e-3).  Differences in
    production mode follow the spec; alias tables decouple the two runs, so
    differences in replay mode (CDF draws, coupled) are timed as well.  Each
    arm is capped in time and reports the accuracy it reached, and the time
    to 1 % extrapolated from it (the error falls as the inverse square root
    of the time spent).  Returns the line."""
    import btegpu
    import synth
    c = synth.config0(n_particles=10_000_000)
    p0 = 0.2
    m = c["modes"]
    N = c["N"]
    eng = btegpu.Engine(local)
    eng.load_modes(m)
    eng.load_geometry(c["geom"])
    r = eng.rta_run(c["T0"], c["dt"], c["maxtime"], N, seed=1, specularity=p0, raw=False)
    W = kappa_weights(c, r["Eeff"])
    rng = np.random.default_rng(20261203)
    movable = np.flatnonzero((m["w"] > 0) & (m["omega"] > 0))
    modes = np.sort(rng.choice(movable, 32, replace=False))
    tau = 1.0 / m["w"][modes]
    clocks = ClockSampler(local)
    clocks.start()

    def acc(rows):
        a = np.asarray(rows)
        if len(a) < 4:
            return float("inf")
        se = a.std(axis=0, ddof=1) / np.sqrt(len(a))
        return 3.0 * float(np.linalg.norm(se) / np.linalg.norm(a.mean(axis=0)))

    # adjoint arm
    rows_a = []
    t0 = time.perf_counter()
    ev_a = 0
    while acc(rows_a) > 0.01 and time.perf_counter() - t0 < cap:
        g = eng.rta_adjoint(W, c["T0"], c["dt"], c["maxtime"], N, seed=100 + len(rows_a),
                            specularity=p0)
        rows_a.append(np.concatenate([g["dphi_dtau"][modes], [g["dphi_dp"]]]))
        ev_a += 2 * int(g["events"])
    t_a = time.perf_counter() - t0
    ga = np.mean(rows_a, axis=0)

    def fd_arm(mode, h, n_part):
        rows = []
        t1 = time.perf_counter()
        runs = 0
        while acc(rows) > 0.01 and time.perf_counter() - t1 < cap:
            seed = 500 + len(rows)
            row = []
            for j, k in enumerate(modes):
                if time.perf_counter() - t1 >= cap:
                    break
                v = []
                for sgn in (1.0, -1.0):
                    w = m["w"].copy()
                    w[k] = 1.0 / (tau[j] * (1.0 + sgn * h))
                    eng.load_materials([w], [c["T0"]])
                    rr = eng.rta_run(c["T0"], c["dt"], c["maxtime"], n_part, seed=seed, mode=mode,
                                     specularity=p0, raw=True)
                    v.append(float(np.sum(W[..., 1] * rr["gz_jx"])) * N / n_part)
                    runs += 1
                row.append((v[0] - v[1]) / (2.0 * h * tau[j]))
            eng.load_materials([], [])
            if len(row) < len(modes):
                break
            v = []
            for sgn in (1.0, -1.0):
                rr = eng.rta_run(c["T0"], c["dt"], c["maxtime"], n_part, seed=seed, mode=mode,
                                 specularity=p0 + sgn * h, raw=True)
                v.append(float(np.sum(W[..., 1] * rr["gz_jx"])) * N / n_part)
                runs += 1
            row.append((v[0] - v[1]) / (2.0 * h))
            rows.append(row)
        return rows, time.perf_counter() - t1, runs

    rows_fp, t_fp, runs_fp = fd_arm(btegpu.MODE_PRODUCTION, 1e-3, N)
    # replay-mode differences: CDF draws keep the two runs coupled; the
    # replay kernel is the bit-exact checker (pcg64, 128-bit tallies), slow,
    # so it runs `replay_particles` per evaluation
    rows_fr, t_fr, runs_fr = fd_arm(btegpu.MODE_REPLAY, 1e-3, replay_particles)
    clk = clocks.stop()

    def agree(rows):
        if len(rows) < 2 or len(rows_a) < 2:
            return None
        f = np.asarray(rows)
        se = np.sqrt(f.var(axis=0, ddof=1) / len(f) + np.var(rows_a, axis=0, ddof=1) / len(rows_a))
        return float(np.max(np.abs(f.mean(axis=0) - ga) / np.maximum(se, 1e-300)))

    def to_1pct(t, a):
        """Seconds to 1 % at the rate observed: accuracy ~ t^-1/2."""
        if not np.isfinite(a) or t <= 0:
            return None
        return t if a <= 0.01 else t * (a / 0.01) ** 2

    acc_a, acc_fp, acc_fr = acc(rows_a), acc(rows_fp), acc(rows_fr)
    t1_a, t1_fp, t1_fr = to_1pct(t_a, acc_a), to_1pct(t_fp, acc_fp), to_1pct(t_fr, acc_fr)
    line = {
        "metric": "seconds to a 1% (3 sigma) gradient of kappa_eff, adjoint",
        "value": t_a, "unit": "s", "n_gpus": 1, "steps": len(rows_a), "warmup": 1,
        "ms_per_step": 1e3 * t_a / max(len(rows_a), 1), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded mode table, no database)",
        "config": {"workload": "plain ribbon at p=0.2: 32x32x6 modes, 1um x 100nm, 50 cells, 301/299K, "
                               "100 bins of 10 ps, N=1e7; dkappa/dtau on 32 seeded modes + dkappa/dp",
                   "accuracy": "3 * ||SE||_2 / ||g||_2 <= 1% over the 33 components",
                   "time_cap_s": cap},
        "adjoint": {"seconds": t_a, "replicas": len(rows_a), "accuracy": acc_a,
                    "events": ev_a, "dkappa_dp": float(ga[-1]), "seconds_to_1pct": t1_a},
        "fd_production": {"seconds": t_fp, "replicas": len(rows_fp), "runs": runs_fp,
                          "accuracy": acc_fp, "max_z_vs_adjoint": agree(rows_fp),
                          "seconds_to_1pct_extrapolated": t1_fp},
        "fd_replay": {"seconds": t_fr, "replicas": len(rows_fr), "runs": runs_fr, "particles_per_run": replay_particles,
                      "accuracy": acc_fr, "max_z_vs_adjoint": agree(rows_fr),
                      "seconds_to_1pct_extrapolated": t1_fr},
        "speedup_over_fd": ({"production": (t1_fp / t1_a) if t1_fp else None,
                             "replay": (t1_fr / t1_a) if t1_fr else None}
                            if t1_a and acc_a <= 0.01 else None),
        "clocks": clk,
    }
    eng.close()
    return line


def time_to_1pct(local, cap):
    """The metric's second half, bounded for the default run: seconds to a
    1 % (3 sigma) kappa_eff over the 64-case sweep, batched against per-case
    launches, and seconds to a 1 % gradient of kappa_eff, the adjoint
    against central differences (each arm capped at `cap` seconds; the
    differences' time to 1 % is extrapolated from the accuracy they reach)."""
    out = {}
    try:
        sw = sweep_arms(local, 0.01, cap)
        out["sweep"] = {
            "workload": sw["config"]["workload"], "tol_3sigma": 0.01, "time_cap_s": cap,
            "batched_s": sw["batched"]["seconds"], "batched_cases_converged": sw["batched"]["cases_converged"],
            "batched_launches": sw["batched"]["launches"], "batched_particles": sw["batched"]["particles"],
            "replica_groups": sw["batched"]["replica_groups"],
            "plain_s": sw["plain"]["seconds"], "plain_cases_converged": sw["plain"]["cases_converged"],
            "plain_launches": sw["plain"]["launches"], "plain_particles": sw["plain"]["particles"],
            "kappa_batched_vs_plain_max_z": sw["kappa_batched_vs_plain_max_z"],
            "speedup_plain_over_batched": sw["speedup_plain_over_batched"],
            "plain_adaptive_s": sw["plain_adaptive"]["seconds"],
            "speedup_plain_adaptive_over_batched": sw["speedup_plain_adaptive_over_batched"],
            "with_table_setup": sw["with_table_setup"], "clocks": sw["clocks"]}
    except Exception as e:  # the summaries must not hide the headline line
        out["sweep"] = {"failed": str(e)}
    try:
        ad = adjoint_arms(local, cap, replay_particles=100_000)
        out["gradient"] = {
            "workload": ad["config"]["workload"], "accuracy": ad["config"]["accuracy"], "time_cap_s": cap,
            "adjoint_s": ad["adjoint"]["seconds_to_1pct"], "adjoint_accuracy": ad["adjoint"]["accuracy"],
            "fd_production_s_extrapolated": ad["fd_production"]["seconds_to_1pct_extrapolated"],
            "fd_production_accuracy": ad["fd_production"]["accuracy"],
            "fd_production_max_z_vs_adjoint": ad["fd_production"]["max_z_vs_adjoint"],
            "fd_replay_s_extrapolated": ad["fd_replay"]["seconds_to_1pct_extrapolated"],
            "fd_replay_accuracy": ad["fd_replay"]["accuracy"],
            "speedup_over_fd": ad["speedup_over_fd"], "clocks": ad["clocks"]}
    except Exception as e:
        out["gradient"] = {"failed": str(e)}
    return out


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.workload == "c4":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the gradient line compares the "
                              "adjoint with differences of this engine"}))
            return 0
        return run_adjoint(args, rank, world, local)
    if args.workload == "c3":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the sweep line compares two arms "
                              "of this engine; the CPU restatement is a parity checker only"}))
            return 0
        return run_sweep(args, rank, world, local)
    if args.workload == "c2":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the beRTA workload line has no "
                              "CPU arm; the restatement's beRTA loop is a parity checker only"}))
            return 0
        return run_berta(args, rank, world, local)
    c = workload(args.workload)
    if args.impl == "reference":
        return reference_arm(args, c, rank, world)

    import torch
    import btegpu
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)

    eng = btegpu.Engine(local)
    eng.load_modes(c["modes"])
    eng.load_geometry(c["geom"])
    per_step = args.per_step or c["per_step"]
    src = source_of(c)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")

    def step(k, seed):
        # each rank carries its own slice of particles (weak scaling); when a
        # step is the whole run (N == per_step) every step reruns it with a
        # new seed
        span = max(c["N"] - per_step + 1, 1)
        base = ((k * world + rank) * per_step) % span
        return eng.rta_run(c["T0"], c["dt"], c["maxtime"], c["N"], seed=seed,
                           mode=btegpu.MODE_PRODUCTION, source=src,
                           specularity=c["specularity"], begin=base, end=base + per_step,
                           raw=False)

    # the first call builds the device tables; the autotuner then picks the
    # kernel's block shape, residency and tally privatisation (not timed)
    import autotune
    trial = max(1000, min(per_step // 8, 250_000))

    def trial_run(begin, end):
        return eng.rta_run(c["T0"], c["dt"], c["maxtime"], c["N"], seed=999,
                           mode=btegpu.MODE_PRODUCTION, source=src,
                           specularity=c["specularity"], begin=begin, end=end, raw=False)
    trial_run(0, trial)
    nbins0 = int(math.floor(c["maxtime"] / c["dt"] + 1e-6))
    choice, tuned = autotune.tune(eng, trial_run, trial, 3 * int(c["geom"]["nboxes"]) * nbins0 * 8)
    for w in range(args.warmup):
        step(w, 1000 + w)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    ev = tal = parts = 0
    kern_ms = 0.0
    e2e_s = 0.0
    for k in range(args.steps):
        flush.fill_(float(k))          # write 256 MB > L2 between steps
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = step(args.warmup + k, 2000 + k)
        e2e_s += time.perf_counter() - t0
        ev += out["events"]
        tal += out["tally_updates"]
        kern_ms += out["kernel_ms"]
        parts += per_step
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    tot = torch.tensor([kern_ms, e2e_s], dtype=torch.float64, device=f"cuda:{local}")
    evs = torch.tensor([float(ev)], dtype=torch.float64, device=f"cuda:{local}")
    if dist:
        dist.all_reduce(tot, op=dist.ReduceOp.MAX)
        dist.all_reduce(evs, op=dist.ReduceOp.SUM)
    kern_ms, e2e_s = float(tot[0]), float(tot[1])
    ev_all = float(evs[0])
    value = ev_all / (kern_ms * 1e-3)
    e2e = ev_all / e2e_s

    if rank == 0:
        nbins = int(math.floor(c["maxtime"] / c["dt"] + 1e-6))
        nboxes = int(c["geom"]["nboxes"])
        d2h = nboxes * nbins * 3 * 8 + 8 * 8 + 16
        h2d = (nbins + 1) * 8 + 8 * (len(c["geom"]["Teq"]) + 1)
        peak, peak_kind = measured_peaks()
        per_launch_bytes = algorithmic_bytes(ev, tal, parts) / args.steps
        achieved = per_launch_bytes / (kern_ms * 1e-3 / args.steps) / 1e9
        prof = profile_figures() if args.workload == "c1" else {}  # ncu figures of the c1 kernel
        ev_launch = ev / args.steps
        traffic = None
        if "dram_bytes_per_event" in prof:
            traffic = prof.get("dram_fixed_bytes", 0.0) + prof["dram_bytes_per_event"] * ev_launch
        fp64 = None
        if "fp64_thread_ops_per_event" in prof:
            mhz = clk.get("sm_mhz") or clk.get("sm_max_mhz") or 2070.0
            lane_peak = prof.get("fp64_lane_ops_per_sm_cycle", 2) * nsm_of_device() * mhz * 1e6
            ops = prof["fp64_thread_ops_per_event"] * value
            fp64 = {"pipe": "fp64", "ops_per_event": prof["fp64_thread_ops_per_event"],
                    "achieved": ops / 1e9, "peak": lane_peak / 1e9, "unit": "Gop/s",
                    "frac": ops / lane_peak, "pipe_busy_pct_ncu": prof.get("fp64_pipe_busy_pct")}
        l2red = None
        if "l2_red_sectors_per_event" in prof and "l2_red_peak_sectors_per_s" in prof:
            red = prof["l2_red_sectors_per_event"] * value
            l2red = {"per_event": prof["l2_red_sectors_per_event"], "achieved": red,
                     "peak": prof["l2_red_peak_sectors_per_s"], "unit": "sectors/s",
                     "frac": red / prof["l2_red_peak_sectors_per_s"]}
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * e2e_s / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded mode table and geometry, no database)",
            "config": {"workload": c["label"], "particles_per_step": per_step,
                       "particles_total": c["N"], "modes": int(c["modes"]["nq"] * c["modes"]["nb"]),
                       "boxes": nboxes, "time_bins": nbins, "l2": "flushed between steps (256 MB write)",
                       "parallelism": f"replicas x{world}"},
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": args.steps,
            "kernel_ms_per_step": kern_ms / args.steps,
            "events_per_step": ev_all / args.steps,
            "tally_updates_per_event": tal / max(ev, 1),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind,
                         "traffic": traffic,
                         "bytes_per_event": per_launch_bytes / max(ev_launch, 1)},
            "co_bound": fp64,
            "l2_reductions": l2red,
            "clocks": clk,
            "tuning": {"block_threads": choice[0], "blocks_per_sm": choice[1],
                       "smem_tally": choice[2], "particles_per_thread": choice[3],
                       "ns_per_event": {f"{k[0]}x{k[1]}{'s' if k[2] else ''}{'p2' if k[3] == 2 else ''}": v
                                        for k, v in tuned.items()}},
        }
        if world == 1 and not args.no_cpu_baseline:
            try:
                cev, cdt, cn = cpu_sample(c, args.cpu_seconds, os.cpu_count() or 1)
                line["cpu_baseline"] = {"value": cev / cdt, "unit": UNIT, "cores": os.cpu_count(),
                                        "kind": "port",
                                        "sample": f"{cn} particles of the same workload "
                                                  f"({cev} events, {cdt:.1f} s)"}
                # the same restatement on one host core, on its own bounded sample
                oev, odt, on = cpu_sample(c, max(2.0, args.cpu_seconds / 3), 1, offset=cn)
                line["cpu_baseline"]["one_core"] = {
                    "value": oev / odt, "unit": UNIT, "cores": 1,
                    "sample": f"{on} particles of the same workload ({oev} events, {odt:.1f} s)"}
            except Exception as e:  # the baseline must not hide the GPU line
                line["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": os.cpu_count(),
                                        "kind": "port", "sample": f"failed: {e}"}
    eng.close()
    if rank == 0:
        if world == 1 and args.workload == "c1" and not args.no_extras:
            line["time_to_1pct"] = time_to_1pct(local, args.extra_seconds)
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
