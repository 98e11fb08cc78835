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
    ap.add_argument("--workload", default="c1", choices=["c1", "c0", "c2"])
    ap.add_argument("--per-step", type=int, default=0, help="particles per step")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    return ap.parse_args()


def workload(name):
    import synth
    if name == "c1":
        c = synth.config1()
        c["label"] = ("transient RTA at scale: 64x64 q x 9 branches (36864 modes), 2um x 500nm, "
                      "100x25 cells of 20nm, 200nm staircase pore, p=0.3, 1K hot spot sigma 50nm, "
                      "200 bins to 10ns, N=1e8")
        c["per_step"] = 2_000_000
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
    E = 1e-21
    for _ in range(4):  # the population scales as 1 / Eeff
        r = eng.berta_run(dt, maxtime, E, seed=7)
        n_end = int(r["nparticles"][-1])
        if n_end >= 10_000:
            E = E * n_end / target
            break
        E = E / 100.0
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
    for k in range(args.steps):
        flush.fill_(float(k))
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        r = eng.berta_run(dt, maxtime, E, seed=200 + k)
        e2e_s += time.perf_counter() - t1
        ps += int(r["particle_steps"])
        kern_ms += float(r["kernel_ms"])
        alive.append(int(r["nparticles"][-1]))
    torch.cuda.synchronize()
    clk = clocks.stop()
    nbx = int(c["geom"]["nboxes"])
    nsteps = btegpu.berta_steps(dt, maxtime)
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
        "clocks": clk,
    }
    print(json.dumps(line))
    eng.close()
    return 0


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
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
        prof = profile_figures()
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
            "clocks": clk,
            "tuning": {"block_threads": choice[0], "blocks_per_sm": choice[1],
                       "smem_tally": choice[2],
                       "ns_per_event": {f"{k[0]}x{k[1]}{'s' if k[2] else ''}": v
                                        for k, v in tuned.items()}},
        }
        if world == 1 and not args.no_cpu_baseline:
            try:
                cev, cdt, cn = cpu_sample(c, args.cpu_seconds, os.cpu_count() or 1)
                line["cpu_baseline"] = {"value": cev / cdt, "unit": UNIT, "cores": os.cpu_count(),
                                        "kind": "port",
                                        "sample": f"{cn} particles of the same workload "
                                                  f"({cev} events, {cdt:.1f} s)"}
            except Exception as e:  # the baseline must not hide the GPU line
                line["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": os.cpu_count(),
                                        "kind": "port", "sample": f"failed: {e}"}
        print(json.dumps(line))
    eng.close()
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
