"""Process replicas of one RTA run: each rank carries a contiguous slice of
the particles and the ranks sum their raw tallies once at the end.

Particles of the RTA loop are independent (src/RTA_MC2D.cpp:2228-2317), so
the run shards with no exchange on the data path; the slices follow
alma::my_jobs (include/utilities.hpp:343-356).  The final sum is a host-side
reduction over torch.distributed (gloo on CPU, NCCL between GPUs).
"""
import numpy as np


def my_jobs(njobs: int, nprocs: int, my_id: int):
    """[begin, end) of the jobs of process my_id (alma::my_jobs)."""
    quot, rem = divmod(njobs, nprocs)
    return quot * my_id + min(rem, my_id), quot * (my_id + 1) + min(rem, my_id + 1)


def exact_to_int(ex: np.ndarray):
    """(hi, lo) int64 pairs of the replay tallies -> Python integers."""
    hi = ex[..., 0].astype(object)
    lo = ex[..., 1].astype(np.uint64).astype(object)
    return hi * (1 << 64) + lo


def reduce_tallies(out: dict, group=None) -> dict:
    """Sum the raw tallies of every rank (in place on rank-local copies).

    FP64 tallies are summed in rank order by all_reduce; the 128-bit replay
    tallies are summed exactly as four 32-bit limbs in int64 lanes, so the
    result equals the single-process run bit for bit."""
    import torch
    import torch.distributed as dist
    res = dict(out)
    for k in ("gz", "gz_jx", "gz_jy"):
        if k in out:
            t = torch.from_numpy(np.ascontiguousarray(out[k], dtype=np.float64))
            dist.all_reduce(t, group=group)
            res[k] = t.numpy()
    if "exact" in out:
        v = exact_to_int(out["exact"]).reshape(-1)
        mask = (1 << 32) - 1
        limbs = np.zeros((v.size, 4), dtype=np.int64)
        for j in range(4):
            limbs[:, j] = [(int(x) >> (32 * j)) & mask for x in v]
        t = torch.from_numpy(limbs)
        dist.all_reduce(t, group=group)
        s = [sum(int(t[i, j]) << (32 * j) for j in range(4)) % (1 << 128) for i in range(v.size)]
        s = [x - (1 << 128) if x >= (1 << 127) else x for x in s]
        hi = np.array([(x >> 64) for x in s], dtype=object)
        lo = np.array([x & ((1 << 64) - 1) for x in s], dtype=object)
        ex = np.zeros(out["exact"].shape, dtype=np.int64)
        ex[..., 0] = np.array([int(h) for h in hi], dtype=np.int64).reshape(ex.shape[:-1])
        ex[..., 1] = np.array([int(x) for x in lo], dtype=np.uint64).view(np.int64).reshape(ex.shape[:-1])
        res["exact"] = ex
    for k in ("events", "wall_hits", "crossings", "absorbed", "specular_hits"):
        if k in out:
            t = torch.tensor([int(out[k])], dtype=torch.int64)
            dist.all_reduce(t, group=group)
            res[k] = int(t[0])
    return res


def run_replica(run, total: int, rank: int, world: int, group=None, **kw) -> dict:
    """Run this rank's slice with `run(begin=..., end=..., **kw)` and sum."""
    b, e = my_jobs(total, world, rank)
    return reduce_tallies(run(begin=b, end=e, **kw), group=group)
