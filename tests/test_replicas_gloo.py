"""Replicas across processes (world size 2, gloo on CPU): the particle slices
of alma::my_jobs, summed once, reproduce the single-process run exactly."""
import os
import sys

import numpy as np
import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, path):
    for sub in ("bte-barna_gb300", "oracle"):
        sys.path.insert(0, os.path.join(REPO, sub))
    import torch.distributed as dist
    import pyoracle
    import replicas
    import synth
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    case = synth.small_case(n_particles=900)
    out = replicas.run_replica(lambda begin, end: pyoracle.rta_run(case, seed=3, begin=begin, end=end),
                               case["N"], rank, world)
    if rank == 0:
        np.save(path, out["exact"])
        with open(path + ".events", "w") as f:
            f.write(str(out["events"]))
    dist.destroy_process_group()


def test_my_jobs_partition():
    import replicas
    for n, p in [(10, 3), (7, 7), (3, 5), (1000, 8)]:
        spans = [replicas.my_jobs(n, p, i) for i in range(p)]
        assert spans[0][0] == 0 and spans[-1][1] == n
        assert all(spans[i][1] == spans[i + 1][0] for i in range(p - 1))
        assert max(e - b for b, e in spans) - min(e - b for b, e in spans) <= 1


def test_two_replicas_sum_to_single_run(tmp_path):
    import pyoracle
    import synth
    path = str(tmp_path / "ex.npy")
    port = 29500 + os.getpid() % 1000
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_worker, args=(r, 2, port, path)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    summed = np.load(path)
    case = synth.small_case(n_particles=900)
    full = pyoracle.rta_run(case, seed=3)
    assert np.array_equal(summed, full["exact"])
    assert int(open(path + ".events").read()) == full["events"]
