"""Autotuner of the production grid kernel.

Tries block shapes, resident blocks per SM (the register/residency variants
of rta_prod_grid), shared-memory tally privatisation and the particles each
thread carries at once (1, or 2 in the interleaved kernel) on a short slice
of the real workload, measures device time per flight event, and leaves the
fastest setting on the engine.  Runs before any timed region.
"""
import btegpu

# (threads per block, blocks per SM, shared-memory tally, particles per thread)
CANDIDATES = [(256, 4, 0, 1), (128, 8, 0, 1), (256, 3, 0, 1), (256, 2, 0, 1), (128, 6, 0, 1), (128, 4, 0, 1),
              (256, 1, 1, 1), (256, 1, 0, 2), (128, 3, 0, 2), (256, 2, 0, 2), (128, 4, 0, 2)]


def tune(engine, run, trial_particles: int, smem_bytes: int, repeats: int = 2):
    """`run(begin, end)` performs one production run of the workload slice.

    Returns (best candidate, {candidate: ns per event})."""
    results = {}
    for cand in CANDIDATES:
        threads, bps, smem, ppt = cand
        if smem and smem_bytes > 200 * 1024:
            continue
        try:
            engine.set_tuning(block_threads=threads, blocks_per_sm=bps, smem_tally=smem,
                              particles_per_thread=ppt)
            best = None
            for r in range(repeats):
                out = run(r * trial_particles, (r + 1) * trial_particles)
                ns = 1e6 * out["kernel_ms"] / max(out["events"], 1)
                best = ns if best is None else min(best, ns)
            results[cand] = best
        except btegpu.BteError:
            continue
    choice = min(results, key=results.get)
    engine.set_tuning(block_threads=choice[0], blocks_per_sm=choice[1], smem_tally=choice[2],
                      particles_per_thread=choice[3])
    return choice, results
