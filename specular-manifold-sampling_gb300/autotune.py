"""Launch-shape autotuner of the unbiased single-scatter solver.

Picks, for one context and a representative device-resident query sample,
the persistent kernels' blocks per SM (warps per SM = 4 x blocks), the
Bernoulli-trial group size (trials run side by side per query = walks in
flight per query) and the number of top tree nodes the trial kernel stages in
shared memory, timing each candidate with the library's own CUDA-event
phase profile (sms_profile_read).  No candidate changes a result: the random
numbers of every walk are fixed by the query's stream, so only speed is
compared.
"""
from __future__ import annotations

import itertools


def _time_ss(ss, ctx, args, seed, repeats):
    best = None
    for r in range(repeats + 1):
        ctx.reset_stats()
        ss.specular_manifold_sampling_device(*args, seed=seed)
        prof = ctx.profile()
        ms = prof["ss_first"]["ms"] + prof["ss_trials"]["ms"]
        if r > 0:   # the first run of a shape warms it up
            best = ms if best is None else min(best, ms)
    return best


def autotune_ss(sms, ctx, queries_ptr: int, n: int, value_ptr: int, count_ptr: int, walks_ptr: int,
                blocks_per_sm=(2, 4, 6, 8, 12, 16), trial_groups=(8, 16, 32), treelets=(0, 64, 128, 256, 384),
                seed: int = 12345, repeats: int = 2) -> dict:
    """Time every (blocks_per_sm, trial_group) pair on the sample (device
    pointers, as SpecularManifoldSingleScatter.specular_manifold_sampling_device),
    then the shared-memory treelet sizes at the fastest pair; set the fastest
    on ctx and return {"best": (bps, group, treelet), "ms": {...}}."""
    ss = sms.SpecularManifoldSingleScatter(ctx)
    args = (queries_ptr, n, value_ptr, count_ptr, walks_ptr)
    timings = {}
    ctx.set_profiling(True)
    try:
        ctx.set_treelet(0)
        for bps, grp in itertools.product(blocks_per_sm, trial_groups):
            ctx.set_launch(bps, 0)
            ctx.set_trial_group(grp)
            timings[(bps, grp, 0)] = _time_ss(ss, ctx, args, seed, repeats)
        bps, grp, _ = min(timings, key=timings.get)
        ctx.set_launch(bps, 0)
        ctx.set_trial_group(grp)
        for t in treelets:
            if t:
                ctx.set_treelet(t)
                timings[(bps, grp, t)] = _time_ss(ss, ctx, args, seed, repeats)
    finally:
        ctx.set_profiling(False)
        ctx.reset_stats()
    choice = min(timings, key=timings.get)
    ctx.set_launch(choice[0], 0)
    ctx.set_trial_group(choice[1])
    ctx.set_treelet(choice[2])
    return {"best": choice, "ms": {f"{b}x{g}x{t}": ms for (b, g, t), ms in timings.items()}}
