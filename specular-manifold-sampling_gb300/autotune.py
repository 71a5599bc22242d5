"""Launch-shape autotuner of the SMS solvers.

Picks, for one context and a representative device-resident query sample,
the persistent kernels' blocks per SM (warps per SM = 4 x blocks), the
Bernoulli-trial group size (trials run side by side per query = walks in
flight per query), the number of top tree nodes the trial kernel stages in
shared memory, and the queries a lane group claims from the trial queue per
atomic (queue chunk); for the multi-scatter and glint estimators, blocks per
SM.  Each candidate is timed with the library's own CUDA-event phase profile
(sms_profile_read).  No candidate changes a result: the random
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
                chunks=(1, 2, 4), seed: int = 12345, repeats: int = 2) -> dict:
    """Time every (blocks_per_sm, trial_group) pair on the sample (device
    pointers, as SpecularManifoldSingleScatter.specular_manifold_sampling_device),
    then the shared-memory treelet sizes and the queue chunk sizes at the
    fastest pair (coordinate search); set the fastest on ctx and return
    {"best": (bps, group, treelet, chunk), "ms": {...}}."""
    ss = sms.SpecularManifoldSingleScatter(ctx)
    args = (queries_ptr, n, value_ptr, count_ptr, walks_ptr)
    timings = {}
    ctx.set_profiling(True)
    try:
        ctx.set_treelet(0)
        ctx.set_queue_chunk(1)
        for bps, grp in itertools.product(blocks_per_sm, trial_groups):
            ctx.set_launch(bps, 0)
            ctx.set_trial_group(grp)
            timings[(bps, grp, 0, 1)] = _time_ss(ss, ctx, args, seed, repeats)
        bps, grp, _, _ = min(timings, key=timings.get)
        ctx.set_launch(bps, 0)
        ctx.set_trial_group(grp)
        for t in treelets:
            if t:
                ctx.set_treelet(t)
                timings[(bps, grp, t, 1)] = _time_ss(ss, ctx, args, seed, repeats)
        tb = min((k for k in timings if k[0] == bps and k[1] == grp), key=timings.get)[2]
        ctx.set_treelet(tb)
        for ch in chunks:
            if ch > 1:
                ctx.set_queue_chunk(ch)
                timings[(bps, grp, tb, ch)] = _time_ss(ss, ctx, args, seed, repeats)
    finally:
        ctx.set_profiling(False)
        ctx.reset_stats()
    choice = min(timings, key=timings.get)
    ctx.set_launch(choice[0], 0)
    ctx.set_trial_group(choice[1])
    ctx.set_treelet(choice[2])
    ctx.set_queue_chunk(choice[3])
    return {"best": choice, "ms": {f"{b}x{g}x{t}x{c}": ms for (b, g, t, c), ms in timings.items()}}


def autotune_blocks(sms, ctx, kind: str, queries_ptr: int, n: int, value_ptr: int, count_ptr: int, walks_ptr: int,
                    blocks_per_sm=(2, 4, 6, 8, 12, 16), seed: int = 12345, repeats: int = 2) -> dict:
    """Blocks per SM of the multi-scatter ("ms") or glint ("glints") kernels,
    timed with their phase of the CUDA-event profile on a device-resident
    sample; sets the fastest on ctx and returns {"best": bps, "ms": {...}}."""
    est = {"ms": sms.SpecularManifoldMultiScatter, "glints": sms.SpecularManifoldGlints}[kind](ctx)
    timings = {}
    ctx.set_profiling(True)
    try:
        for bps in blocks_per_sm:
            ctx.set_launch(bps, 0)
            best = None
            for r in range(repeats + 1):
                ctx.reset_stats()
                est.specular_manifold_sampling_device(queries_ptr, n, value_ptr, count_ptr, walks_ptr, seed=seed)
                ms = ctx.profile()[kind]["ms"]
                if r > 0:
                    best = ms if best is None else min(best, ms)
            timings[bps] = best
    finally:
        ctx.set_profiling(False)
        ctx.reset_stats()
    choice = min(timings, key=timings.get)
    ctx.set_launch(choice, 0)
    return {"best": choice, "ms": {str(b): t for b, t in timings.items()}}
