"""Benchmark: SMS connections/s on the water-heightfield single-scatter workload.

Workload (one "step"): unbiased single-scatter SMS for 1,048,576 shading points
uniform on [-1,1]^2 under a water surface z = 1 + 32 sinusoids tessellated to
512x512 vertices (522,242 triangles, IOR 1.33), spherical area light r=0.1 at
height 10, Bernoulli trials capped at 256, 20 Newton iterations.  A connection
is one query's full estimator call (specular_manifold_sampling for the caster).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Our arm times K persistent-kernel launches on device-resident queries (value),
then the same K steps through the host-pointer C-ABI entry point with pinned
host buffers (e2e).  The reference arm times the CPU oracle (the scalar
restatement of the reference's scalar_rgb path; the reference itself cannot be
built here) on all host cores over a bounded sample of the same workload.
Multi-GPU: replicas only (each rank solves its own 1M-query shard).
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
PKG_DIR = ROOT / "specular-manifold-sampling_gb300"
sys.path.insert(0, str(ROOT))

N_QUERIES = 1 << 20
METRIC = "SMS connections/s"
UNIT = "connections/s"
WORKLOAD = "water heightfield 512x512 (522,242 tris), unbiased SMS, 1M shading points, trials<=256"


def load_package():
    if "sms_gb300" in sys.modules:
        return sys.modules["sms_gb300"]
    spec = importlib.util.spec_from_file_location(
        "sms_gb300", PKG_DIR / "__init__.py", submodule_search_locations=[str(PKG_DIR)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["sms_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


# Nominal FP32 SIMT peak of one GB300: 152 SMs x 128 FP32 lanes x 2 FLOP (FMA)
# x the SM clock (no measured figure exists for it; the clock is the one sampled
# during the timed region, else the 2070 MHz maximum).
def fp32_peak_tflops(sm_mhz=None):
    return 152 * 128 * 2 * (sm_mhz or 2070.0) * 1e6 / 1e12


# Algorithmic bytes of the traversal, per the oracle's tree (a node: box 24 B +
# child / leaf word 8 B = 32 B; a triangle: 3 vertices = 36 B).  One device node
# record holds the boxes of both children, which the traversal tests together:
# two oracle nodes, 64 B.
NODE_RECORD_BYTES = 2 * 32
TRIANGLE_BYTES = 36


def flops_per_unit():
    """FP32 work per ray / box test / triangle test / Newton iteration of each
    benchmark configuration, counted by the oracle's op-counting build
    (profiles/flops_per_unit.json, written by oracle/count_flops.py)."""
    p = ROOT / "profiles" / "flops_per_unit.json"
    return json.loads(p.read_text())["configs"] if p.exists() else {}


def fp32_work(units, rays, box_tests, tri_tests):
    """FLOPs of a kernel from its own ray, box-test and triangle-test counts."""
    if not units:
        return None
    return rays * units["flops_per_ray"] + box_tests * units["flops_per_box"] + tri_tests * units["flops_per_triangle"]


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1].split()[0]))
                smax.append(float(parts[2].split()[0]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def shard(rank: int, n: int) -> tuple[int, int]:
    """Replica sharding: rank r solves queries [r n, (r+1) n) of the global
    set on PCG32 streams starting at r n, so N ranks reproduce one N n-query
    run exactly (no data-path collective)."""
    return rank * n, rank * n


def max_over_ranks(torch, values, device):
    """Element-wise maximum of per-rank timings (identity without a process group)."""
    import torch.distributed as dist
    t = torch.tensor(values, dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def cpu_baseline_sample(sms, W, n_sample: int, nthreads: int, seed: int = 1, osc=None):
    """Time the oracle on a bounded sample of the workload (first n_sample
    queries of the 1M set).  Returns (connections/s, seconds, n_sample)."""
    from oracle import oracle as O
    osc = osc or O.OracleScene(W.water_scene())
    q = W.water_queries(n_sample)
    t0 = time.perf_counter()
    osc.connect_batch(W.water_config(), q, seed=seed, nthreads=nthreads)
    dt = time.perf_counter() - t0
    return n_sample / dt, dt, n_sample


def cpu_baseline_configs(sms, W, cores: int):
    """The oracle's connections/s on bounded samples of the other benchmark
    configurations, all cores and one thread."""
    from oracle import oracle as O
    cases = [
        ("sphere_biased_m16", W.sphere_scene, W.sphere_config, lambda: W.sphere_queries(64), {}, 1024),
        ("slab_two_bounce_biased_m32", W.slab_scene, W.slab_config, lambda: W.slab_queries(8192), {"multi": True},
         512),
        ("glints_8192_vectorized_m64", W.glint_scene, W.glint_config,
         lambda: np.ascontiguousarray(W.glint_queries(1024)[:, ::16]), {"glints": True}, 4096),
    ]
    out = {}
    for name, scene, config, queries, kw, n1 in cases:
        osc = O.OracleScene(scene())
        q = queries()
        cfg = config()
        osc.connect_batch(cfg, q[:, :64], seed=1, nthreads=cores, **kw)   # first touch (LEAN, caches)
        t0 = time.perf_counter()
        osc.connect_batch(cfg, q, seed=2, nthreads=cores, **kw)
        dt = time.perf_counter() - t0
        q1 = np.ascontiguousarray(q[:, :n1])
        t1 = time.perf_counter()
        osc.connect_batch(cfg, q1, seed=2, nthreads=1, **kw)
        dt1 = time.perf_counter() - t1
        out[name] = {"value": q.shape[1] / dt, "unit": UNIT, "cores": cores, "kind": "port",
                     "single_thread": n1 / dt1,
                     "sample": f"{q.shape[1]} queries ({dt:.2f} s); single thread {n1} queries ({dt1:.2f} s)"}
    return out


def basin_sample(sms, W, ctx, n: int = 16384):
    """Per-walk parity on a sample of the headline workload's walks (explicit
    seeds, light centre): the fraction of walks whose outcome differs between
    the oracle's FP32, FP32-FMA and FP64 builds and one-ulp input nudges (basin
    crossings), and the GPU's mismatch against the oracle on the rest."""
    sys.path.insert(0, str(ROOT / "tests"))
    import basin as B
    from oracle import oracle as O
    desc = W.water_scene()
    cfg = sms.SMSConfig()
    q = W.water_queries(n)
    u = W.pcg32_streams_f32(11, np.arange(n, dtype=np.uint64), 2)
    w = np.zeros((8, n), np.float32)
    w[0], w[1], w[2] = 0.0, 0.05, 10.0
    w[6], w[7] = u[0], u[1]
    ens = B.oracle_walks(O, desc, "walk_batch", cfg, 0, q, w)
    base = O.OracleScene(desc)
    for name, rows in (("seed", slice(6, 8)), ("light", slice(0, 3))):
        for up in (True, False):
            ens[f"{name}_{'up' if up else 'down'}"] = base.walk_batch(cfg, 0, q, B.nudge(w, rows, up))
    mask = B.well_conditioned_walks(ens)
    saved = ctx.config
    ctx.set_config(cfg)
    out_g = sms.SpecularManifoldSingleScatter(ctx).sample_path(0, q, w)
    ctx.set_config(saved)
    agree = B.walk_outcome_equal(out_g, ens["f32"])
    loo = B.leave_one_out_rates(ens)
    return {"walks": n, "basin_crossing_fraction": 1.0 - float(mask.mean()),
            "gpu_mismatch_well_conditioned": float(np.mean(~agree[mask])),
            "gpu_mismatch_all": float(np.mean(~agree)),
            "oracle_leave_one_out_max": max(loo.values()),
            "note": "first walks of the headline scene from explicit seeds (light centre); well conditioned = "
                    "same outcome in the oracle's FP32, FP32-FMA and FP64 builds and with the seed sample or the light point "
                    "nudged one ulp"}


class DeviceTimer:
    """CUDA-event time of work issued on one stream."""

    def __init__(self, torch, stream):
        self.torch, self.stream = torch, stream

    def __enter__(self):
        self.a = self.torch.cuda.Event(enable_timing=True)
        self.b = self.torch.cuda.Event(enable_timing=True)
        self.a.record(self.stream)
        return self

    def __exit__(self, *exc):
        self.b.record(self.stream)
        self.b.synchronize()
        self.ms = self.a.elapsed_time(self.b)


def connect_timed(torch, sms, ctx, kind, q_dev, n, seed, stream_offset=0):
    """One device-pointer connection call; returns (value (3, n) on device, ms)."""
    dev = q_dev.device
    val = torch.empty((3, n), dtype=torch.float32, device=dev)
    cnt = torch.empty(n, dtype=torch.int32, device=dev)
    wlk = torch.empty(n, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)
    est = {"ss": sms.SpecularManifoldSingleScatter, "ms": sms.SpecularManifoldMultiScatter,
           "glints": sms.SpecularManifoldGlints}[kind](ctx)
    with DeviceTimer(torch, stream) as t:
        est.specular_manifold_sampling_device(q_dev.data_ptr(), n, val.data_ptr(), cnt.data_ptr(), wlk.data_ptr(),
                                              seed=seed, stream_offset=stream_offset)
    return val, t.ms


def secondary_configs(torch, sms, W, dev, only=None, calls=5, max_queries=None, tune=True):
    """Throughput of the other solver configurations (one GPU): sphere
    (biased, 16 walks), two-bounce slab (biased, 32 walks, 512k queries) and
    glints (8192^2 FP16 slope map, 1024^2 pixels, 64 seeds, vectorized).
    only: run just that configuration (for profiling one kernel), on its first
    max_queries queries if given."""
    out = {}
    cases = [
        ("sphere_biased_m16", "ss", W.sphere_scene, W.sphere_config, lambda: W.sphere_queries(64), 16),
        ("slab_two_bounce_biased_m32", "ms", W.slab_scene, W.slab_config, lambda: W.slab_queries(1 << 19), 32),
        ("glints_8192_vectorized_m64", "glints", W.glint_scene, W.glint_config, lambda: W.glint_queries(1024), 64),
    ]
    for name, kind, scene, config, queries, walks in cases:
        if only and name != only:
            continue
        ctx = sms.Context(sms.Scene(scene()), config(), device=dev)
        qh = queries()
        if max_queries:
            qh = qh[:, :max_queries]
        q = torch.from_numpy(np.ascontiguousarray(qh, np.float32)).to(f"cuda:{dev}")
        n = q.shape[1]
        tuned = None
        if tune and kind in ("ms", "glints"):
            # blocks per SM of the persistent kernels, picked on the same queries
            from sms_gb300.autotune import autotune_blocks
            bufs = [torch.empty((3, n), dtype=torch.float32, device=f"cuda:{dev}"),
                    torch.empty(n, dtype=torch.int32, device=f"cuda:{dev}"),
                    torch.empty(n, dtype=torch.int32, device=f"cuda:{dev}")]
            torch.cuda.synchronize()
            tuned = autotune_blocks(sms, ctx, kind, q.data_ptr(), n, *(b.data_ptr() for b in bufs), repeats=1)
        for i in range(3):
            connect_timed(torch, sms, ctx, kind, q, n, seed=50 + i)
        ctx.reset_stats()
        ms = [connect_timed(torch, sms, ctx, kind, q, n, seed=60 + i)[1] for i in range(calls)]
        st = ctx.stats()
        t = float(np.mean(ms))
        its_per_s = st["newton_iterations"] / (calls * t / 1e3)
        out[name] = {"queries": n, "ms_per_call": t, "connections_per_s": n / (t / 1e3),
                     "walks_per_s": st["walks"] / (calls * t / 1e3), "walks_per_connection": walks,
                     "newton_iterations_per_walk": st["newton_iterations"] / max(1, st["walks"]),
                     "newton_iterations_per_s": its_per_s}
        if tuned:
            out[name]["launch"] = {"blocks_per_sm": tuned["best"], "autotune_ms": tuned["ms"]}
        units = flops_per_unit().get(name)
        if units:
            if kind == "glints":
                flops = st["newton_iterations"] * units["flops_per_newton_iteration"]
            else:
                flops = fp32_work(units, st["rays"], 2 * st["bvh_nodes"], st["tri_tests"])
            tf = flops / (calls * t / 1e3) / 1e12
            out[name]["fp32"] = {"achieved_tflops": tf, "peak_tflops": fp32_peak_tflops(),
                                 "frac": tf / fp32_peak_tflops(), "peak_kind": "nominal",
                                 "flops_per_newton_iteration": units["flops_per_newton_iteration"]}
        if kind == "glints":
            # one iteration gathers a 2x2 FP16 (sx, sy) texel block: 16 B of the
            # 256 MiB slope map (larger than L2)
            peak, _ = peaks()
            gbs = its_per_s * 16 / 1e9
            out[name]["roofline"] = {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s",
                                     "frac": gbs / peak, "bytes_per_iteration": 16}
        else:
            out[name]["rays_per_s"] = st["rays"] / (calls * t / 1e3)
        ctx.close()
    return out


def render_study(torch, sms, W, dev, width=512, height=512, spp=16):
    """Whole images through the path tracer around the SMS solver (sms_render):
    the pool scene (512^2 water heightfield over a diffuse floor, sphere area
    light), path_sms_ss with the unbiased estimator (cap 256), plain path
    tracing and the paper's comparison integrator path_filtered_ss (the same
    light paths as path_sms_ss, found by BSDF and emitter sampling),
    width x height x spp samples; the oracle's restatement of path_sms_ss on
    the host cores for a bounded 64 x 64 x 4 sample."""
    from oracle import oracle as O
    desc = W.pool_scene(res=512)
    cfg = W.water_config()
    ctx = sms.Context(sms.Scene(desc), cfg, device=dev)
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)
    img = torch.zeros((height, width, 3), dtype=torch.float32, device=f"cuda:{dev}")
    torch.cuda.synchronize()
    cam = W.pool_camera(width, height)
    out = {"scene": "pool: 512^2 water heightfield (IOR 1.33) over a diffuse floor, sphere area light r=0.5",
           "image": [width, height], "spp": spp}
    for integ in ("path_sms_ss", "path", "path_filtered_ss"):
        opt = sms.RenderOptions(integrator=integ, spp=spp, seed=1)
        ctx.render_device(cam, opt, img.data_ptr())
        ctx.reset_stats()
        times = []
        for k in range(3):
            opt.seed = 2 + k
            with DeviceTimer(torch, stream) as t:
                ctx.render_device(cam, opt, img.data_ptr())
            times.append(t.ms)
        st = ctx.stats()
        ms = float(np.mean(times))
        out[integ] = {"ms_per_image": ms, "samples_per_s": width * height * spp / (ms / 1e3),
                      "sms_connections_per_s": st["connections"] / (3 * ms / 1e3),
                      "sms_walks_per_s": st["walks"] / (3 * ms / 1e3), "mean": float(img.mean().item())}
    cores = os.cpu_count() or 1
    ccam = W.pool_camera(64, 64)
    opt = sms.RenderOptions(integrator="path_sms_ss", spp=4, seed=1)
    osc = O.OracleScene(desc)
    t0 = time.perf_counter()
    osc.render(cfg, ccam, opt, nthreads=cores)
    dt = time.perf_counter() - t0
    out["cpu_oracle"] = {"samples_per_s": 64 * 64 * 4 / dt, "cores": cores, "kind": "port",
                         "sample": f"64x64 pixels x 4 spp path_sms_ss, {dt:.2f} s"}
    out["speedup_vs_cpu_oracle"] = out["path_sms_ss"]["samples_per_s"] / out["cpu_oracle"]["samples_per_s"]
    ctx.close()
    # glints: the 8192^2 slope-map plane of the glint configuration, path_sms_glints
    gdesc = W.glint_scene()
    gcfg = W.glint_config()
    gctx = sms.Context(sms.Scene(gdesc), gcfg, device=dev)
    gstream = torch.cuda.ExternalStream(gctx.stream, device=dev)
    gcam = W.glint_render_camera(width, height)
    gopt = sms.RenderOptions(integrator="path_sms_glints", spp=spp, seed=1)
    with DeviceTimer(torch, gstream) as t_first:   # includes the LEAN pyramid build
        gctx.render_device(gcam, gopt, img.data_ptr())
    gctx.reset_stats()
    times = []
    for k in range(3):
        gopt.seed = 2 + k
        with DeviceTimer(torch, gstream) as t:
            gctx.render_device(gcam, gopt, img.data_ptr())
        times.append(t.ms)
    st = gctx.stats()
    ms = float(np.mean(times))
    out["path_sms_glints"] = {"scene": "glint plane, 8192^2 FP16 slope map, point light; biased vectorized M=64",
                              "ms_per_image": ms, "samples_per_s": width * height * spp / (ms / 1e3),
                              "glint_connections_per_s": st["connections"] / (3 * ms / 1e3),
                              "first_image_ms_with_lean_build": t_first.ms, "mean": float(img.mean().item())}
    gosc = O.OracleScene(gdesc)
    gosc.glint_lean_pdf(0.5, 0.5, [1e-3, 0.0, 0.0, 1e-3], [0.0, 0.0, 1.0], [0.0, 0.0, 1.0])   # builds its LEAN pyramid
    t0 = time.perf_counter()
    gosc.render(gcfg, W.glint_render_camera(64, 64), sms.RenderOptions(integrator="path_sms_glints", spp=1, seed=1),
                nthreads=cores)
    dt = time.perf_counter() - t0
    out["path_sms_glints"]["cpu_oracle"] = {"samples_per_s": 64 * 64 / dt, "cores": cores, "kind": "port",
                                            "sample": f"64x64 pixels x 1 spp path_sms_glints, {dt:.2f} s"}
    gctx.close()
    return out


def learned_study(torch, sms, W, ctx, dev, pairs=4 << 20, steps=20000, batch=8192, lr=1e-3, res=256,
                  ref_spp=4096, sigma_scale=1.0, weighted=True, walks_per_query=8):
    """Learned seed proposal on the water workload: training pairs from the
    uniform-seed solver, GPU training, then equal-time caustic RMSE of
    learned vs uniform seeding against a ref_spp uniform-seed image of
    res x res receiver points."""
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)
    cfg = W.water_config()
    ctx.set_config(cfg)
    ctx.set_trial_group(0)   # 32 lanes per query for uniform seeds, 8 for learned ones
    prop = sms.SeedProposal(ctx, 0, seed=1, capacity=pairs)
    prop.set_options(sigma_scale, weighted)
    chunk = 1 << 20
    total, calls = 0, 0
    with DeviceTimer(torch, stream) as t_collect:
        while total < pairs and calls < 16:
            q = torch.from_numpy(W.water_queries(chunk, seed=77, first=calls * chunk)).to(f"cuda:{dev}")
            torch.cuda.synchronize()
            total = prop.collect(q.data_ptr(), chunk, seed=77, stream_offset=calls * chunk,
                                 walks_per_query=walks_per_query)
            calls += 1
    prop.normalize()
    loss0, _ = prop.loss_grad(batch)
    warm = min(100, max(1, steps // 10))
    prop.train(steps=warm, batch=batch, lr=lr)   # graph capture + warm-up
    t0 = time.perf_counter()
    with DeviceTimer(torch, stream) as t_train:
        loss = prop.train(steps=steps - warm, batch=batch, lr=lr)
    train_wall = time.perf_counter() - t0
    step_ms = t_train.ms / max(1, steps - warm)
    flop_step = 3 * 2 * batch * (96 * 64 + 3 * 64 * 64 + 64 * 48)   # forward + backward GEMMs
    # images: pixel centres of a res x res grid on the receiver, spp samples each
    c = (np.arange(res) + 0.5) / res * 2.0 - 1.0
    yy, xx = np.meshgrid(c, c, indexing="ij")
    pix = W.plane_queries(np.stack([xx.ravel(), yy.ravel()], axis=1).astype(np.float32))
    npix = pix.shape[1]

    # trial-group size for learned seeds, tuned on a 16-spp sample of the image
    from sms_gb300.autotune import autotune_ss
    ctx.set_proposal(prop, 0.1)
    qs = torch.from_numpy(np.tile(pix, (1, 16))).to(f"cuda:{dev}")
    ns = qs.shape[1]
    vs = torch.empty((3, ns), dtype=torch.float32, device=f"cuda:{dev}")
    cs = torch.empty(ns, dtype=torch.int32, device=f"cuda:{dev}")
    ws = torch.empty(ns, dtype=torch.int32, device=f"cuda:{dev}")
    torch.cuda.synchronize()
    tune = autotune_ss(sms, ctx, qs.data_ptr(), ns, vs.data_ptr(), cs.data_ptr(), ws.data_ptr(),
                       blocks_per_sm=(16,), trial_groups=(8, 16, 32), treelets=(0,), chunks=(1,), seed=99)
    learned_group = tune["best"][1]
    ctx.set_proposal(None)
    ctx.set_launch(0, 0)
    ctx.set_trial_group(0)
    ctx.set_treelet(0)

    def render(spp, seed, offset, learned, stats=None):
        ctx.set_proposal(prop if learned else None, 0.1)
        ctx.set_trial_group(learned_group if learned else 0)
        if stats is not None:
            ctx.reset_stats()
            ctx.set_profiling(True)
        per_call = max(1, (1 << 21) // npix)
        acc = torch.zeros(npix, dtype=torch.float64, device=f"cuda:{dev}")
        ms = 0.0
        done = 0
        while done < spp:
            k = min(per_call, spp - done)
            q = torch.from_numpy(np.tile(pix, (1, k))).to(f"cuda:{dev}")
            v, t = connect_timed(torch, sms, ctx, "ss", q, npix * k, seed=seed, stream_offset=offset + done * npix)
            acc += v[0].view(k, npix).double().sum(0)
            ms += t
            done += k
        ctx.set_proposal(None)
        if stats is not None:
            st, pr = ctx.stats(), ctx.profile()
            ctx.set_profiling(False)
            conns = npix * spp
            stats.update({
                "first_ms": pr["ss_first"]["ms"], "trials_ms": pr["ss_trials"]["ms"],
                "queued_fraction": st["bernoulli_trial_calls"] / conns,
                "trials_per_queued": st["bernoulli_trial_iterations"] / max(1, st["bernoulli_trial_calls"]),
                "walks_per_connection": st["walks"] / conns,
                "speculative_walks_per_connection": st["speculative_walks"] / conns,
                "newton_iterations_per_walk": st["newton_iterations"] / max(1, st["walks"]),
                "first_walk_converged": st["solver_succeeded"] / max(1, st["solver_succeeded"] + st["solver_failed"]),
            })
        return (acc / spp).cpu().numpy(), ms

    ref, ref_ms = render(ref_spp, 11, 1 << 30, False)
    rows = []
    for learned in (False, True):
        for spp in (8, 16, 32, 64):
            extra = {} if spp == 64 else None
            img, ms = render(spp, 12 + spp, 1 << 28, learned, extra)
            rmse = float(np.sqrt(np.mean((img - ref) ** 2)))
            row = {"seeding": "learned" if learned else "uniform", "spp": spp, "ms": ms, "rmse": rmse}
            if extra:
                row["profile"] = extra
            rows.append(row)
    uni64 = next(r for r in rows if r["seeding"] == "uniform" and r["spp"] == 64)
    reach = [r for r in rows if r["seeding"] == "learned" and r["rmse"] <= uni64["rmse"]]
    t_equal = min(r["ms"] for r in reach) if reach else None
    # least-squares fit MSE(spp) = a / spp + b per seeding over the renders (b:
    # the reference's own noise and the truncation-bias difference); time per
    # sample from the 64-spp render.  Equal-RMSE time ratio = (a t)_uniform /
    # (a t)_learned.
    fit = {}
    for mode in ("uniform", "learned"):
        rs = [r for r in rows if r["seeding"] == mode]
        A = np.array([[1.0 / r["spp"], 1.0] for r in rs])
        y = np.array([r["rmse"] ** 2 for r in rs])
        (a, b), *_ = np.linalg.lstsq(A, y, rcond=None)
        t1 = next(r["ms"] for r in rs if r["spp"] == 64) / 64.0
        fit[mode] = {"mse_per_sample": float(a), "mse_floor": float(b), "ms_per_sample": t1}
    t_equal_fit = None
    if fit["learned"]["mse_per_sample"] > 0:
        t_equal_fit = uni64["ms"] * (fit["learned"]["mse_per_sample"] * fit["learned"]["ms_per_sample"]) / (
            fit["uniform"]["mse_per_sample"] * fit["uniform"]["ms_per_sample"])
    # per-sample efficiency: MSE x time at 64 spp (lower is better)
    eff = {}
    for mode in ("uniform", "learned"):
        r = next(x for x in rows if x["seeding"] == mode and x["spp"] == 64)
        eff[mode] = r["rmse"] ** 2 * r["ms"]
    prop.close()
    return {
        "workload": f"water 512^2 unbiased (trials<=256), {res}x{res} receiver image, reference {ref_spp} spp uniform",
        "pairs": total, "collect_ms": t_collect.ms, "collect_queries": calls * chunk,
        "train": {"steps": steps, "batch": batch, "lr": lr, "loss_start": loss0, "loss_end": loss,
                  "ms_per_step": step_ms, "wall_s": train_wall,
                  "roofline": {"bound": "tensor", "achieved": flop_step / (step_ms / 1e3) / 1e12,
                               "unit": "TFLOP/s", "flop_per_step": flop_step}},
        "reference_ms": ref_ms,
        "learned_trial_group": learned_group,
        "renders": rows,
        "learned_ms_to_uniform64_rmse": t_equal,
        "time_ratio_to_equal_rmse": (uni64["ms"] / t_equal) if t_equal else None,
        "time_ratio_to_equal_rmse_fit": (uni64["ms"] / t_equal_fit) if t_equal_fit else None,
        "mse_fit": fit,
        "mse_x_time_ratio_64spp": eff["uniform"] / max(eff["learned"], 1e-30),
    }


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    sms = load_package()
    from sms_gb300 import workloads as W
    cores = os.cpu_count() or 1
    sample = int(os.environ.get("SMS_REF_SAMPLE", str(N_QUERIES)))
    vals = []
    for _ in range(args.warmup):
        cpu_baseline_sample(sms, W, 1024, cores)
    times = []
    for _ in range(args.steps):
        v, dt, n = cpu_baseline_sample(sms, W, sample, cores)
        vals.append(v)
        times.append(dt)
    value = float(np.sum([sample] * len(times)) / np.sum(times))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(times)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": {"workload": WORKLOAD, "sample_queries_per_step": sample},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"first {sample} of the 1M queries per step"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    dev = local if torch.cuda.is_available() else 0
    torch.cuda.set_device(dev)
    sms = load_package()
    from sms_gb300 import workloads as W

    n = args.queries
    desc = W.water_scene()
    cfg = W.water_config()
    ctx = sms.Context(sms.Scene(desc), cfg, device=dev)
    ss = sms.SpecularManifoldSingleScatter(ctx)
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)
    first, offset = shard(rank, n)
    q_host = W.water_queries(n, first=first)
    q_dev = torch.from_numpy(q_host).to(f"cuda:{dev}")
    val = torch.empty((3, n), dtype=torch.float32, device=f"cuda:{dev}")
    cnt = torch.empty(n, dtype=torch.int32, device=f"cuda:{dev}")
    wlk = torch.empty(n, dtype=torch.int32, device=f"cuda:{dev}")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{dev}")

    def step(seed):
        with torch.cuda.stream(stream):
            flush.zero_()   # L2 flush between steps (256 MiB write)
        ss.specular_manifold_sampling_device(q_dev.data_ptr(), n, val.data_ptr(), cnt.data_ptr(),
                                             wlk.data_ptr(), seed=seed, stream_offset=offset)

    tuned = None
    if not args.no_autotune:
        # launch shape (blocks per SM x trial group) picked on a quarter of the
        # step's queries; no shape changes a result
        from sms_gb300.autotune import autotune_ss
        m = max(1, n // 4)
        tuned = autotune_ss(sms, ctx, q_dev.data_ptr(), m, val.data_ptr(), cnt.data_ptr(), wlk.data_ptr())
    for i in range(args.warmup):
        step(100 + i)
    torch.cuda.synchronize()
    ctx.reset_stats()
    ctx.set_profiling(True)
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(dev)
    clocks.start()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    t0 = time.perf_counter()
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            ev[i][0].record(stream)
        ss.specular_manifold_sampling_device(q_dev.data_ptr(), n, val.data_ptr(), cnt.data_ptr(),
                                             wlk.data_ptr(), seed=1 + i, stream_offset=offset)
        with torch.cuda.stream(stream):
            ev[i][1].record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    step_ms_list = [a.elapsed_time(b) for a, b in ev]
    st = ctx.stats()
    prof = ctx.profile()
    ctx.set_profiling(False)

    # e2e through the host-pointer C-ABI call, pinned host buffers
    qh = torch.from_numpy(q_host).pin_memory()
    vh = torch.empty((3, n), dtype=torch.float32).pin_memory()
    ch = torch.empty(n, dtype=torch.int32).pin_memory()
    wh = torch.empty(n, dtype=torch.int32).pin_memory()
    import ctypes as C
    lib = sms.load_library()
    res = sms._Result(vh.data_ptr(), ch.data_ptr(), wh.data_ptr())
    sms._check(lib.sms_ss_connect_batch(ctx.handle, qh.data_ptr(), n, 200, offset, C.byref(res)))
    e2e_t = []
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        sms._check(lib.sms_ss_connect_batch(ctx.handle, qh.data_ptr(), n, 1 + i, offset, C.byref(res)))
        e2e_t.append(time.perf_counter() - t1)
    clk = clocks.stop()

    step_ms = float(np.mean(step_ms_list))
    total_s = float(np.sum(step_ms_list)) / 1e3
    e2e_s = float(np.sum(e2e_t))
    total_s, e2e_s = max_over_ranks(torch, [total_s, e2e_s], f"cuda:{dev}")
    value = world * n * args.steps / total_s
    e2e_value = world * n * args.steps / e2e_s

    # Roofline of the dominant kernel.  Algorithmic bytes per launch = the BVH
    # nodes (32 B each; a device node record holds two) and triangles (36 B)
    # its traversals fetch, as counted by the kernel.  Its FP32 work = rays x
    # FLOPs per ray + box tests x FLOPs per box + triangle tests x FLOPs per
    # triangle, the per-unit figures counted by the oracle on this workload.
    phases = {k: v for k, v in prof.items() if v["launches"]}
    dom = max(phases, key=lambda k: phases[k]["ms"])
    dp = phases[dom]
    per_launch_ms = dp["ms"] / dp["launches"]
    alg_bytes = (dp["bvh_nodes"] * NODE_RECORD_BYTES + dp["tri_tests"] * TRIANGLE_BYTES) / dp["launches"]
    peak, peak_kind = peaks()
    achieved = alg_bytes / (per_launch_ms / 1e3) / 1e9
    units = flops_per_unit().get("water_512_unbiased")
    fp32 = None
    if units:
        flops = fp32_work(units, dp["rays"], 2 * dp["bvh_nodes"], dp["tri_tests"]) / dp["launches"]
        tf = flops / (per_launch_ms / 1e3) / 1e12
        fp32 = {"achieved_tflops": tf, "peak_tflops": fp32_peak_tflops(), "frac": tf / fp32_peak_tflops(),
                "peak_kind": "nominal: 152 SMs x 128 lanes x FMA x 2070 MHz", "flops_per_launch": flops,
                "flops_per_ray": units["flops_per_ray"], "flops_per_box": units["flops_per_box"],
                "flops_per_triangle": units["flops_per_triangle"],
                "note": "FLOPs counted by the oracle's op-counting build on this workload "
                        "(profiles/flops_per_unit.json) x the kernel's own ray / box / triangle counts "
                        "(speculative trial walks included)"}
    traffic = None
    tpath = ROOT / "profiles" / "traffic.json"
    if tpath.exists():
        traffic = json.loads(tpath.read_text()).get(dom)
    gpu_launches = int(sum(v["launches"] for v in phases.values()))
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "queries_per_step": n, "l2": "flushed between steps (256 MiB write)",
                   "parallelism": f"replicas x{world}",
                   "launch": ({"blocks_per_sm": tuned["best"][0], "trial_group": tuned["best"][1],
                               "treelet_nodes": tuned["best"][2], "queue_chunk": tuned["best"][3],
                               "autotune_ms": tuned["ms"]} if tuned else "library default")},
        "walks_per_s": world * st["walks"] / total_s,
        "newton_iterations_per_walk": st["newton_iterations"] / max(1, st["walks"]),
        "trials_per_connection": st["bernoulli_trial_iterations"] / max(1, st["bernoulli_trial_calls"]),
        "converged_fraction_first_walk": st["solver_succeeded"] / max(1, st["solver_succeeded"] + st["solver_failed"]),
        "rays_per_s": world * st["rays"] / total_s,
        "speculative_walk_fraction": st["speculative_walks"] / max(1, st["walks"] + st["speculative_walks"]),
        "phases_ms_per_step": {k: v["ms"] / args.steps for k, v in phases.items()},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                     "bytes_per_launch": alg_bytes, "launch_ms": per_launch_ms, "fp32": fp32,
                     "note": "algorithmic bytes = BVH nodes (32 B; two per device node record) + triangles "
                             "(36 B) fetched by the kernel's traversals; the scene is L2-resident, so DRAM "
                             "traffic stays far below; the kernel is latency- and issue-bound (fp32)"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": n * 16 * 4,
                "d2h_bytes_per_step": n * 5 * 4},
        "gpu_launches": gpu_launches,
        "clocks": clk,
        "wall_s": wall,
    }
    if rank == 0 and world == 1 and not args.no_learned:
        bf16_peak = None
        pp = ROOT / "MEASURED_PEAKS.json"
        if pp.exists():
            bf16_peak = json.loads(pp.read_text()).get("bf16_tflops")
        lt = learned_study(torch, sms, W, ctx, dev, pairs=args.learned_pairs, steps=args.learned_steps,
                           ref_spp=args.ref_spp)
        rl = lt["train"]["roofline"]
        rl["peak"] = bf16_peak or 1900.0
        rl["frac"] = rl["achieved"] / rl["peak"]
        rl["peak_kind"] = "measured" if bf16_peak else "fallback"
        line["learned"] = lt
    if rank == 0 and world == 1 and not args.no_configs:
        line["configs"] = secondary_configs(torch, sms, W, dev)
    if rank == 0 and world == 1 and not args.no_render:
        line["render"] = render_study(torch, sms, W, dev, args.render_size, args.render_size, args.render_spp)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import oracle as O
        cores = os.cpu_count() or 1
        sample = int(os.environ.get("SMS_CPU_SAMPLE", str(N_QUERIES)))
        osc = O.OracleScene(W.water_scene())
        v, dt, ns = cpu_baseline_sample(sms, W, sample, cores, osc=osc)
        v1, dt1, ns1 = cpu_baseline_sample(sms, W, 8192, 1, osc=osc)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": f"first {ns} of the 1M queries, {dt:.1f} s; single thread: first "
                                          f"{ns1} queries, {dt1:.1f} s",
                                "single_thread": v1, "build": "g++ -O3, binned-SAH tree, std::thread per core",
                                "configs": cpu_baseline_configs(sms, W, cores),
                                "parity_sample": basin_sample(sms, W, ctx)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-proposal study")
    ap.add_argument("--no-autotune", action="store_true", help="library default launch shape")
    ap.add_argument("--queries", type=int, default=N_QUERIES, help="queries per step (smaller cases for ncu)")
    ap.add_argument("--learned-pairs", type=int, default=4 << 20)
    ap.add_argument("--learned-steps", type=int, default=20000)
    ap.add_argument("--ref-spp", type=int, default=4096)
    ap.add_argument("--no-configs", action="store_true", help="skip the sphere / slab / glint configurations")
    ap.add_argument("--no-render", action="store_true", help="skip the path-tracer images")
    ap.add_argument("--render-only", action="store_true",
                    help="only the path-tracer images (one JSON object; for profiling the renderer)")
    ap.add_argument("--secondary-only", default=None,
                    help="only this secondary configuration, 3 warm-up and `--steps` timed calls (one JSON "
                         "object; for profiling its kernel)")
    ap.add_argument("--render-size", type=int, default=512)
    ap.add_argument("--render-spp", type=int, default=16)
    args = ap.parse_args()
    if args.render_only:
        import torch
        sms = load_package()
        from sms_gb300 import workloads as W
        print(json.dumps({"render": render_study(torch, sms, W, 0, args.render_size, args.render_size,
                                                 args.render_spp)}), flush=True)
        return
    if args.secondary_only:
        import torch
        sms = load_package()
        from sms_gb300 import workloads as W
        mq = args.queries if args.queries != N_QUERIES else None
        print(json.dumps({"configs": secondary_configs(torch, sms, W, 0, only=args.secondary_only,
                                                       calls=args.steps, max_queries=mq,
                                                       tune=not args.no_autotune)}), flush=True)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
