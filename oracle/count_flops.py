"""Algorithmic FP32 work per unit of the benchmark workloads, counted by the
oracle's op-counting build (liboracle_ops.so, oracle/op_count.h).

TEST / MEASUREMENT INFRASTRUCTURE ONLY: it runs the oracle on a sample of
each benchmark configuration and writes profiles/flops_per_unit.json, which
bench.py reads to turn the kernels' own ray, BVH-node and triangle counts into
FLOP/s.  Nothing in the library imports it.

  python oracle/count_flops.py            (about a minute on 8 cores)
"""
from __future__ import annotations

import importlib.util
import json
import os
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
# run as a script, sys.path[0] is oracle/ itself, where "oracle" would name oracle.py
sys.path[:] = [str(ROOT)] + [p for p in sys.path if Path(p or ".").resolve() != ROOT / "oracle"]


def _package():
    if "sms_gb300" in sys.modules:
        return sys.modules["sms_gb300"]
    pkg = ROOT / "specular-manifold-sampling_gb300"
    spec = importlib.util.spec_from_file_location("sms_gb300", pkg / "__init__.py",
                                                  submodule_search_locations=[str(pkg)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["sms_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def main() -> None:
    _package()
    from sms_gb300 import workloads as W
    from oracle import oracle as O
    O.build()
    nt = os.cpu_count() or 1
    cases = {
        "water_512_unbiased": (W.water_scene(), W.water_config(), W.water_queries(16384), {}),
        "sphere_biased_m16": (W.sphere_scene(), W.sphere_config(), W.sphere_queries(64), {}),
        "sphere_conductor_biased_m16": (W.sphere_scene(conductor=True), W.sphere_config(), W.sphere_queries(64), {}),
        "slab_two_bounce_biased_m32": (W.slab_scene(), W.slab_config(), W.slab_queries(4096), {"multi": True}),
        "glints_8192_vectorized_m64": (W.glint_scene(), W.glint_config(), W.glint_queries(1024)[:, ::64],
                                       {"glints": True}),
    }
    out = {"how": "python oracle/count_flops.py: the oracle's counting build on a sample of each benchmark "
                  "configuration; add, sub, mul, div, sqrt and transcendentals count 1 FLOP each (an FMA is 2)",
           "configs": {}}
    for name, (desc, cfg, q, kw) in cases.items():
        r = O.flops_per_unit(desc, cfg, q, seed=1, nthreads=nt, **kw)
        st = r.pop("stats")
        c = r.pop("counts")
        r["sample_queries"] = r.pop("queries")
        r["newton_iterations_per_walk"] = st["newton_iterations"] / max(1, st["walks"])
        r["rays_per_walk"] = c["rays"] / max(1, st["walks"])
        r["counts"] = c
        out["configs"][name] = r
        print(name, {k: round(v, 2) for k, v in r.items() if isinstance(v, float)}, flush=True)
    path = ROOT / "profiles" / "flops_per_unit.json"
    path.write_text(json.dumps(out, indent=1) + "\n")
    print("wrote", path)


if __name__ == "__main__":
    main()
