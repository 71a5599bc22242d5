"""Generate the golden fixtures under tests/golden/ (run from the repo root:
``python tests/golden/make_golden.py``).

  kat.json             known-answer values:
                       * PCG32 (initstate 42, initseq 54): the first outputs of
                         O'Neill's reference demo for the generator the
                         reference's independent sampler uses
                         (include/mitsuba/core/random.h:50-52);
                       * Fresnel values asserted by the reference's own test
                         src/librender/tests/test_fresnel.py:7-39 (read as text);
                       * square_to_uniform_sphere corner values
                         (include/mitsuba/core/warp.h:262-267).
  sphere_analytic.json specular solutions on the benchmark sphere (centre
                       (0,0,1.5), radius 1, light (0,0,5)) for shading points on
                       z=0, found independently in FP64 by a 1-D root find in the
                       plane of incidence: mirror reflection (conductor) and
                       refraction into the sphere (IOR 1.5).
  oracle_small.npz     oracle outputs on small cases (regression pin of the
                       restatement; the GPU tests compare the library to the
                       oracle run live on the same host).
  oracle_nm.npz        the same for normal-mapped casters: per-walk outputs
                       with the two-stage solver and unbiased estimates with
                       and without it on the 4-period normal-mapped plane
                       (``--only nm`` regenerates this file alone).
"""
from __future__ import annotations

import importlib.util
import json
import math
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
OUT = Path(__file__).resolve().parent


def load_package():
    spec = importlib.util.spec_from_file_location(
        "sms_gb300", ROOT / "specular-manifold-sampling_gb300" / "__init__.py",
        submodule_search_locations=[str(ROOT / "specular-manifold-sampling_gb300")])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["sms_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


# ------------------------------------------------------------ analytic sphere
C = np.array([0.0, 0.0, 1.5])
R = 1.0
L = np.array([0.0, 0.0, 5.0])


def _unit(v):
    return v / np.linalg.norm(v)


def _refract(w, n, eta_):
    """Direction of travel after refraction of the ray that arrives along -w
    (w points away from the surface), relative IOR eta_ inside."""
    eta = 1.0 / eta_
    if w @ n < 0:
        eta = 1.0 / eta
        n = -n
    c = w @ n
    root = 1.0 - eta * eta * (1.0 - c * c)
    if root < 0:
        return None
    return -eta * (w - c * n) - n * math.sqrt(root)


def _residual(theta, x, mode):
    """Signed in-plane mismatch at the sphere point at polar angle theta in the
    vertical plane through x (x on the +x axis after rotation)."""
    v = C + R * np.array([math.sin(theta), 0.0, -math.cos(theta)])
    n = (v - C) / R
    wi = _unit(x - v)
    wo = _unit(L - v)
    if mode == "reflect":
        if wi @ n <= 0 or wo @ n <= 0:
            return None
        t = 2.0 * (wi @ n) * n - wi
    else:
        t = _refract(wi, n, 1.5)
        if t is None or (wi @ n) * (wo @ n) >= 0:
            return None
    return t[0] * wo[2] - t[2] * wo[0], v


def solve(rho, mode):
    """All solutions for a shading point at distance rho from the axis."""
    x = np.array([rho, 0.0, 0.0])
    thetas = np.linspace(-math.pi, math.pi, 20001)
    sols = []
    prev = None
    for th in thetas:
        r = _residual(th, x, mode)
        if r is not None and prev is not None and np.sign(r[0]) != np.sign(prev[1][0]):
            a, b = prev[0], th
            fa = prev[1][0]
            for _ in range(200):
                m = 0.5 * (a + b)
                rm = _residual(m, x, mode)
                if rm is None:
                    break
                if np.sign(rm[0]) == np.sign(fa):
                    a, fa = m, rm[0]
                else:
                    b = m
            rm = _residual(0.5 * (a + b), x, mode)
            if rm is not None and abs(rm[0]) < 1e-12:
                # the ray from x must reach v before any other part of the sphere
                v = rm[1]
                d = _unit(v - x)
                oc = x - C
                bq = oc @ d
                disc = bq * bq - (oc @ oc - R * R)
                t_near = -bq - math.sqrt(max(disc, 0.0))
                if abs(t_near - np.linalg.norm(v - x)) < 1e-9:
                    sols.append((0.5 * (a + b), v.tolist()))
        prev = (th, r) if r is not None else None
    return sols


def analytic_cases():
    cases = []
    for mode in ("reflect", "refract"):
        for rho in [round(0.1 * k, 2) for k in range(1, 21)]:
            for th, v in solve(rho, mode):
                cases.append({"mode": mode, "x": [rho, 0.0, 0.0], "theta": th, "solution": v})
    return cases


def nm_cases(sms, W, O):
    desc = W.nm_plane_scene(freq=4)
    osc = O.OracleScene(desc)
    n = 128
    q = W.nm_plane_queries(n)
    w = np.zeros((10, n), np.float32)
    w[0:3] = np.array([0.3, -0.2, 4.0], np.float32)[:, None]
    w[6:10] = W.pcg32_streams_f32(13, np.arange(n, dtype=np.uint64), 4)
    res = {"nm_walk_twostage": osc.walk_batch(sms.SMSConfig(twostage=True), 0, q, w)}
    for two in (False, True):
        cfg = sms.SMSConfig(biased=False, max_trials=64, twostage=two)
        v, c, wk, st = osc.connect_batch(cfg, W.nm_plane_queries(256), seed=9, nthreads=1)
        tag = "twostage" if two else "plain"
        res[f"nm_{tag}_value"], res[f"nm_{tag}_count"], res[f"nm_{tag}_walks"] = v, c, wk
    return res


def main():
    sms = load_package()
    from sms_gb300 import workloads as W
    sys.path.insert(0, str(ROOT))
    from oracle import oracle as O

    np.savez_compressed(OUT / "oracle_nm.npz", **nm_cases(sms, W, O))
    if "--only" in sys.argv and sys.argv[sys.argv.index("--only") + 1] == "nm":
        print("wrote oracle_nm.npz")
        return

    r = W.Pcg32(42, 54)
    kat = {
        "pcg32_42_54_u32": [r.next_u32() for _ in range(6)],
        # test_fresnel.py:11-16 (cos_theta_i, eta) -> (F, cos_theta_t)
        "fresnel": [
            [1.0, 1.5, 0.04, -1.0],
            [-1.0, 1.5, 0.04, 1.0],
            [1.0, 1.0 / 1.5, 0.04, -1.0],
            [-1.0, 1.0 / 1.5, 0.04, 1.0],
            [0.0, 1.5, 1.0, -math.sqrt(1 - 1 / 1.5 ** 2)],
            [0.0, 1.0 / 1.5, 1.0, 0.0],
            # test_fresnel.py:18-27: 45 degrees, 1 -> 1.5
            [math.cos(math.radians(45)), 1.5, 0.5 * (0.09201336304552442 ** 2 + 0.3033370452904235 ** 2),
             -math.cos(math.radians(28.1255057020557))],
            # test_fresnel.py:29-32: 45 degrees, 1.5 -> 1 (total internal reflection)
            [math.cos(math.radians(45)), 1.0 / 1.5, 1.0, 0.0],
            # test_fresnel.py:34-39: 10 degrees, 1.5 -> 1
            [math.cos(math.radians(10)), 1.0 / 1.5, 0.5 * (0.19046797197779405 ** 2 + 0.20949431963852014 ** 2),
             -math.cos(math.radians(15.098086605159006))],
        ],
        # square_to_uniform_sphere(u, v) = (r cos 2pi u, r sin 2pi u, 1 - 2v)
        "uniform_sphere": [[0.0, 0.0, 0.0, 0.0, 1.0], [0.0, 1.0, 0.0, 0.0, -1.0],
                           [0.0, 0.5, 1.0, 0.0, 0.0], [0.25, 0.5, 0.0, 1.0, 0.0]],
    }
    (OUT / "kat.json").write_text(json.dumps(kat, indent=1))
    cases = analytic_cases()
    (OUT / "sphere_analytic.json").write_text(json.dumps(cases, indent=1))

    # oracle regression pins (small)
    res = {}
    for cond in (False, True):
        desc = W.sphere_scene(conductor=cond)
        q = W.sphere_queries(16)
        o = O.OracleScene(desc)
        v, c, w, st = o.connect_batch(W.sphere_config(), q, seed=1, nthreads=1)
        tag = "cond" if cond else "glass"
        res[f"sphere_{tag}_value"], res[f"sphere_{tag}_count"] = v, c
    desc = W.water_scene(res=64)
    q = W.water_queries(256)
    v, c, w, st = O.OracleScene(desc).connect_batch(W.water_config(), q, seed=5, nthreads=1)
    res["water64_value"], res["water64_count"], res["water64_walks"] = v, c, w
    np.savez_compressed(OUT / "oracle_small.npz", **res)
    print(f"wrote kat.json, sphere_analytic.json ({len(cases)} solutions), oracle_small.npz")


if __name__ == "__main__":
    main()
