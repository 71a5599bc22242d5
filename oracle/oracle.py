"""ctypes binding of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline / reference arm of bench.py, always as the checker or the CPU
baseline, never as part of the GPU library.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
LIB_PATH = ORACLE_DIR / "liboracle.so"
FMA_LIB_PATH = ORACLE_DIR / "liboracle_fma.so"
# The four builds of sms_oracle.cpp (oracle/Makefile): FP32 (the oracle proper),
# FP32 with FMA contraction (chaos floor), FP64 (basin classifier) and FP32 on
# the counting scalar of op_count.h (operation counts, results identical to f32).
VARIANT_PATHS = {"f32": LIB_PATH, "fma": FMA_LIB_PATH, "f64": ORACLE_DIR / "liboracle_f64.so",
                 "ops": ORACLE_DIR / "liboracle_ops.so"}
OP_COUNT_NAMES = ("add", "mul", "div", "sqrt", "transcendental", "box_tests", "triangle_tests", "box_flops",
                  "triangle_flops", "rays")

_LIB = None
_LIBS = {}


class _Config(C.Structure):
    _fields_ = [("biased", C.c_int32), ("twostage", C.c_int32),
                ("halfvector_constraints", C.c_int32), ("mnee_init", C.c_int32),
                ("step_scale", C.c_float), ("max_iterations", C.c_int32),
                ("solver_threshold", C.c_float), ("uniqueness_threshold", C.c_float),
                ("max_trials", C.c_int32), ("bounces", C.c_int32),
                ("bsdf_strategy_only", C.c_int32), ("sms_strategy_only", C.c_int32),
                ("glints_vectorized", C.c_int32)]


class _Bsdf(C.Structure):
    _fields_ = [("type", C.c_int32), ("eta", C.c_float), ("k", C.c_float),
                ("albedo", C.c_float * 3), ("alpha", C.c_float), ("twosided", C.c_int32),
                ("nonlinear", C.c_int32)]


class _Camera(C.Structure):
    _fields_ = [("to_world", C.c_float * 16), ("fov", C.c_float), ("fov_axis", C.c_int32),
                ("width", C.c_int32), ("height", C.c_int32), ("near_clip", C.c_float), ("far_clip", C.c_float)]


class _RenderOptions(C.Structure):
    _fields_ = [("integrator", C.c_int32), ("max_depth", C.c_int32), ("rr_depth", C.c_int32),
                ("spp", C.c_int32), ("disable_reflected_emitters", C.c_int32), ("biased_mnee", C.c_int32),
                ("seed", C.c_uint64), ("max_paths", C.c_uint32),
                ("glint_diff_scale_factor_clamp", C.c_float), ("samples_per_pass", C.c_uint32),
                ("timeout", C.c_float), ("caustics_enabled", C.c_int32), ("glints_enabled", C.c_int32),
                ("non_sms_paths_enabled", C.c_int32), ("glints", _Config),
                ("rfilter", C.c_int32), ("rfilter_stddev", C.c_float)]


_INTEGRATORS = {"path": 0, "path_sms_ss": 1, "path_sms_ms": 2, "path_sms_glints": 3, "path_filtered_ss": 4,
                "path_filtered_ms": 5, "path_sms_teaser": 6, "path_filtered_teaser": 7}
_FOV_AXES = {"x": 0, "y": 1, "diagonal": 2, "smaller": 3, "larger": 4}


def build() -> Path:
    """Compile the oracle's four builds with the committed Makefile."""
    r = subprocess.run(["make", "-s", "-j4", "-C", str(ORACLE_DIR)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB_PATH


def load(fma: bool = False, variant: str | None = None):
    """The oracle library; fma=True gives the FMA-contracted build used to
    measure the floating-point chaos floor; variant picks any of the builds
    of VARIANT_PATHS by name."""
    global _LIB
    key = variant or ("fma" if fma else "f32")
    if key in _LIBS:
        return _LIBS[key]
    path = VARIANT_PATHS[key]
    if not path.exists():
        build()
    lib = C.CDLL(str(path))
    vp, i32, u32, u64, f32 = C.c_void_p, C.c_int32, C.c_uint32, C.c_uint64, C.c_float
    sig = {
        "oracle_scene_create": (vp, []),
        "oracle_scene_destroy": (None, [vp]),
        "oracle_scene_add_sphere": (i32, [vp, C.POINTER(f32), f32, i32, C.POINTER(_Bsdf), u32]),
        "oracle_scene_add_mesh": (i32, [vp, vp, vp, vp, u32, vp, u32, C.POINTER(_Bsdf), u32]),
        "oracle_scene_add_point_emitter": (i32, [vp, C.POINTER(f32), C.POINTER(f32), u32]),
        "oracle_scene_add_area_emitter": (i32, [vp, i32, C.POINTER(f32), u32]),
        "oracle_scene_finalize": (None, [vp]),
        "oracle_ss_walk_batch": (i32, [vp, C.POINTER(_Config), i32, vp, vp, u32, vp]),
        "oracle_ss_connect_batch": (i32, [vp, C.POINTER(_Config), vp, u32, u64, u64, vp, vp, vp, C.c_int,
                                          vp]),
        "oracle_ms_walk_batch": (i32, [vp, C.POINTER(_Config), i32, vp, vp, u32, vp]),
        "oracle_ms_connect_batch": (i32, [vp, C.POINTER(_Config), vp, u32, u64, u64, vp, vp, vp, C.c_int, vp]),
        "oracle_scene_set_normalmap": (i32, [vp, i32, vp, u32, f32]),
        "oracle_scene_set_lean_fallback": (i32, [vp, f32, f32, f32]),
        "oracle_lean_fb_eval": (i32, [vp, vp, vp, u32, vp]),
        "oracle_lean_fb_sample": (i32, [vp, vp, vp, u32, vp]),
        "oracle_shape_bsdf_eval": (i32, [vp, i32, vp, vp, u32, vp]),
        "oracle_shape_bsdf_sample": (i32, [vp, i32, vp, vp, u32, vp]),
        "oracle_roughplastic_tables": (i32, [vp, i32, vp]),
        "oracle_glint_walk_batch": (i32, [vp, C.POINTER(_Config), vp, vp, u32, vp]),
        "oracle_glint_connect_batch": (i32, [vp, C.POINTER(_Config), vp, u32, u64, u64, vp, vp, vp, C.c_int, vp]),
        "oracle_nm_slope": (None, [vp, f32, f32, vp]),
        "oracle_ss_emitter_batch": (i32, [vp, vp, u32, u64, u64, vp]),
        "oracle_ss_step_at": (i32, [vp, i32, i32, f32, f32, vp, vp, vp]),
        "oracle_ss_connect_learned_batch": (i32, [vp, C.POINTER(_Config), vp, u32, u64, u64, i32, f32, vp, vp,
                                                  vp, vp, vp, C.c_int, vp]),
        "oracle_fresnel": (f32, [f32, f32, C.POINTER(f32)]),
        "oracle_glint_lean_pdf": (f32, [vp, f32, f32, vp, vp, vp]),
        "oracle_render": (i32, [vp, C.POINTER(_Config), C.POINTER(_Camera), C.POINTER(_RenderOptions), vp, C.c_int]),
        "oracle_fresnel_conductor": (f32, [f32, f32, f32]),
        "oracle_uniform_sphere": (None, [f32, f32, C.POINTER(f32)]),
        "oracle_sample_slope_gaussian": (None, [vp, f32, f32, f32, vp, vp]),
        "oracle_pcg32": (None, [u64, u64, u32, vp]),
        "oracle_pcg32_f32": (None, [u64, u64, u32, vp]),
        "oracle_build_kind": (i32, []),
        "oracle_opcount_read": (None, [vp]),
        "oracle_opcount_reset": (None, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIBS[key] = lib
    if key == "f32":
        _LIB = lib
    return lib


def op_counts(lib) -> dict:
    """Operation counts of the counting build since the last reset_op_counts."""
    out = np.zeros(len(OP_COUNT_NAMES), np.uint64)
    lib.oracle_opcount_read(out.ctypes.data)
    d = dict(zip(OP_COUNT_NAMES, (int(x) for x in out)))
    d["flops"] = sum(d[k] for k in OP_COUNT_NAMES[:5])
    return d


def reset_op_counts(lib) -> None:
    lib.oracle_opcount_reset()


def flops_per_unit(desc, config, queries, seed: int = 1, nthreads: int | None = None, **kw) -> dict:
    """Algorithmic FP32 work of one connection batch, from the counting build:
    FLOPs per ray cast outside the traversal (Newton steps, vertex builds,
    sampling, contributions: all non-traversal work divided by the rays cast),
    per BVH box test and per ray-triangle test.  A kernel's FLOPs are then
    rays x per_ray + box tests x per_box + triangle tests x per_triangle with
    its own counts (its tree differs from the oracle's)."""
    lib = load(variant="ops")
    sc = OracleScene(desc, variant="ops")
    reset_op_counts(lib)
    _, _, _, st = sc.connect_batch(config, queries, seed=seed, nthreads=nthreads, **kw)
    c = op_counts(lib)
    trav = c["box_flops"] + c["triangle_flops"]
    return {"flops_per_ray": (c["flops"] - trav) / max(1, c["rays"]),
            "flops_per_box": c["box_flops"] / max(1, c["box_tests"]),
            "flops_per_triangle": c["triangle_flops"] / max(1, c["triangle_tests"]),
            "flops_per_newton_iteration": c["flops"] / max(1, st["newton_iterations"]),
            "transcendentals_per_newton_iteration": c["transcendental"] / max(1, st["newton_iterations"]),
            "counts": c, "stats": st, "queries": int(queries.shape[1])}


def _f3(v):
    return (C.c_float * 3)(*[float(x) for x in v])


def _cfg(config) -> _Config:
    c = _Config()
    for name, _ in _Config._fields_:
        setattr(c, name, getattr(config, name))
    return c


def _bsdf(b) -> _Bsdf:
    r = _Bsdf()
    r.type, r.eta, r.k = b.type, b.eta, b.k
    r.albedo[:] = [float(x) for x in b.albedo]
    r.alpha = float(getattr(b, "alpha", 0.0))
    r.twosided = int(getattr(b, "twosided", False))
    r.nonlinear = int(getattr(b, "nonlinear", False))
    return r


class OracleScene:
    """The oracle's copy of a SceneDesc (same shape ids, same emitter order)."""

    def __init__(self, desc, fma: bool = False, variant: str | None = None):
        lib = load(fma, variant)
        self._lib = lib
        self._h = lib.oracle_scene_create()
        self._keep = []
        for kind, idx in desc.order:
            if kind == "sphere":
                c, r, flip, b, flags = desc.spheres[idx]
                lib.oracle_scene_add_sphere(self._h, _f3(c), r, int(flip), C.byref(_bsdf(b)), flags)
            else:
                P, N, UV, F, b, flags = desc.meshes[idx]
                self._keep += [P, N, UV, F]
                lib.oracle_scene_add_mesh(self._h, P.ctypes.data, None if N is None else N.ctypes.data,
                                          None if UV is None else UV.ctypes.data, P.shape[0],
                                          F.ctypes.data, F.shape[0], C.byref(_bsdf(b)), flags)
        for pos, I, flags in desc.point_emitters:
            lib.oracle_scene_add_point_emitter(self._h, _f3(pos), _f3(I), flags)
        for sid, L, flags in desc.area_emitters:
            lib.oracle_scene_add_area_emitter(self._h, sid, _f3(L), flags)
        if getattr(desc, "normalmap", None) is not None:
            sid, slopes, tiles = desc.normalmap
            sl = np.ascontiguousarray(slopes, np.float16)
            self._keep.append(sl)
            lib.oracle_scene_set_normalmap(self._h, sid, sl.ctypes.data, sl.shape[0], tiles)
            if getattr(desc, "lean_fallback", None) is not None:
                a, e, k = desc.lean_fallback
                if lib.oracle_scene_set_lean_fallback(self._h, float(a), float(e), float(k)) != 0:
                    raise ValueError("lean fallback without a normal map")
        lib.oracle_scene_finalize(self._h)

    def lean_fb_eval(self, wi: np.ndarray, wo: np.ndarray) -> np.ndarray:
        """The normal map's LEAN fallback BSDF for local-frame pairs (3, n):
        rows eval (BSDF x cos_o), pdf."""
        a = np.ascontiguousarray(wi, np.float32)
        b = np.ascontiguousarray(wo, np.float32)
        out = np.zeros((2, a.shape[1]), np.float32)
        if self._lib.oracle_lean_fb_eval(self._h, a.ctypes.data, b.ctypes.data, a.shape[1], out.ctypes.data) != 0:
            raise ValueError("the scene has no LEAN fallback")
        return out

    def lean_fb_sample(self, wi: np.ndarray, u: np.ndarray) -> np.ndarray:
        """Sampling of the LEAN fallback from local wi (3, n) with numbers u
        (2, n): rows ok, wo (3), weight, pdf."""
        a = np.ascontiguousarray(wi, np.float32)
        uu = np.ascontiguousarray(u, np.float32)
        out = np.zeros((6, a.shape[1]), np.float32)
        if self._lib.oracle_lean_fb_sample(self._h, a.ctypes.data, uu.ctypes.data, a.shape[1], out.ctypes.data) != 0:
            raise ValueError("the scene has no LEAN fallback")
        return out

    def shape_bsdf_eval(self, shape: int, wi: np.ndarray, wo: np.ndarray) -> np.ndarray:
        """A shape's BSDF for local-frame pairs (3, n): rows eval (BSDF x
        cos_o, 3), pdf."""
        a = np.ascontiguousarray(wi, np.float32)
        b = np.ascontiguousarray(wo, np.float32)
        out = np.zeros((4, a.shape[1]), np.float32)
        if self._lib.oracle_shape_bsdf_eval(self._h, shape, a.ctypes.data, b.ctypes.data, a.shape[1],
                                            out.ctypes.data) != 0:
            raise ValueError(f"no shape {shape}")
        return out

    def shape_bsdf_sample(self, shape: int, wi: np.ndarray, u: np.ndarray) -> np.ndarray:
        """Sampling of a shape's BSDF from local wi (3, n) with numbers u (3,
        n): rows ok, wo (3), weight (3), pdf."""
        a = np.ascontiguousarray(wi, np.float32)
        uu = np.ascontiguousarray(u, np.float32)
        out = np.zeros((8, a.shape[1]), np.float32)
        if self._lib.oracle_shape_bsdf_sample(self._h, shape, a.ctypes.data, uu.ctypes.data, a.shape[1],
                                              out.ctypes.data) != 0:
            raise ValueError(f"no shape {shape}")
        return out

    def roughplastic_tables(self, shape: int) -> np.ndarray:
        """A roughplastic shape's transmittance table (64), internal
        reflectance and specular sampling weight."""
        out = np.zeros(66, np.float32)
        if self._lib.oracle_roughplastic_tables(self._h, shape, out.ctypes.data) != 0:
            raise ValueError(f"shape {shape} is not roughplastic")
        return out

    def walk_batch(self, config, caster: int, queries: np.ndarray, walk_in: np.ndarray) -> np.ndarray:
        n = queries.shape[1]
        q = np.ascontiguousarray(queries, np.float32)
        w = np.ascontiguousarray(walk_in, np.float32)
        if w.shape != (10 if config.twostage else 8, n):
            raise ValueError(f"walk_in shape {w.shape} does not fit the config")
        out = np.zeros((11, n), np.float32)
        self._lib.oracle_ss_walk_batch(self._h, C.byref(_cfg(config)), caster, q.ctypes.data, w.ctypes.data, n,
                                  out.ctypes.data)
        return out

    def ms_walk_batch(self, config, caster: int, queries: np.ndarray, walk_in: np.ndarray) -> np.ndarray:
        """Multi-scatter first-path walks: rows ok, iterations, first vertex (3),
        last vertex (3), seed-path ok."""
        n = queries.shape[1]
        q = np.ascontiguousarray(queries, np.float32)
        w = np.ascontiguousarray(walk_in, np.float32)
        out = np.zeros((9, n), np.float32)
        self._lib.oracle_ms_walk_batch(self._h, C.byref(_cfg(config)), caster, q.ctypes.data, w.ctypes.data, n,
                                       out.ctypes.data)
        return out

    def glint_walk_batch(self, config, queries: np.ndarray, walk_in: np.ndarray) -> np.ndarray:
        """sample_glint with explicit light point (rows 0-2) and footprint
        sample (rows 3-4); out rows ok, iterations, uv_final (2), uv_init (2)."""
        n = queries.shape[1]
        q = np.ascontiguousarray(queries, np.float32)
        w = np.ascontiguousarray(walk_in, np.float32)
        out = np.zeros((6, n), np.float32)
        self._lib.oracle_glint_walk_batch(self._h, C.byref(_cfg(config)), q.ctypes.data, w.ctypes.data, n,
                                          out.ctypes.data)
        return out

    def slope(self, u: float, v: float) -> np.ndarray:
        out = np.zeros(6, np.float32)
        self._lib.oracle_nm_slope(self._h, u, v, out.ctypes.data)
        return out

    def connect_batch(self, config, queries: np.ndarray, seed: int = 0, stream_offset: int = 0,
                      nthreads: int | None = None, multi: bool = False, glints: bool = False):
        n = queries.shape[1]
        q = np.ascontiguousarray(queries, np.float32)
        value = np.zeros((3, n), np.float32)
        count = np.zeros(n, np.int32)
        walks = np.zeros(n, np.int32)
        stats = np.zeros(8, np.uint64)
        nt = nthreads or os.cpu_count() or 1
        fn = (self._lib.oracle_glint_connect_batch if glints else
              self._lib.oracle_ms_connect_batch if multi else self._lib.oracle_ss_connect_batch)
        fn(self._h, C.byref(_cfg(config)), q.ctypes.data, n, seed, stream_offset, value.ctypes.data,
           count.ctypes.data, walks.ctypes.data, nt, stats.ctypes.data)
        names = ["solver_succeeded", "solver_failed", "bernoulli_trial_calls", "bernoulli_trial_iterations",
                 "bernoulli_trial_iterations_max", "walks", "newton_iterations", "connections"]
        return value, count, walks, dict(zip(names, stats.tolist()))

    def step_at(self, shape: int, halfvector: bool, u: float, v: float, x, lp) -> np.ndarray:
        """ok, C (2), J (2x2 row-major) of the single-scatter Newton step at the
        sphere point with uv (u, v)."""
        out = np.zeros(7, np.float32)
        xa = np.ascontiguousarray(x, np.float32)
        la = np.ascontiguousarray(lp, np.float32)
        self._lib.oracle_ss_step_at(self._h, shape, int(halfvector), u, v, xa.ctypes.data, la.ctypes.data,
                                    out.ctypes.data)
        return out

    def emitter_batch(self, queries: np.ndarray, seed: int = 0, stream_offset: int = 0) -> np.ndarray:
        """The single-scatter estimator's emitter sample per query: rows ei.p
        (3), valid."""
        n = queries.shape[1]
        q = np.ascontiguousarray(queries, np.float32)
        out = np.zeros((4, n), np.float32)
        self._lib.oracle_ss_emitter_batch(self._h, q.ctypes.data, n, seed, stream_offset, out.ctypes.data)
        return out

    def connect_learned_batch(self, config, queries: np.ndarray, shape: int, defensive: float, frame: np.ndarray,
                              mixture: np.ndarray, seed: int = 0, stream_offset: int = 0,
                              nthreads: int | None = None):
        """Unbiased single scatter seeded by a learned proposal: mixture is the
        processed per-query mixture (40 x n), frame the caster's uv frame."""
        n = queries.shape[1]
        q = np.ascontiguousarray(queries, np.float32)
        fr = np.ascontiguousarray(frame, np.float32)
        mx = np.ascontiguousarray(mixture, np.float32)
        assert mx.shape == (40, n) and fr.shape == (10,)
        value = np.zeros((3, n), np.float32)
        count = np.zeros(n, np.int32)
        walks = np.zeros(n, np.int32)
        stats = np.zeros(8, np.uint64)
        nt = nthreads or os.cpu_count() or 1
        self._lib.oracle_ss_connect_learned_batch(self._h, C.byref(_cfg(config)), q.ctypes.data, n, seed,
                                                  stream_offset, shape, defensive, fr.ctypes.data, mx.ctypes.data,
                                                  value.ctypes.data, count.ctypes.data, walks.ctypes.data, nt,
                                                  stats.ctypes.data)
        names = ["solver_succeeded", "solver_failed", "bernoulli_trial_calls", "bernoulli_trial_iterations",
                 "bernoulli_trial_iterations_max", "walks", "newton_iterations", "connections"]
        return value, count, walks, dict(zip(names, stats.tolist()))

    def glint_lean_pdf(self, u: float, v: float, duv, wi, wo) -> float:
        """LEAN-mapping density of the glints integrator's MIS (local frame)."""
        a = np.ascontiguousarray(duv, np.float32)
        b = np.ascontiguousarray(wi, np.float32)
        c = np.ascontiguousarray(wo, np.float32)
        return float(self._lib.oracle_glint_lean_pdf(self._h, u, v, a.ctypes.data, b.ctypes.data, c.ctypes.data))

    def render(self, config, camera, options, nthreads: int | None = None) -> np.ndarray:
        """The library's sms_render restated path by path: camera / options
        are objects with the fields of the library's Camera / RenderOptions."""
        cam = _Camera()
        M = np.asarray(camera.to_world, np.float32).reshape(16)
        for k in range(16):
            cam.to_world[k] = float(M[k])
        cam.fov, cam.fov_axis = camera.fov, _FOV_AXES[camera.fov_axis]
        cam.width, cam.height = int(camera.width), int(camera.height)
        cam.near_clip, cam.far_clip = camera.near_clip, camera.far_clip
        o = _RenderOptions()
        o.integrator = _INTEGRATORS[options.integrator]
        o.max_depth, o.rr_depth, o.spp = options.max_depth, options.rr_depth, options.spp
        o.disable_reflected_emitters = int(options.disable_reflected_emitters)
        o.biased_mnee, o.seed, o.max_paths = int(options.biased_mnee), options.seed, options.max_paths
        o.glint_diff_scale_factor_clamp = float(getattr(options, "glint_diff_scale_factor_clamp", 0.0))
        o.caustics_enabled = int(getattr(options, "caustics_enabled", True))
        o.glints_enabled = int(getattr(options, "glints_enabled", True))
        o.non_sms_paths_enabled = int(getattr(options, "non_sms_paths_enabled", True))
        o.rfilter = {"box": 0, "gaussian": 1}[getattr(options, "rfilter", "box")]
        o.rfilter_stddev = float(getattr(options, "rfilter_stddev", 0.5))
        gcfg = getattr(options, "glints", None)
        if gcfg is not None:
            o.glints = _cfg(gcfg)
        else:   # SMSConfig defaults (manifold.h:11-45)
            o.glints.step_scale, o.glints.max_iterations, o.glints.solver_threshold = 1.0, 20, 1e-5
            o.glints.uniqueness_threshold, o.glints.max_trials, o.glints.bounces = 1e-4, -1, 2
        img = np.zeros((camera.height, camera.width, 3), np.float32)
        nt = nthreads or os.cpu_count() or 1
        self._lib.oracle_render(self._h, C.byref(_cfg(config)), C.byref(cam), C.byref(o), img.ctypes.data, nt)
        return img

    def __del__(self):
        if getattr(self, "_h", None) and getattr(self, "_lib", None) is not None:
            self._lib.oracle_scene_destroy(self._h)
            self._h = None


def sample_slope_gaussian(mu, a: float, b: float, c: float, u) -> np.ndarray:
    """The two-stage solver's slope draw from N(mu, (a, c; c, b)) for the
    uniform pair u (manifold.h:326-345)."""
    m = np.ascontiguousarray(mu, np.float32)
    uu = np.ascontiguousarray(u, np.float32)
    out = np.zeros(2, np.float32)
    load().oracle_sample_slope_gaussian(m.ctypes.data, a, b, c, uu.ctypes.data, out.ctypes.data)
    return out
