"""GB300 (sm_103a) Specular Manifold Sampling -- host-side Python mirror.

The product is the C-ABI library ``libsms_gb300.so`` (declared in
``include/sms_gb300.h``).  This module binds it with ctypes and mirrors the
reference's Python-facing interface for the SMS path
(src/librender/python/manifold_v.cpp:8-100):

    SMSConfig                        include/mitsuba/render/manifold.h:11-45
    SpecularManifoldSingleScatter    include/mitsuba/render/manifold_ss.h
        .specular_manifold_sampling  manifold_ss.cpp:28-201 (batched)
        .sample_path(..., p_start)   manifold_ss.cpp:203-279 (batched)

Where the reference takes one SurfaceInteraction per call, these methods take a
wavefront of shading points as arrays.  Loading fails loudly when the compiled
library is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field, fields
from pathlib import Path

import numpy as np

PKG_DIR = Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "libsms_gb300.so"

QUERY_FIELDS = 16
NOALLOC_MAX_QUERIES = 1 << 18
WALK_IN_FIELDS = 8
SS_WALK_IN_FIELDS_TWOSTAGE = 10
WALK_OUT_FIELDS = 11
MS_WALK_OUT_FIELDS = 9
GLINT_QUERY_FIELDS = 21
GLINT_WALK_IN_FIELDS = 5
GLINT_WALK_OUT_FIELDS = 6

SHAPE_CAUSTIC_RECEIVER = 1 << 0
SHAPE_CAUSTIC_CASTER_SINGLE = 1 << 1
SHAPE_CAUSTIC_CASTER_MULTI = 1 << 2
SHAPE_CAUSTIC_BOUNCER = 1 << 3
SHAPE_GLINTY = 1 << 4
EMITTER_CAUSTIC_SINGLE = 1 << 0
EMITTER_CAUSTIC_MULTI = 1 << 1

BSDF_DIFFUSE, BSDF_DIELECTRIC, BSDF_CONDUCTOR, BSDF_ROUGHPLASTIC = 0, 1, 2, 3

PROPOSAL_FEATURES = 9
PROPOSAL_OUTPUTS = 40
PROPOSAL_PARAMS = 21808

RFILTERS = {"box": 0, "gaussian": 1}
INTEGRATORS = {"path": 0, "path_sms_ss": 1, "path_sms_ms": 2, "path_sms_glints": 3, "path_filtered_ss": 4,
               "path_filtered_ms": 5, "path_sms_teaser": 6, "path_filtered_teaser": 7}
FOV_AXES = {"x": 0, "y": 1, "diagonal": 2, "smaller": 3, "larger": 4}

STATUS_NAMES = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "device limit",
                4: "unsupported", 5: "parse error", 6: "no device"}


class SMSError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


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


class _Result(C.Structure):
    _fields_ = [("value", C.c_void_p), ("count", C.c_void_p), ("walks", C.c_void_p)]


class _MeshData(C.Structure):
    _fields_ = [("n_vertices", C.c_uint32), ("n_faces", C.c_uint32), ("positions", C.POINTER(C.c_float)),
                ("normals", C.POINTER(C.c_float)), ("texcoords", C.POINTER(C.c_float)),
                ("faces", C.POINTER(C.c_uint32))]


class _Stats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in (
        "solver_succeeded", "solver_failed", "bernoulli_trial_calls",
        "bernoulli_trial_iterations", "bernoulli_trial_iterations_max", "walks",
        "newton_iterations", "connections", "rays", "bvh_nodes", "tri_tests",
        "speculative_walks")]


PHASES = ["ss_first", "ss_trials", "ss_biased", "ss_walk", "ms", "glints", "ms_walk", "glint_walk"]


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


class _Profile(C.Structure):
    _fields_ = [("ms", C.c_double * 8), ("launches", C.c_uint64 * 8), ("rays", C.c_uint64 * 8),
                ("bvh_nodes", C.c_uint64 * 8), ("tri_tests", C.c_uint64 * 8)]


_LIB = None


def load_library(path: str | os.PathLike | None = None):
    """Load libsms_gb300.so (raises if it has not been built)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with build.py (no CPU fallback exists)")
    lib = C.CDLL(str(p))
    vp, i32, u32, u64, f32 = C.c_void_p, C.c_int32, C.c_uint32, C.c_uint64, C.c_float
    sig = {
        "sms_last_error": (C.c_char_p, []),
        "sms_config_default": (None, [C.POINTER(_Config)]),
        "sms_config_parse_xml": (i32, [C.c_char_p, C.POINTER(_Config), C.c_char_p, C.c_size_t]),
        "sms_scene_create": (i32, [C.POINTER(vp)]),
        "sms_scene_destroy": (None, [vp]),
        "sms_scene_add_sphere": (i32, [vp, C.POINTER(f32), f32, i32, C.POINTER(_Bsdf), u32, C.POINTER(i32)]),
        "sms_scene_add_mesh": (i32, [vp, vp, vp, vp, u32, vp, u32, C.POINTER(_Bsdf), u32, C.POINTER(i32)]),
        "sms_scene_add_point_emitter": (i32, [vp, C.POINTER(f32), C.POINTER(f32), u32]),
        "sms_scene_add_area_emitter": (i32, [vp, i32, C.POINTER(f32), u32]),
        "sms_ctx_create": (i32, [vp, C.POINTER(_Config), i32, C.POINTER(vp)]),
        "sms_ctx_destroy": (None, [vp]),
        "sms_ctx_set_config": (i32, [vp, C.POINTER(_Config)]),
        "sms_ctx_stream": (vp, [vp]),
        "sms_ctx_set_launch": (i32, [vp, i32, i32]),
        "sms_ctx_set_trial_group": (i32, [vp, i32]),
        "sms_ctx_set_treelet": (i32, [vp, i32]),
        "sms_ctx_set_queue_chunk": (i32, [vp, i32]),
        "sms_stats_read": (i32, [vp, C.POINTER(_Stats)]),
        "sms_stats_reset": (i32, [vp]),
        "sms_ctx_set_profiling": (i32, [vp, i32]),
        "sms_profile_read": (i32, [vp, C.POINTER(_Profile)]),
        "sms_ss_connect_batch": (i32, [vp, vp, u32, u64, u64, C.POINTER(_Result)]),
        "sms_ss_connect_batch_device": (i32, [vp, vp, u32, u64, u64, C.POINTER(_Result)]),
        "sms_ss_walk_batch": (i32, [vp, i32, vp, vp, u32, vp]),
        "sms_ss_connect_batch_noalloc": (i32, [vp, vp, u32, u64, u64, C.POINTER(_Result)]),
        "sms_ms_connect_batch": (i32, [vp, vp, u32, u64, u64, C.POINTER(_Result)]),
        "sms_ms_connect_batch_device": (i32, [vp, vp, u32, u64, u64, C.POINTER(_Result)]),
        "sms_ms_walk_batch": (i32, [vp, i32, vp, vp, u32, vp]),
        "sms_scene_set_normalmap": (i32, [vp, i32, vp, u32, f32]),
        "sms_scene_set_lean_fallback": (i32, [vp, f32, f32, f32]),
        "sms_glint_connect_batch": (i32, [vp, vp, u32, u64, u64, C.POINTER(_Result)]),
        "sms_glint_connect_batch_device": (i32, [vp, vp, u32, u64, u64, C.POINTER(_Result)]),
        "sms_glint_walk_batch": (i32, [vp, vp, vp, u32, vp]),
        "sms_proposal_create": (i32, [vp, i32, u64, u32, C.POINTER(vp)]),
        "sms_proposal_destroy": (i32, [vp]),
        "sms_proposal_collect": (i32, [vp, vp, u32, u64, u64, i32, C.POINTER(u32)]),
        "sms_proposal_set_data": (i32, [vp, vp, vp, vp, u32]),
        "sms_proposal_get_data": (i32, [vp, vp, vp, vp, u32, C.POINTER(u32)]),
        "sms_proposal_set_options": (i32, [vp, f32, i32]),
        "sms_proposal_normalize": (i32, [vp]),
        "sms_proposal_train": (i32, [vp, i32, i32, f32, C.POINTER(f32)]),
        "sms_proposal_loss_grad": (i32, [vp, i32, C.POINTER(f32), vp]),
        "sms_proposal_get_state": (i32, [vp, vp, vp, vp, vp, C.POINTER(u32)]),
        "sms_proposal_set_state": (i32, [vp, vp, vp, vp, vp, u32]),
        "sms_proposal_eval": (i32, [vp, vp, u32, i32, vp]),
        "sms_ctx_set_proposal": (i32, [vp, vp, f32]),
        "sms_proposal_frame": (i32, [vp, vp]),
        "sms_obj_load": (i32, [C.c_char_p, i32, i32, C.POINTER(_MeshData)]),
        "sms_mesh_data_free": (None, [C.POINTER(_MeshData)]),
        "sms_render_options_default": (None, [C.POINTER(_RenderOptions)]),
        "sms_render_sms_seed": (u64, [u64]),
        "sms_render": (i32, [vp, C.POINTER(_Camera), C.POINTER(_RenderOptions), vp]),
        "sms_render_spp_done": (u32, [vp]),
        "sms_render_device": (i32, [vp, C.POINTER(_Camera), C.POINTER(_RenderOptions), vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def _check(status: int):
    if status != 0:
        msg = _LIB.sms_last_error().decode() if _LIB is not None else ""
        raise SMSError(status, msg)


def _f3(v) -> C.Array:
    a = (C.c_float * 3)(*[float(x) for x in v])
    return a


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


# ------------------------------------------------------------------ config
@dataclass
class SMSConfig:
    """Same fields, names and defaults as the reference's SMSConfig."""
    biased: bool = False
    twostage: bool = False
    halfvector_constraints: bool = False
    mnee_init: bool = False
    step_scale: float = 1.0
    max_iterations: int = 20
    solver_threshold: float = 1e-5
    uniqueness_threshold: float = 1e-4
    max_trials: int = -1
    bounces: int = 1
    bsdf_strategy_only: bool = False
    sms_strategy_only: bool = False
    glints_vectorized: bool = False

    def to_c(self) -> _Config:
        c = _Config()
        for f in fields(self):
            setattr(c, f.name, getattr(self, f.name))
        return c

    @staticmethod
    def from_c(c: _Config) -> "SMSConfig":
        kw = {}
        for f in fields(SMSConfig):
            v = getattr(c, f.name)
            kw[f.name] = bool(v) if f.type in ("bool", bool) else v
        return SMSConfig(**kw)

    @staticmethod
    def from_xml(xml: str) -> tuple["SMSConfig", str]:
        """Parse an <integrator type="path_sms_*"> block like the reference's
        integrator constructors (path_sms_ss.cpp:47-61)."""
        lib = load_library()
        c = _Config()
        buf = C.create_string_buffer(64)
        _check(lib.sms_config_parse_xml(xml.encode(), C.byref(c), buf, 64))
        return SMSConfig.from_c(c), buf.value.decode()


def default_config() -> SMSConfig:
    lib = load_library()
    c = _Config()
    lib.sms_config_default(C.byref(c))
    return SMSConfig.from_c(c)


# ------------------------------------------------------------------- scene
@dataclass
class Bsdf:
    type: int = BSDF_DIFFUSE
    eta: float = 1.0
    k: float = 0.0
    albedo: tuple = (0.5, 0.5, 0.5)
    alpha: float = 0.0       # Beckmann roughness (rough dielectric / conductor), 0 = smooth
    twosided: bool = False   # the BSDF acts on both sides (twosided.cpp); not a dielectric
    nonlinear: bool = False  # roughplastic's nonlinear internal scattering

    def to_c(self) -> _Bsdf:
        b = _Bsdf()
        b.type, b.eta, b.k = self.type, self.eta, self.k
        b.albedo[:] = [float(x) for x in self.albedo]
        b.alpha = self.alpha
        b.twosided = int(self.twosided)
        b.nonlinear = int(self.nonlinear)
        return b


@dataclass
class SceneDesc:
    """Backend-neutral scene description (shapes + emitters) that can be
    instantiated on the GPU library or, in tests, on the CPU oracle."""
    spheres: list = field(default_factory=list)   # (center, radius, flip, Bsdf, flags)
    meshes: list = field(default_factory=list)    # (P, N, UV, F, Bsdf, flags)
    order: list = field(default_factory=list)     # ("sphere"|"mesh", index) in shape-id order
    point_emitters: list = field(default_factory=list)  # (pos, I, flags)
    normalmap: tuple | None = None   # (shape_id, (res, res, 2) float16 slopes, tiles)
    lean_fallback: tuple | None = None   # the normal map's LEAN fallback BSDF: (alpha, eta, k)
    area_emitters: list = field(default_factory=list)   # (shape_id, L, flags)

    def add_sphere(self, center, radius, bsdf: Bsdf, flags: int = 0, flip: bool = False) -> int:
        self.spheres.append((tuple(center), float(radius), bool(flip), bsdf, flags))
        self.order.append(("sphere", len(self.spheres) - 1))
        return len(self.order) - 1

    def add_mesh(self, P, F, bsdf: Bsdf, flags: int = 0, N=None, UV=None) -> int:
        P = np.ascontiguousarray(P, dtype=np.float32).reshape(-1, 3)
        F = np.ascontiguousarray(F, dtype=np.uint32).reshape(-1, 3)
        N = None if N is None else np.ascontiguousarray(N, dtype=np.float32).reshape(-1, 3)
        UV = None if UV is None else np.ascontiguousarray(UV, dtype=np.float32).reshape(-1, 2)
        self.meshes.append((P, N, UV, F, bsdf, flags))
        self.order.append(("mesh", len(self.meshes) - 1))
        return len(self.order) - 1

    def add_obj(self, path, bsdf: Bsdf, flags: int = 0, face_normals: bool = False,
                flip_tex_coords: bool = True) -> int:
        """Add a Wavefront OBJ mesh (the reference's obj shape plugin)."""
        P, F, N, UV = load_obj(path, face_normals, flip_tex_coords)
        return self.add_mesh(P, F, bsdf, flags, N=N, UV=UV)

    def add_point_emitter(self, pos, intensity, flags: int = EMITTER_CAUSTIC_SINGLE):
        self.point_emitters.append((tuple(pos), tuple(intensity), flags))

    def add_area_emitter(self, shape_id: int, radiance, flags: int = EMITTER_CAUSTIC_SINGLE):
        self.area_emitters.append((shape_id, tuple(radiance), flags))


def load_scene(path):
    """(SceneDesc, SMSConfig or None, integrator type or None) from a scene XML
    file in the reference's format (the subset described in scene_xml.py)."""
    import sys
    from .scene_xml import load_scene_xml
    return load_scene_xml(sys.modules[__name__], path)


def load_render_setup(path):
    """(Camera, RenderOptions) from a scene file's <sensor> and <integrator>."""
    import sys
    from .scene_xml import load_render_setup as _lrs
    return _lrs(sys.modules[__name__], path)


def load_obj(path, face_normals: bool = False, flip_tex_coords: bool = True):
    """(positions (nv, 3), faces (nf, 3), normals (nv, 3) or None, texcoords
    (nv, 2) or None) of a Wavefront OBJ file, read by the library."""
    lib = load_library()
    m = _MeshData()
    _check(lib.sms_obj_load(str(path).encode(), int(face_normals), int(flip_tex_coords), C.byref(m)))
    try:
        nv, nf = m.n_vertices, m.n_faces
        P = np.ctypeslib.as_array(m.positions, shape=(nv, 3)).copy()
        F = np.ctypeslib.as_array(m.faces, shape=(nf, 3)).copy()
        N = np.ctypeslib.as_array(m.normals, shape=(nv, 3)).copy() if m.normals else None
        UV = np.ctypeslib.as_array(m.texcoords, shape=(nv, 2)).copy() if m.texcoords else None
    finally:
        lib.sms_mesh_data_free(C.byref(m))
    return P, F, N, UV


class Scene:
    """Host-side scene builder of the GPU library (sms_scene)."""

    def __init__(self, desc: SceneDesc):
        lib = load_library()
        h = C.c_void_p()
        _check(lib.sms_scene_create(C.byref(h)))
        self._h = h
        self.desc = desc
        self._keep = []
        for kind, idx in desc.order:
            sid = C.c_int32()
            if kind == "sphere":
                c, r, flip, b, flags = desc.spheres[idx]
                _check(lib.sms_scene_add_sphere(h, _f3(c), r, int(flip), C.byref(b.to_c()), flags,
                                                C.byref(sid)))
            else:
                P, N, UV, F, b, flags = desc.meshes[idx]
                self._keep += [P, N, UV, F]
                _check(lib.sms_scene_add_mesh(h, _ptr(P), None if N is None else _ptr(N),
                                              None if UV is None else _ptr(UV), P.shape[0], _ptr(F),
                                              F.shape[0], C.byref(b.to_c()), flags, C.byref(sid)))
        for pos, I, flags in desc.point_emitters:
            _check(lib.sms_scene_add_point_emitter(h, _f3(pos), _f3(I), flags))
        for sid, L, flags in desc.area_emitters:
            _check(lib.sms_scene_add_area_emitter(h, sid, _f3(L), flags))
        if desc.normalmap is not None:
            sid, slopes, tiles = desc.normalmap
            sl = np.ascontiguousarray(slopes, np.float16)
            if sl.ndim != 3 or sl.shape[0] != sl.shape[1] or sl.shape[2] != 2:
                raise ValueError("slopes must have shape (res, res, 2)")
            self._keep.append(sl)
            _check(lib.sms_scene_set_normalmap(h, sid, _ptr(sl), sl.shape[0], float(tiles)))
        if desc.lean_fallback is not None:
            a, e, k = desc.lean_fallback
            _check(lib.sms_scene_set_lean_fallback(h, float(a), float(e), float(k)))

    @property
    def handle(self):
        return self._h

    def __del__(self):
        if getattr(self, "_h", None) and _LIB is not None:
            _LIB.sms_scene_destroy(self._h)
            self._h = None


class Context:
    """Device copy of a scene plus solver config (sms_ctx)."""

    def __init__(self, scene: Scene, config: SMSConfig, device: int = 0):
        lib = load_library()
        h = C.c_void_p()
        _check(lib.sms_ctx_create(scene.handle, C.byref(config.to_c()), device, C.byref(h)))
        self._h = h
        self.config = config

    @property
    def handle(self):
        return self._h

    @property
    def stream(self) -> int:
        return _LIB.sms_ctx_stream(self._h) or 0

    def set_config(self, config: SMSConfig):
        _check(_LIB.sms_ctx_set_config(self._h, C.byref(config.to_c())))
        self.config = config

    def set_launch(self, blocks_per_sm: int = 0, threads_per_block: int = 0):
        _check(_LIB.sms_ctx_set_launch(self._h, blocks_per_sm, threads_per_block))

    def set_trial_group(self, group: int = 0):
        """Lanes per query of the Bernoulli-trial kernel (0 auto, 8, 16, 32)."""
        _check(_LIB.sms_ctx_set_trial_group(self._h, group))

    def set_treelet(self, nodes: int = 0):
        """Top node records of the tree the Bernoulli-trial kernel stages in
        shared memory (0..384, 0 = none)."""
        _check(_LIB.sms_ctx_set_treelet(self._h, nodes))

    def set_queue_chunk(self, chunk: int = 1):
        """Queries a Bernoulli-trial lane group claims per atomic (1..64)."""
        _check(_LIB.sms_ctx_set_queue_chunk(self._h, chunk))

    def stats(self) -> dict:
        s = _Stats()
        _check(_LIB.sms_stats_read(self._h, C.byref(s)))
        return {n: getattr(s, n) for n, _ in _Stats._fields_}

    def reset_stats(self):
        _check(_LIB.sms_stats_reset(self._h))

    def set_profiling(self, enable: bool = True):
        _check(_LIB.sms_ctx_set_profiling(self._h, int(enable)))

    def profile(self) -> dict:
        """Per-phase kernel time (CUDA events) and traversal counters."""
        p = _Profile()
        _check(_LIB.sms_profile_read(self._h, C.byref(p)))
        return {name: {"ms": p.ms[k], "launches": p.launches[k], "rays": p.rays[k],
                       "bvh_nodes": p.bvh_nodes[k], "tri_tests": p.tri_tests[k]}
                for k, name in enumerate(PHASES)}

    def render(self, camera: "Camera", options: "RenderOptions") -> np.ndarray:
        """Image (height, width, 3) float32 of the path tracer (sms_render)."""
        img = np.zeros((camera.height, camera.width, 3), np.float32)
        _check(_LIB.sms_render(self._h, C.byref(camera.to_c()), C.byref(options.to_c()), _ptr(img)))
        return img

    def render_spp_done(self) -> int:
        """Samples per pixel of the last render (fewer than spp after a timeout)."""
        return int(_LIB.sms_render_spp_done(self._h))

    def render_device(self, camera: "Camera", options: "RenderOptions", image_ptr: int):
        """Render into a device buffer of height * width * 3 floats."""
        _check(_LIB.sms_render_device(self._h, C.byref(camera.to_c()), C.byref(options.to_c()), image_ptr))

    def set_proposal(self, proposal: "SeedProposal | None", defensive: float = 0.1):
        """Seed the unbiased single-scatter estimator from a learned proposal
        (None restores uniform seeding)."""
        _check(_LIB.sms_ctx_set_proposal(self._h, proposal.handle if proposal else None, defensive))
        self._proposal = proposal

    def close(self):
        if getattr(self, "_h", None) and _LIB is not None:
            _LIB.sms_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


class SeedProposal:
    """Learned seed proposal for one single-scatter caster (sms_proposal).

    No counterpart in the reference, whose walks are seeded uniformly on the
    caster (manifold_ss.cpp:223).  The network maps (shading point, light
    sample, shading normal) to an 8-component Gaussian mixture over the
    caster's uv frame; bound with Context.set_proposal it seeds the unbiased
    estimator, mixed with the uniform seeding."""

    def __init__(self, ctx: Context, caster: int, seed: int = 0, capacity: int = 1 << 22):
        h = C.c_void_p()
        _check(_LIB.sms_proposal_create(ctx.handle, caster, seed, capacity, C.byref(h)))
        self._h = h
        self._ctx = ctx
        self.capacity = capacity

    @property
    def handle(self):
        return self._h

    def collect(self, queries_ptr: int, n: int, seed: int = 0, stream_offset: int = 0,
                walks_per_query: int = 1) -> int:
        """Append the solver's converged uniform-seed walks for device queries;
        returns the pairs held."""
        total = C.c_uint32()
        _check(_LIB.sms_proposal_collect(self._h, queries_ptr, n, seed, stream_offset, walks_per_query,
                                         C.byref(total)))
        return total.value

    def set_data(self, features: np.ndarray, uv: np.ndarray, weights: np.ndarray | None = None):
        n = features.shape[1]
        f = _soa(features, PROPOSAL_FEATURES, n)
        u = _soa(uv, 2, n)
        w = None if weights is None else np.ascontiguousarray(weights, np.float32).reshape(n)
        _check(_LIB.sms_proposal_set_data(self._h, _ptr(f), _ptr(u), None if w is None else _ptr(w), n))

    def get_data(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """Training set: features (9 x n), uv (2 x n), weights (n)."""
        n = C.c_uint32()
        _check(_LIB.sms_proposal_get_data(self._h, None, None, None, 0, C.byref(n)))
        f = np.zeros((PROPOSAL_FEATURES, n.value), np.float32)
        u = np.zeros((2, n.value), np.float32)
        w = np.zeros(n.value, np.float32)
        _check(_LIB.sms_proposal_get_data(self._h, _ptr(f), _ptr(u), _ptr(w), n.value, C.byref(n)))
        return f, u, w

    def set_options(self, sigma_scale: float = 1.0, weighted: bool = True):
        """Seeding sharpness (sigma multiplier) and contribution-weighted training."""
        _check(_LIB.sms_proposal_set_options(self._h, sigma_scale, int(weighted)))

    def normalize(self):
        _check(_LIB.sms_proposal_normalize(self._h))

    def train(self, steps: int, batch: int = 8192, lr: float = 1e-3) -> float:
        loss = C.c_float()
        _check(_LIB.sms_proposal_train(self._h, steps, batch, lr, C.byref(loss)))
        return loss.value

    def loss_grad(self, batch: int) -> tuple[float, np.ndarray]:
        loss = C.c_float()
        g = np.zeros(PROPOSAL_PARAMS, np.float32)
        _check(_LIB.sms_proposal_loss_grad(self._h, batch, C.byref(loss), _ptr(g)))
        return loss.value, g

    def state(self) -> dict:
        p, m, v = (np.zeros(PROPOSAL_PARAMS, np.float32) for _ in range(3))
        norm = np.zeros(2 * PROPOSAL_FEATURES, np.float32)
        step = C.c_uint32()
        _check(_LIB.sms_proposal_get_state(self._h, _ptr(p), _ptr(m), _ptr(v), _ptr(norm), C.byref(step)))
        return {"params": p, "adam_m": m, "adam_v": v, "norm": norm, "step": step.value}

    def load_state(self, st: dict):
        arr = {k: np.ascontiguousarray(st[k], np.float32) for k in ("params", "adam_m", "adam_v", "norm")
               if st.get(k) is not None}
        _check(_LIB.sms_proposal_set_state(
            self._h, _ptr(arr["params"]), _ptr(arr["adam_m"]) if "adam_m" in arr else None,
            _ptr(arr["adam_v"]) if "adam_v" in arr else None, _ptr(arr["norm"]) if "norm" in arr else None,
            int(st.get("step", 0))))

    def save(self, path):
        """Checkpoint (weights, Adam state, normalisation, step) as .npz."""
        np.savez(path, **self.state())

    def load(self, path):
        with np.load(path) as z:
            self.load_state({k: z[k] for k in z.files})

    def frame(self) -> np.ndarray:
        """kind, org (3), ax_u (3), ax_v (3) of the caster's uv frame."""
        f = np.zeros(10, np.float32)
        _check(_LIB.sms_proposal_frame(self._h, _ptr(f)))
        return f

    def eval(self, features: np.ndarray, mixture: bool = False) -> np.ndarray:
        """Raw outputs (40 x n) or the processed mixture: cdf (8), means
        (8 x 2), sigmas (8 x 2)."""
        n = features.shape[1]
        f = _soa(features, PROPOSAL_FEATURES, n)
        out = np.zeros((PROPOSAL_OUTPUTS, n), np.float32)
        _check(_LIB.sms_proposal_eval(self._h, _ptr(f), n, int(mixture), _ptr(out)))
        return out

    def close(self):
        if getattr(self, "_h", None) and _LIB is not None:
            _LIB.sms_proposal_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


# --------------------------------------------------------------- rendering
@dataclass
class Camera:
    """Perspective sensor (src/sensors/perspective.cpp): camera-to-world 4x4
    (camera x left, y up, z forward), field of view in degrees along fov_axis,
    film size, clip distances."""
    to_world: np.ndarray = field(default_factory=lambda: np.eye(4, dtype=np.float32))
    fov: float = 45.0
    width: int = 64
    height: int = 64
    fov_axis: str = "x"
    near_clip: float = 1e-2
    far_clip: float = 1e4

    @staticmethod
    def look_at(origin, target, up, fov: float = 45.0, width: int = 64, height: int = 64,
                fov_axis: str = "x") -> "Camera":
        """The reference's look_at transform (include/mitsuba/core/transform.h):
        columns left, up, forward, origin."""
        o, t, u = (np.asarray(v, np.float64) for v in (origin, target, up))
        d = t - o
        d /= np.linalg.norm(d)
        left = np.cross(u, d)
        left /= np.linalg.norm(left)
        new_up = np.cross(d, left)
        M = np.eye(4)
        M[:3, 0], M[:3, 1], M[:3, 2], M[:3, 3] = left, new_up, d, o
        return Camera(M.astype(np.float32), fov, width, height, fov_axis)

    def to_c(self) -> _Camera:
        c = _Camera()
        M = np.asarray(self.to_world, np.float32).reshape(16)
        for k in range(16):
            c.to_world[k] = float(M[k])
        c.fov = self.fov
        c.fov_axis = FOV_AXES[self.fov_axis]
        c.width, c.height = int(self.width), int(self.height)
        c.near_clip, c.far_clip = self.near_clip, self.far_clip
        return c


@dataclass
class RenderOptions:
    """Integrator parameters: path, path_sms_ss, path_sms_ms, path_sms_glints,
    path_filtered_ss, path_filtered_ms, path_sms_teaser or path_filtered_teaser
    with the MonteCarloIntegrator fields
    (src/librender/integrator.cpp:300-320), the sampling integrator's passes,
    timeout and glint ray-differential clamp (:35-41) and the SMS integrators'
    switches (path_sms_ss.cpp:59-60)."""
    integrator: str = "path_sms_ss"
    max_depth: int = -1
    rr_depth: int = 5
    spp: int = 1
    disable_reflected_emitters: bool = False
    biased_mnee: bool = False
    seed: int = 0
    max_paths: int = 0
    glint_diff_scale_factor_clamp: float = 0.0
    samples_per_pass: int = 0         # 0 = spp (integrator.cpp:35)
    timeout: float = -1.0             # seconds, <= 0: none (integrator.cpp:36)
    # path_sms_teaser (path_sms_teaser.cpp:60-81): the context's config is the
    # caustics_* block, glints the glints_* block
    caustics_enabled: bool = True
    glints_enabled: bool = True
    non_sms_paths_enabled: bool = True
    glints: "SMSConfig | None" = None
    # the film's reconstruction filter: "box" or "gaussian" (the reference
    # film's default, stddev 0.5; src/rfilters/gaussian.cpp)
    rfilter: str = "box"
    rfilter_stddev: float = 0.5

    def to_c(self) -> _RenderOptions:
        o = _RenderOptions()
        o.integrator = INTEGRATORS[self.integrator]
        o.max_depth, o.rr_depth, o.spp = self.max_depth, self.rr_depth, self.spp
        o.disable_reflected_emitters = int(self.disable_reflected_emitters)
        o.biased_mnee = int(self.biased_mnee)
        o.seed, o.max_paths = self.seed, self.max_paths
        o.glint_diff_scale_factor_clamp = self.glint_diff_scale_factor_clamp
        o.samples_per_pass, o.timeout = self.samples_per_pass, self.timeout
        o.caustics_enabled, o.glints_enabled = int(self.caustics_enabled), int(self.glints_enabled)
        o.non_sms_paths_enabled = int(self.non_sms_paths_enabled)
        o.glints = (self.glints or SMSConfig()).to_c()
        o.rfilter = RFILTERS[self.rfilter]
        o.rfilter_stddev = float(self.rfilter_stddev)
        return o


def sms_render_seed(seed: int) -> int:
    """State seed of the path tracer's SMS random-number streams."""
    return int(load_library().sms_render_sms_seed(seed))


def _soa(a: np.ndarray, rows: int, n: int) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    if a.shape != (rows, n):
        raise ValueError(f"expected SoA array of shape ({rows}, {n}), got {a.shape}")
    return a


class SpecularManifoldSingleScatter:
    """Batched SpecularManifoldSingleScatter (include/mitsuba/render/manifold_ss.h)."""

    def __init__(self, ctx: Context):
        self.ctx = ctx

    def specular_manifold_sampling(self, queries: np.ndarray, seed: int = 0, stream_offset: int = 0):
        """queries: (16, n) float32 SoA.  Returns (value (3, n), count (n,), walks (n,))."""
        n = queries.shape[1]
        q = _soa(queries, QUERY_FIELDS, n)
        value = np.zeros((3, n), np.float32)
        count = np.zeros(n, np.int32)
        walks = np.zeros(n, np.int32)
        r = _Result(_ptr(value), _ptr(count), _ptr(walks))
        _check(_LIB.sms_ss_connect_batch(self.ctx.handle, _ptr(q), n, seed, stream_offset, C.byref(r)))
        return value, count, walks

    def specular_manifold_sampling_device(self, queries_ptr: int, n: int, value_ptr: int, count_ptr: int,
                                          walks_ptr: int, seed: int = 0, stream_offset: int = 0):
        """Device-pointer variant (asynchronous on ctx.stream)."""
        r = _Result(value_ptr, count_ptr, walks_ptr)
        _check(_LIB.sms_ss_connect_batch_device(self.ctx.handle, queries_ptr, n, seed, stream_offset,
                                                C.byref(r)))

    def specular_manifold_sampling_noalloc(self, queries_ptr: int, n: int, value_ptr: int, count_ptr: int,
                                           walks_ptr: int, seed: int = 0, stream_offset: int = 0):
        """Allocation-free device-pointer variant (sms_ss_connect_batch_noalloc):
        at most NOALLOC_MAX_QUERIES queries per call; see the C header."""
        r = _Result(value_ptr, count_ptr, walks_ptr)
        _check(_LIB.sms_ss_connect_batch_noalloc(self.ctx.handle, queries_ptr, n, seed, stream_offset,
                                                 C.byref(r)))

    def sample_path(self, caster: int, queries: np.ndarray, walk_in: np.ndarray) -> np.ndarray:
        """Per-walk sample_path with explicit emitter point and start point.
        walk_in: (8, n) rows ei.p(3), p_start(3), sample(2); with the twostage
        solver (10, n), rows 8-9 the smoothed solve's slope sample.  Returns (11, n)."""
        n = queries.shape[1]
        q = _soa(queries, QUERY_FIELDS, n)
        w = _soa(walk_in, SS_WALK_IN_FIELDS_TWOSTAGE if self.ctx.config.twostage else WALK_IN_FIELDS, n)
        out = np.zeros((WALK_OUT_FIELDS, n), np.float32)
        _check(_LIB.sms_ss_walk_batch(self.ctx.handle, caster, _ptr(q), _ptr(w), n, _ptr(out)))
        return out


class SpecularManifoldMultiScatter:
    """Batched SpecularManifoldMultiScatter (include/mitsuba/render/manifold_ms.h);
    the chain length is config.bounces."""

    def __init__(self, ctx: Context):
        self.ctx = ctx

    def specular_manifold_sampling(self, queries: np.ndarray, seed: int = 0, stream_offset: int = 0):
        n = queries.shape[1]
        q = _soa(queries, QUERY_FIELDS, n)
        value = np.zeros((3, n), np.float32)
        count = np.zeros(n, np.int32)
        walks = np.zeros(n, np.int32)
        r = _Result(_ptr(value), _ptr(count), _ptr(walks))
        _check(_LIB.sms_ms_connect_batch(self.ctx.handle, _ptr(q), n, seed, stream_offset, C.byref(r)))
        return value, count, walks

    def specular_manifold_sampling_device(self, queries_ptr: int, n: int, value_ptr: int, count_ptr: int,
                                          walks_ptr: int, seed: int = 0, stream_offset: int = 0):
        r = _Result(value_ptr, count_ptr, walks_ptr)
        _check(_LIB.sms_ms_connect_batch_device(self.ctx.handle, queries_ptr, n, seed, stream_offset,
                                                C.byref(r)))

    def sample_path(self, caster: int, queries: np.ndarray, walk_in: np.ndarray) -> np.ndarray:
        """First-path walks with explicit light point / start point; returns
        (9, n): ok, iterations, first vertex (3), last vertex (3), seed ok."""
        n = queries.shape[1]
        q = _soa(queries, QUERY_FIELDS, n)
        w = _soa(walk_in, WALK_IN_FIELDS, n)
        out = np.zeros((MS_WALK_OUT_FIELDS, n), np.float32)
        _check(_LIB.sms_ms_walk_batch(self.ctx.handle, caster, _ptr(q), _ptr(w), n, _ptr(out)))
        return out


class SpecularManifoldGlints:
    """Batched SpecularManifoldGlints / SpecularManifoldGlintsVectorized
    (include/mitsuba/render/manifold_glints.h): the SMS strategy over pixel
    footprints; value = sms_weight x ei.weight (MIS and sensor importance are
    the integrator's)."""

    def __init__(self, ctx: Context):
        self.ctx = ctx

    def specular_manifold_sampling(self, queries: np.ndarray, seed: int = 0, stream_offset: int = 0):
        n = queries.shape[1]
        q = _soa(queries, GLINT_QUERY_FIELDS, n)
        value = np.zeros((3, n), np.float32)
        count = np.zeros(n, np.int32)
        walks = np.zeros(n, np.int32)
        r = _Result(_ptr(value), _ptr(count), _ptr(walks))
        _check(_LIB.sms_glint_connect_batch(self.ctx.handle, _ptr(q), n, seed, stream_offset, C.byref(r)))
        return value, count, walks

    def specular_manifold_sampling_device(self, queries_ptr: int, n: int, value_ptr: int, count_ptr: int,
                                          walks_ptr: int, seed: int = 0, stream_offset: int = 0):
        r = _Result(value_ptr, count_ptr, walks_ptr)
        _check(_LIB.sms_glint_connect_batch_device(self.ctx.handle, queries_ptr, n, seed, stream_offset,
                                                   C.byref(r)))

    def sample_glint(self, queries: np.ndarray, walk_in: np.ndarray) -> np.ndarray:
        """walk_in (5, n): light point (3), footprint sample xi_start (2);
        returns (6, n): ok, iterations, uv_final (2), uv_init (2)."""
        n = queries.shape[1]
        q = _soa(queries, GLINT_QUERY_FIELDS, n)
        w = _soa(walk_in, GLINT_WALK_IN_FIELDS, n)
        out = np.zeros((GLINT_WALK_OUT_FIELDS, n), np.float32)
        _check(_LIB.sms_glint_walk_batch(self.ctx.handle, _ptr(q), _ptr(w), n, _ptr(out)))
        return out
