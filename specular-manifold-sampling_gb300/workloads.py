"""Synthetic SMS workloads with the shapes, sizes and seeds of the benchmark
configurations (the reference's paper scenes are partly missing and are not
used).  Every random draw comes from PCG32 streams so the GPU library, the
oracle and the tests see identical inputs.

  sphere_scene      glass sphere r=1 at (0,0,1.5), IOR 1.5, over the plane z=0,
                    point light (0,0,5) I=100; 64x64 query grid on [-2,2]^2;
                    biased SMS, 16 trials, 20 iterations, threshold 1e-5.
  slab_scene        two-bounce glass slab (IOR 1.5): top face z = 1.3 + h1 and
                    bottom face z = 1 + h2, with h1, h2 independent sums of 8
                    sinusoids (total amplitude <= 0.01) on 256x256 vertex grids
                    over [-1,1]^2; point light (0,0,5); queries uniform on
                    [-1,1]^2; biased SMS, 32 trials, 30 iterations, 2 bounces.
  glint_scene       normal-mapped conductor plane [-0.5,0.5]^2 at z=0 (uv in
                    [0,1]^2); FP16 slope map res^2 (8192^2 for the benchmark)
                    from a Gaussian random field with correlation length 4
                    texels and slope std 0.15 (seed 7); pinhole camera
                    (1024^2, 30 deg FOV) at 60 deg from the normal, point light
                    in the mirror direction; one query per pixel that sees the
                    plane, footprints from ray differentials; biased SMS, 64
                    seeds, 10 iterations.
  water_scene       z = 1 + sum of 32 sinusoids (a ~ U(0.002,0.02),
                    |k| ~ U(2,40), uniform direction and phase) tessellated to a
                    512x512 vertex grid over [-1,1]^2 (522,242 triangles), IOR
                    1.33; spherical area light r=0.1 at (0,0,10); queries
                    uniform on [-1,1]^2; unbiased SMS, trials capped at 256.

The receiver plane z=0 is not part of the ray-cast scene: every ray of the
single-scatter path starts on it or above it and ends above it, so no ray can
reach it past the ray epsilon.
"""
from __future__ import annotations

import math

import numpy as np

from . import (BSDF_CONDUCTOR, BSDF_DIELECTRIC, BSDF_DIFFUSE, EMITTER_CAUSTIC_MULTI, EMITTER_CAUSTIC_SINGLE,
               SHAPE_CAUSTIC_BOUNCER, SHAPE_CAUSTIC_RECEIVER, SHAPE_CAUSTIC_CASTER_MULTI, SHAPE_CAUSTIC_CASTER_SINGLE, SHAPE_GLINTY,
               QUERY_FIELDS, Bsdf, SceneDesc, SMSConfig)

_MUL = np.uint64(6364136223846793005)
_M64 = (1 << 64) - 1


class Pcg32:
    """Scalar PCG32 (O'Neill), same stream convention as the device code."""

    def __init__(self, initstate: int, initseq: int = 0):
        self.state = 0
        self.inc = ((initseq << 1) | 1) & _M64
        self.next_u32()
        self.state = (self.state + initstate) & _M64
        self.next_u32()

    def next_u32(self) -> int:
        old = self.state
        self.state = (old * 6364136223846793005 + self.inc) & _M64
        xs = (((old >> 18) ^ old) >> 27) & 0xFFFFFFFF
        rot = old >> 59
        return ((xs >> rot) | (xs << ((-rot) & 31))) & 0xFFFFFFFF

    def next_f32(self) -> float:
        bits = (self.next_u32() >> 9) | 0x3F800000
        return float(np.array([bits], np.uint32).view(np.float32)[0]) - 1.0


def pcg32_streams_f32(initstate: int, streams: np.ndarray, count: int) -> np.ndarray:
    """`count` float32 draws from each of many PCG32 streams, vectorized over
    streams.  Returns an array of shape (count, len(streams))."""
    with np.errstate(over="ignore"):
        inc = (np.asarray(streams, np.uint64) << np.uint64(1)) | np.uint64(1)
        state = np.zeros_like(inc)

        def step(st):
            old = st
            new = old * _MUL + inc
            xs = (((old >> np.uint64(18)) ^ old) >> np.uint64(27)).astype(np.uint32)
            rot = (old >> np.uint64(59)).astype(np.uint32)
            out = (xs >> rot) | (xs << ((np.uint32(32) - rot) & np.uint32(31)))
            return new, out

        state, _ = step(state)
        state = state + np.uint64(initstate)
        state, _ = step(state)
        res = np.empty((count, len(inc)), np.float32)
        for k in range(count):
            state, u = step(state)
            res[k] = ((u >> np.uint32(9)) | np.uint32(0x3F800000)).view(np.float32) - np.float32(1.0)
    return res


def plane_queries(xy: np.ndarray, albedo: float = 0.5) -> np.ndarray:
    """SoA queries (16, n) for shading points (x, y, 0) on the receiver z = 0."""
    n = xy.shape[0]
    q = np.zeros((QUERY_FIELDS, n), np.float32)
    q[0], q[1] = xy[:, 0], xy[:, 1]
    q[5] = 1.0          # n = (0, 0, 1)
    q[6] = 1.0          # dp_du = (1, 0, 0)
    q[10] = 1.0         # dp_dv = (0, 1, 0)
    q[12:15] = albedo
    q[15] = 1.0         # camera above the receiver
    return q


# ----------------------------------------------------------------- sphere
def sphere_scene(conductor: bool = False) -> SceneDesc:
    d = SceneDesc()
    b = Bsdf(BSDF_CONDUCTOR, 0.2, 3.0) if conductor else Bsdf(BSDF_DIELECTRIC, 1.5)
    d.add_sphere((0.0, 0.0, 1.5), 1.0, b, SHAPE_CAUSTIC_CASTER_SINGLE)
    d.add_point_emitter((0.0, 0.0, 5.0), (100.0, 100.0, 100.0), EMITTER_CAUSTIC_SINGLE)
    return d


def sphere_queries(res: int = 64, extent: float = 2.0) -> np.ndarray:
    c = (np.arange(res, dtype=np.float64) + 0.5) / res * (2 * extent) - extent
    yy, xx = np.meshgrid(c, c, indexing="ij")
    xy = np.stack([xx.ravel(), yy.ravel()], axis=1).astype(np.float32)
    return plane_queries(xy)


def sphere_config() -> SMSConfig:
    return SMSConfig(biased=True, max_trials=16, max_iterations=20, solver_threshold=1e-5)


# ------------------------------------------------------------------ water
def water_params(n_waves: int = 32, seed: int = 2):
    r = Pcg32(seed, 0)
    waves = []
    for _ in range(n_waves):
        a = 0.002 + (0.02 - 0.002) * r.next_f32()
        km = 2.0 + (40.0 - 2.0) * r.next_f32()
        ang = 2.0 * math.pi * r.next_f32()
        ph = 2.0 * math.pi * r.next_f32()
        waves.append((a, km * math.cos(ang), km * math.sin(ang), ph))
    return waves


def heightfield_mesh(res: int, extent: float, base: float, waves, flip_normals: bool = False):
    """Vertex grid res x res over [-extent, extent]^2 with z = base + waves.
    Returns (P, N, UV, F) with analytic vertex normals and grid uvs."""
    t = np.linspace(-extent, extent, res, dtype=np.float64)
    yy, xx = np.meshgrid(t, t, indexing="ij")
    z = np.full_like(xx, base)
    zx = np.zeros_like(xx)
    zy = np.zeros_like(xx)
    for a, kx, ky, ph in waves:
        arg = kx * xx + ky * yy + ph
        z += a * np.sin(arg)
        c = a * np.cos(arg)
        zx += c * kx
        zy += c * ky
    P = np.stack([xx, yy, z], axis=-1).reshape(-1, 3).astype(np.float32)
    Nn = np.stack([-zx, -zy, np.ones_like(z)], axis=-1)
    Nn /= np.linalg.norm(Nn, axis=-1, keepdims=True)
    if flip_normals:
        Nn = -Nn
    N = Nn.reshape(-1, 3).astype(np.float32)
    u = (xx - xx.min()) / (xx.max() - xx.min())
    v = (yy - yy.min()) / (yy.max() - yy.min())
    UV = np.stack([u, v], axis=-1).reshape(-1, 2).astype(np.float32)
    i, j = np.meshgrid(np.arange(res - 1), np.arange(res - 1), indexing="ij")
    v00 = (i * res + j).ravel()
    v10 = v00 + 1
    v01 = v00 + res
    v11 = v01 + 1
    if flip_normals:
        F = np.concatenate([np.stack([v00, v11, v10], 1), np.stack([v00, v01, v11], 1)])
    else:
        F = np.concatenate([np.stack([v00, v10, v11], 1), np.stack([v00, v11, v01], 1)])
    return P, N, UV, F.astype(np.uint32)


def water_scene(res: int = 512, light_radiance: float = 3000.0) -> SceneDesc:
    d = SceneDesc()
    P, N, UV, F = heightfield_mesh(res, 1.0, 1.0, water_params())
    d.add_mesh(P, F, Bsdf(BSDF_DIELECTRIC, 1.33), SHAPE_CAUSTIC_CASTER_SINGLE, N=N, UV=UV)
    light = d.add_sphere((0.0, 0.0, 10.0), 0.1, Bsdf(BSDF_DIFFUSE, 1.0, 0.0, (0.0, 0.0, 0.0)), 0)
    d.add_area_emitter(light, (light_radiance,) * 3, EMITTER_CAUSTIC_SINGLE)
    return d


def water_queries(n: int, seed: int = 3, first: int = 0) -> np.ndarray:
    u = pcg32_streams_f32(seed, np.arange(first, first + n, dtype=np.uint64), 2)
    xy = np.stack([2.0 * u[0] - 1.0, 2.0 * u[1] - 1.0], axis=1).astype(np.float32)
    return plane_queries(xy)


def water_config() -> SMSConfig:
    return SMSConfig(biased=False, max_trials=256, max_iterations=20)


# ------------------------------------------------------------------- pool
def pool_scene(res: int = 128, light_radius: float = 0.5, light_z: float = 4.0, radiance: float = 40.0,
               point_light: bool = False, floor_albedo: float = 0.5, wave_scale: float = 1.0,
               floor_bsdf=None) -> SceneDesc:
    """Rendering scene: the water heightfield of water_scene with its wave
    amplitudes scaled by wave_scale (0: flat; res x res grid over [-1, 1]^2
    around z = 1, dielectric 1.33, caustic_caster_single) over a
    diffuse floor z = 0 on [-2, 2]^2 (caustic_receiver), lit by a sphere area
    light (or a point light of intensity radiance * light_radius^2 * pi at the
    same place), flagged caustic_emitter_single.  floor_bsdf replaces the
    floor's diffuse BSDF."""
    d = SceneDesc()
    fl = np.array([[-2, -2, 0], [2, -2, 0], [2, 2, 0], [-2, 2, 0]], np.float32)
    fuv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    d.add_mesh(fl, np.array([[0, 1, 2], [0, 2, 3]], np.uint32),
               floor_bsdf if floor_bsdf is not None else Bsdf(BSDF_DIFFUSE, 1.0, 0.0, (floor_albedo,) * 3),
               SHAPE_CAUSTIC_RECEIVER, UV=fuv)
    waves = [(a * wave_scale, kx, ky, ph) for (a, kx, ky, ph) in water_params()] if wave_scale > 0 else []
    P, N, UV, F = heightfield_mesh(res, 1.0, 1.0, waves)
    d.add_mesh(P, F, Bsdf(BSDF_DIELECTRIC, 1.33), SHAPE_CAUSTIC_CASTER_SINGLE, N=N, UV=UV)
    if point_light:
        I = radiance * math.pi * light_radius * light_radius
        d.add_point_emitter((0.0, 0.0, light_z), (I, I, I), EMITTER_CAUSTIC_SINGLE)
    else:
        light = d.add_sphere((0.0, 0.0, light_z), light_radius, Bsdf(BSDF_DIFFUSE, 1.0, 0.0, (0.0, 0.0, 0.0)), 0)
        d.add_area_emitter(light, (radiance,) * 3, EMITTER_CAUSTIC_SINGLE)
    return d


def pool_camera(width: int = 64, height: int = 64, fov: float = 40.0):
    from . import Camera
    return Camera.look_at((0.0, -3.2, 3.6), (0.0, 0.0, 0.4), (0.0, 0.0, 1.0), fov, width, height)


def teaser_scene(sphere_res: int = 24, map_res: int = 256) -> SceneDesc:
    """A small stand-in for the combined integrator's scene (path_sms_teaser):
    a diffuse floor z = 0 on [-2, 2]^2 (caustic_receiver), a mirror sphere r =
    0.35 at (-0.7, 0, 0.8) (caustic_caster_single: a reflection caustic), a
    glass sphere r = 0.4 at (0.6, 0, 0.9) tessellated to a mesh
    (caustic_caster_multi: the two refractions of the multi-scatter chain), a
    normal-mapped conductor tile z = 0.01 on [-1.5, 1.5] x [-1.9, -1.1] (glinty,
    FP16 slope map map_res^2), and a point light at (0, 0.5, 4) flagged for both
    caustic estimators."""
    d = SceneDesc()
    fl = np.array([[-2, -2, 0], [2, -2, 0], [2, 2, 0], [-2, 2, 0]], np.float32)
    fuv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    quad = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
    d.add_mesh(fl, quad, Bsdf(BSDF_DIFFUSE, 1.0, 0.0, (0.5, 0.5, 0.5)), SHAPE_CAUSTIC_RECEIVER, UV=fuv)
    d.add_sphere((-0.7, 0.0, 0.8), 0.35, Bsdf(BSDF_CONDUCTOR, 0.2, 3.0), SHAPE_CAUSTIC_CASTER_SINGLE)
    # glass sphere as a UV-sphere mesh with analytic normals
    nt, nph = sphere_res, 2 * sphere_res
    th = np.linspace(0.0, math.pi, nt + 1)
    ph = np.linspace(0.0, 2.0 * math.pi, nph + 1)
    T, PH = np.meshgrid(th, ph, indexing="ij")
    nrm = np.stack([np.sin(T) * np.cos(PH), np.sin(T) * np.sin(PH), np.cos(T)], axis=-1).reshape(-1, 3)
    P = (np.array([0.6, 0.0, 0.9]) + 0.4 * nrm).astype(np.float32)
    UV = np.stack([PH / (2.0 * math.pi), T / math.pi], axis=-1).reshape(-1, 2).astype(np.float32)
    F = []
    for i in range(nt):
        for j in range(nph):
            a0, a1, b0, b1 = i * (nph + 1) + j, i * (nph + 1) + j + 1, (i + 1) * (nph + 1) + j, (i + 1) * (nph + 1) + j + 1
            if i > 0:
                F.append((a0, b0, a1))
            if i < nt - 1:
                F.append((a1, b0, b1))
    d.add_mesh(P, np.array(F, np.uint32), Bsdf(BSDF_DIELECTRIC, 1.5), SHAPE_CAUSTIC_CASTER_MULTI,
               N=nrm.astype(np.float32), UV=UV)
    tile = np.array([[-1.5, -1.9, 0.01], [1.5, -1.9, 0.01], [1.5, -1.1, 0.01], [-1.5, -1.1, 0.01]], np.float32)
    sid = d.add_mesh(tile, quad, Bsdf(BSDF_CONDUCTOR, 1.0, 6.0), SHAPE_GLINTY, UV=fuv)
    d.normalmap = (sid, glint_slopes(map_res), 1.0)
    d.add_point_emitter((0.0, 0.5, 4.0), (60.0, 60.0, 60.0), EMITTER_CAUSTIC_SINGLE | EMITTER_CAUSTIC_MULTI)
    return d


def teaser_camera(width: int = 32, height: int = 32, fov: float = 45.0):
    from . import Camera
    return Camera.look_at((0.0, -3.4, 2.6), (0.0, -0.3, 0.3), (0.0, 0.0, 1.0), fov, width, height)


# ------------------------------------------------------------------- slab
def slab_waves(seed: int, n_waves: int = 8):
    r = Pcg32(seed, 0)
    waves = []
    for _ in range(n_waves):
        a = 0.0005 + (0.00125 - 0.0005) * r.next_f32()
        km = 2.0 + (20.0 - 2.0) * r.next_f32()
        ang = 2.0 * math.pi * r.next_f32()
        ph = 2.0 * math.pi * r.next_f32()
        waves.append((a, km * math.cos(ang), km * math.sin(ang), ph))
    return waves


def slab_scene(res: int = 256, alpha: float = 0.0) -> SceneDesc:
    """Glass slab: top face caustic_caster_multi (normals up), bottom face
    caustic_bouncer (normals down, i.e. outward), IOR 1.5; point light.
    alpha > 0: both faces rough (Beckmann roughdielectric)."""
    d = SceneDesc()
    glass = Bsdf(BSDF_DIELECTRIC, 1.5, alpha=alpha)
    P, N, UV, F = heightfield_mesh(res, 1.0, 1.3, slab_waves(4))
    d.add_mesh(P, F, glass, SHAPE_CAUSTIC_CASTER_MULTI, N=N, UV=UV)
    P, N, UV, F = heightfield_mesh(res, 1.0, 1.0, slab_waves(5), flip_normals=True)
    d.add_mesh(P, F, glass, SHAPE_CAUSTIC_BOUNCER, N=N, UV=UV)
    d.add_point_emitter((0.0, 0.0, 5.0), (100.0, 100.0, 100.0), EMITTER_CAUSTIC_MULTI)
    return d


def slab_queries(n: int, seed: int = 6, first: int = 0) -> np.ndarray:
    u = pcg32_streams_f32(seed, np.arange(first, first + n, dtype=np.uint64), 2)
    xy = np.stack([2.0 * u[0] - 1.0, 2.0 * u[1] - 1.0], axis=1).astype(np.float32)
    return plane_queries(xy)


def slab_config() -> SMSConfig:
    return SMSConfig(biased=True, max_trials=32, max_iterations=30, bounces=2)


# -------------------------------------------------- normal-mapped caster
def nm_plane_slopes(res: int = 256, amp: float = 0.15, freq: int = 1) -> np.ndarray:
    """(res, res, 2) float16 slopes of a smooth periodic bump pattern (freq
    periods of the base pattern across the map)."""
    t = (np.arange(res) + 0.5) / res
    vv, uu = np.meshgrid(t, t, indexing="ij")
    sx = amp * np.sin(2 * np.pi * freq * (2 * uu + vv))
    sy = (amp / 1.5) * np.cos(2 * np.pi * freq * (uu - 2 * vv))
    return np.stack([sx, sy], axis=-1).astype(np.float16)


def nm_plane_scene(conductor: bool = False, res: int = 256, alpha: float = 0.0, amp: float = 0.15,
                   freq: int = 1) -> SceneDesc:
    """The quad z = 1 over [-1, 1]^2 carrying a slope map (the normalmap BSDF
    around a dielectric or conductor), flagged as a single-scatter caster.  The
    point light sits above it (refraction down to the receiver z = 0) or, for
    the conductor, below the receiver (reflection down to it)."""
    d = SceneDesc()
    P = np.array([[-1, -1, 1.0], [1, -1, 1.0], [1, 1, 1.0], [-1, 1, 1.0]], np.float32)
    UV = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    F = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
    b = Bsdf(BSDF_CONDUCTOR, 0.2, 3.0, alpha=alpha) if conductor else Bsdf(BSDF_DIELECTRIC, 1.5, alpha=alpha)
    sid = d.add_mesh(P, F, b, SHAPE_CAUSTIC_CASTER_SINGLE, UV=UV)
    d.normalmap = (sid, nm_plane_slopes(res, amp, freq), 1.0)
    d.add_point_emitter((0.3, -0.2, -3.0) if conductor else (0.3, -0.2, 4.0), (100.0,) * 3,
                        EMITTER_CAUSTIC_SINGLE)
    return d


def nm_plane_queries(n: int, seed: int = 9, extent: float = 0.8) -> np.ndarray:
    """Receiver points (x, y, 0) uniform in [-extent, extent]^2."""
    u = pcg32_streams_f32(seed, np.arange(n, dtype=np.uint64), 2)
    return plane_queries(((u.T * 2.0 - 1.0) * extent).astype(np.float32))


# ----------------------------------------------------------------- glints
GLINT_QUERY_FIELDS = 21


def glint_slopes(res: int, seed: int = 7, corr: float = 4.0, std: float = 0.15) -> np.ndarray:
    """(res, res, 2) float16 slopes (sx, sy): white noise smoothed by a Gaussian
    of `corr` texels (wrapping, like the tiled lookup), scaled to std `std`."""
    from scipy.ndimage import gaussian_filter
    rng = np.random.default_rng(seed)
    out = np.empty((res, res, 2), np.float16)
    for c in range(2):
        w = rng.standard_normal((res, res), dtype=np.float32)
        w = gaussian_filter(w, sigma=corr, mode="wrap", truncate=3.0)
        w *= np.float32(std / float(w.std()))
        out[..., c] = w.astype(np.float16)
    return out


GLINT_CAM_DIST = 2.0
GLINT_ELEV = math.radians(60.0)


def glint_camera():
    cam = np.array([0.0, -math.sin(GLINT_ELEV), math.cos(GLINT_ELEV)]) * GLINT_CAM_DIST
    light = np.array([0.0, math.sin(GLINT_ELEV), math.cos(GLINT_ELEV)]) * GLINT_CAM_DIST
    return cam, light


def glint_scene(map_res: int = 8192, slopes: np.ndarray | None = None, intensity: float = 50.0,
                conductor=(1.0, 6.0), alpha: float = 0.0) -> SceneDesc:
    """alpha > 0: a rough (Beckmann) conductor under the slope map."""
    d = SceneDesc()
    P = np.array([[-0.5, -0.5, 0.0], [0.5, -0.5, 0.0], [0.5, 0.5, 0.0], [-0.5, 0.5, 0.0]], np.float32)
    UV = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    F = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
    sid = d.add_mesh(P, F, Bsdf(BSDF_CONDUCTOR, conductor[0], conductor[1], alpha=alpha), SHAPE_GLINTY, UV=UV)
    d.normalmap = (sid, glint_slopes(map_res) if slopes is None else slopes, 1.0)
    _, light = glint_camera()
    d.add_point_emitter(tuple(light), (intensity,) * 3, EMITTER_CAUSTIC_SINGLE)
    return d


def glint_queries(width: int = 1024, fov_deg: float = 30.0, diff_scale: float = 1.0) -> np.ndarray:
    """One query per pixel whose primary ray hits the plane: p, n, dp_du, dp_dv,
    uv, duv_dx, duv_dy (interaction.h:216-248 compute_partials, scaled by
    diff_scale) and the sensor position.  Shape (21, n)."""
    cam, _ = glint_camera()
    fwd = -cam / np.linalg.norm(cam)
    up = np.array([0.0, 0.0, 1.0])
    right = np.cross(fwd, up)
    right /= np.linalg.norm(right)
    upv = np.cross(right, fwd)
    tan_h = math.tan(math.radians(fov_deg) / 2)
    j, i = np.meshgrid(np.arange(width), np.arange(width), indexing="ij")

    def dirs(px, py):
        sx = (2.0 * (px + 0.5) / width - 1.0) * tan_h
        sy = (1.0 - 2.0 * (py + 0.5) / width) * tan_h
        d = fwd[None, None, :] + sx[..., None] * right[None, None, :] + sy[..., None] * upv[None, None, :]
        return d / np.linalg.norm(d, axis=-1, keepdims=True)

    d0 = dirs(i.astype(np.float64), j.astype(np.float64))
    dx = dirs(i + 1.0, j.astype(np.float64))
    dy = dirs(i.astype(np.float64), j + 1.0)
    t = -cam[2] / d0[..., 2]
    p = cam[None, None, :] + t[..., None] * d0
    hit = (t > 0) & (np.abs(p[..., 0]) <= 0.5) & (np.abs(p[..., 1]) <= 0.5)
    p, d0, dx, dy = p[hit], d0[hit], dx[hit], dy[hit]
    n = np.array([0.0, 0.0, 1.0])

    def offset_point(dd):
        tt = (0.0 - cam[2]) / dd[:, 2]   # plane z = 0 (n . p = 0)
        return cam[None, :] + tt[:, None] * dd

    dp_dx = (offset_point(dx) - p) * diff_scale
    dp_dy = (offset_point(dy) - p) * diff_scale
    m = p.shape[0]
    q = np.zeros((GLINT_QUERY_FIELDS, m), np.float32)
    q[0:3] = p.T
    q[5] = 1.0
    q[6] = 1.0            # dp_du = (1, 0, 0): uv = (x + 0.5, y + 0.5)
    q[10] = 1.0           # dp_dv = (0, 1, 0)
    q[12] = p[:, 0] + 0.5
    q[13] = p[:, 1] + 0.5
    q[14], q[15] = dp_dx[:, 0], dp_dx[:, 1]
    q[16], q[17] = dp_dy[:, 0], dp_dy[:, 1]
    q[18:21] = cam[:, None]
    return q


def lean_fallback_scene(map_res: int = 256, fallback=(0.05, 0.2, 3.0), radiance: float = 30.0) -> SceneDesc:
    """The normal map's LEAN fallback BSDF at work: the normal-mapped conductor
    plane of glint_scene (z = 0, [-0.5, 0.5]^2, map glint_slopes) with the
    fallback (alpha, eta, k), a diffuse wall facing it (y = -0.6, normal +y),
    and a sphere area light above.  Camera rays (lean_fallback_camera) hit the
    wall first; paths that bounce from the wall to the plane meet it without
    uv partials, where the plane reflects like its LEAN distribution."""
    d = glint_scene(map_res=map_res, conductor=(0.2, 3.0))
    d.point_emitters.clear()
    d.lean_fallback = tuple(float(x) for x in fallback)
    W = np.array([[-0.6, -0.6, 0.0], [0.6, -0.6, 0.0], [0.6, -0.6, 1.0], [-0.6, -0.6, 1.0]], np.float32)
    F = np.array([[0, 2, 1], [0, 3, 2]], np.uint32)
    UV = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    d.add_mesh(W, F, Bsdf(BSDF_DIFFUSE, 1.0, 0.0, (0.6, 0.6, 0.6)), SHAPE_CAUSTIC_RECEIVER, UV=UV)
    light = d.add_sphere((0.0, 0.6, 1.4), 0.25, Bsdf(BSDF_DIFFUSE, 1.0, 0.0, (0.0, 0.0, 0.0)), 0)
    d.add_area_emitter(light, (radiance,) * 3, EMITTER_CAUSTIC_SINGLE)
    return d


def lean_fallback_camera(width: int = 32, height: int = 32):
    """Looks at the wall of lean_fallback_scene from in front of the plane."""
    from . import Camera
    return Camera.look_at((0.0, 1.2, 0.6), (0.0, -0.6, 0.4), (0.0, 0.0, 1.0), 45.0, width, height)


def plane_light_scene(below: bool, twosided: bool, width: int = 16, height: int = 16, bsdf=None):
    """(SceneDesc, Camera): a plane z = 0 (normal +z, twosided or not; diffuse
    unless a Bsdf is given) lit by a sphere light outside the camera's view,
    light and camera both above the plane or both below it (looking at its
    back)."""
    from . import Camera
    d = SceneDesc()
    fl = np.array([[-3, -3, 0], [3, -3, 0], [3, 3, 0], [-3, 3, 0]], np.float32)
    d.add_mesh(fl, np.array([[0, 1, 2], [0, 2, 3]], np.uint32),
               bsdf if bsdf is not None else Bsdf(BSDF_DIFFUSE, 1.0, 0.0, (0.6,) * 3, twosided=twosided))
    z = -2.0 if below else 2.0
    light = d.add_sphere((1.5, 0.0, z), 0.3, Bsdf(BSDF_DIFFUSE, 1.0, 0.0, (0.0,) * 3), 0)
    d.add_area_emitter(light, (30.0,) * 3, 0)
    cam = Camera.look_at((0.0, 0.0, -3.0 if below else 3.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 40.0, width, height)
    return d, cam


def glint_render_camera(width: int = 64, height: int = 64, fov: float = 30.0):
    """The glint benchmark's camera (60 degrees from the normal, looking at the
    plane's centre) as a Camera for the path tracer."""
    from . import Camera
    cam, _ = glint_camera()
    return Camera.look_at(tuple(cam), (0.0, 0.0, 0.0), (0.0, 0.0, 1.0), fov, width, height)


def glint_config() -> SMSConfig:
    return SMSConfig(biased=True, max_trials=64, max_iterations=10, glints_vectorized=True)
