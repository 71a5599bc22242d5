"""The oracle pinned against known answers (no GPU).

* PCG32 against O'Neill's published demo stream (the reference's sampler RNG,
  include/mitsuba/core/random.h:50-52);
* Fresnel against the values the reference's own test asserts
  (src/librender/tests/test_fresnel.py:7-39) and the conductor/dielectric
  agreement of test03 there;
* the uniform-sphere warp (include/mitsuba/core/warp.h:262-267);
* converged walks against specular solutions derived independently in FP64
  (tests/golden/sphere_analytic.json), tolerance 1e-5 at scene scale 1;
* bit-exact regression of small estimator runs (tests/golden/oracle_small.npz).
"""
import ctypes as C
import json
import math
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def kat():
    return json.loads((GOLDEN / "kat.json").read_text())


def test_pcg32_reference_stream(oracle, workloads, kat):
    lib = oracle.load()
    out = np.zeros(6, np.uint32)
    lib.oracle_pcg32(42, 54, 6, out.ctypes.data)
    assert out.tolist() == kat["pcg32_42_54_u32"]
    r = workloads.Pcg32(42, 54)
    assert [r.next_u32() for _ in range(6)] == kat["pcg32_42_54_u32"]


def test_pcg32_float_streams_agree(oracle, workloads):
    lib = oracle.load()
    f = np.zeros(5, np.float32)
    lib.oracle_pcg32_f32(7, 3, 5, f.ctypes.data)
    v = workloads.pcg32_streams_f32(7, np.array([3], np.uint64), 5).ravel()
    assert np.array_equal(f, v)
    r = workloads.Pcg32(7, 3)
    assert np.array_equal(np.float32([r.next_f32() for _ in range(5)]), f)
    assert np.all((f >= 0) & (f < 1))


def test_fresnel_reference_values(oracle, kat):
    lib = oracle.load()
    ct = C.c_float()
    for cos_i, eta, F_ref, ct_ref in kat["fresnel"]:
        F = lib.oracle_fresnel(cos_i, eta, C.byref(ct))
        assert F == pytest.approx(F_ref, abs=1e-5), (cos_i, eta)
        assert ct.value == pytest.approx(ct_ref, abs=1e-5), (cos_i, eta)


def test_fresnel_conductor_matches_dielectric_for_real_ior(oracle):
    # test_fresnel.py:60-72 (test03_fresnel_conductor)
    lib = oracle.load()
    for th in np.linspace(0, math.pi / 2, 20):
        c = math.cos(th)
        for eta in (1.5, 1 / 1.5):
            a = lib.oracle_fresnel(c, eta, None)
            b = lib.oracle_fresnel_conductor(c, eta, 0.0)
            assert a == pytest.approx(b, abs=1e-5)


def test_snell(oracle):
    # test_fresnel.py:75-83 (test04_snell)
    lib = oracle.load()
    ct = C.c_float()
    for th in np.linspace(0, math.pi / 2, 20):
        lib.oracle_fresnel(math.cos(th), 1.5, C.byref(ct))
        assert math.sin(th) - 1.5 * math.sin(math.acos(ct.value)) == pytest.approx(0, abs=1e-5)


def test_uniform_sphere(oracle, kat):
    lib = oracle.load()
    out = (C.c_float * 3)()
    for u, v, x, y, z in kat["uniform_sphere"]:
        lib.oracle_uniform_sphere(u, v, out)
        assert list(out) == pytest.approx([x, y, z], abs=1e-6)


@pytest.mark.parametrize("mode", ["reflect", "refract"])
def test_walks_converge_to_analytic_solutions(sms, workloads, oracle, mode):
    W = workloads
    cases = [c for c in json.loads((GOLDEN / "sphere_analytic.json").read_text()) if c["mode"] == mode]
    assert cases
    desc = W.sphere_scene(conductor=(mode == "reflect"))
    o = oracle.OracleScene(desc)
    xy = np.array([[c["x"][0], 0.0] for c in cases for _ in (1, -1)], np.float32)
    q = W.plane_queries(xy)
    n = q.shape[1]
    w = np.zeros((8, n), np.float32)
    w[2] = 5.0
    for i, c in enumerate(cases):
        for j, s in enumerate((1, -1)):
            th = c["theta"] + 0.03 * s
            w[3:6, 2 * i + j] = [math.sin(th), 0.0, 1.5 - math.cos(th)]
    out = o.walk_batch(sms.SMSConfig(), 0, q, w)
    sol = np.array([c["solution"] for c in cases for _ in (1, -1)]).T
    ok = out[0] > 0.5
    assert ok.mean() >= 0.9
    err = np.linalg.norm(out[2:5, ok] - sol[:, ok], axis=0)
    assert err.max() < 1e-5


def test_oracle_regression(sms, workloads, oracle):
    W = workloads
    ref = np.load(GOLDEN / "oracle_small.npz")
    for cond in (False, True):
        tag = "cond" if cond else "glass"
        v, c, w, st = oracle.OracleScene(W.sphere_scene(conductor=cond)).connect_batch(
            W.sphere_config(), W.sphere_queries(16), seed=1, nthreads=2)
        assert np.array_equal(c, ref[f"sphere_{tag}_count"])
        np.testing.assert_allclose(v, ref[f"sphere_{tag}_value"], rtol=1e-6, atol=1e-9)
    v, c, w, st = oracle.OracleScene(W.water_scene(res=64)).connect_batch(
        W.water_config(), W.water_queries(256), seed=5, nthreads=2)
    assert np.array_equal(c, ref["water64_count"])
    assert np.array_equal(w, ref["water64_walks"])
    np.testing.assert_allclose(v, ref["water64_value"], rtol=1e-6, atol=1e-9)


def test_nan_walks_are_misses(sms, workloads, oracle):
    """A start point at the shading point gives a NaN direction: the walk fails."""
    W = workloads
    o = oracle.OracleScene(W.sphere_scene())
    q = W.sphere_queries(1)
    w = np.zeros((8, 1), np.float32)
    w[2] = 5.0
    w[3:6, 0] = q[0:3, 0]
    w[3:6, 0][2] = 1e-30  # non-zero so it counts as an explicit start, ~ the shading point
    out = o.walk_batch(sms.SMSConfig(), 0, q, w)
    assert out[0, 0] == 0.0


def _flat_slab(sms, W):
    """Two parallel glass faces z = 1 (bouncer, normals down) and z = 1.3
    (caster_multi, normals up), IOR 1.5, point light (0.3, -0.2, 5)."""
    d = sms.SceneDesc()
    glass = sms.Bsdf(sms.BSDF_DIELECTRIC, 1.5)
    P, N, UV, F = W.heightfield_mesh(8, 2.0, 1.3, [])
    d.add_mesh(P, F, glass, sms.SHAPE_CAUSTIC_CASTER_MULTI, N=N, UV=UV)
    P, N, UV, F = W.heightfield_mesh(8, 2.0, 1.0, [], flip_normals=True)
    d.add_mesh(P, F, glass, sms.SHAPE_CAUSTIC_BOUNCER, N=N, UV=UV)
    d.add_point_emitter((0.3, -0.2, 5.0), (100.0, 100.0, 100.0), sms.EMITTER_CAUSTIC_MULTI)
    return d


def _slab_solution(x, light, h1=1.0, t=0.3, eta=1.5):
    """Entry and exit points of the double refraction through a flat slab,
    from a bisection on the incidence angle (FP64, independent of the oracle)."""
    dxy = np.array(light[:2]) - np.array(x[:2])
    D = np.linalg.norm(dxy)
    h2 = light[2] - (h1 + t)
    f = lambda th: h1 * math.tan(th) + t * math.tan(math.asin(math.sin(th) / eta)) + h2 * math.tan(th) - D
    a, b = 0.0, math.pi / 2 - 1e-9
    for _ in range(200):
        m = 0.5 * (a + b)
        a, b = (m, b) if f(m) < 0 else (a, m)
    th = 0.5 * (a + b)
    u = dxy / D
    p1 = np.array([*(np.array(x[:2]) + h1 * math.tan(th) * u), h1])
    th_t = math.asin(math.sin(th) / eta)
    p2 = np.array([*(p1[:2] + t * math.tan(th_t) * u), h1 + t])
    return p1, p2


def test_ms_walks_converge_to_flat_slab_solution(sms, workloads, oracle):
    W = workloads
    o = oracle.OracleScene(_flat_slab(sms, W))
    xs = np.array([[0.0, 0.0], [0.5, 0.2], [-0.4, 0.6], [1.0, -1.0]], np.float32)
    q = W.plane_queries(xs)
    light = (0.3, -0.2, 5.0)
    w = np.zeros((8, len(xs)), np.float32)
    w[0], w[1], w[2] = light
    for i, x in enumerate(xs):
        p1, p2 = _slab_solution((x[0], x[1], 0.0), light)
        w[3:6, i] = p2 + np.array([0.05, -0.03, 0.0])   # start near the exit point
    out = o.ms_walk_batch(sms.SMSConfig(bounces=2, max_iterations=30), 0, q, w)
    assert np.all(out[0] == 1) and np.all(out[8] == 1)
    for i, x in enumerate(xs):
        p1, p2 = _slab_solution((x[0], x[1], 0.0), light)
        assert np.linalg.norm(out[2:5, i] - p1) < 1e-5
        assert np.linalg.norm(out[5:8, i] - p2) < 1e-5


def test_block_tridiagonal_matches_dense_solve():
    """The block Thomas recursion of manifold_ms.cpp:1192-1232, written out in
    FP64, equals a dense solve of the same 2k x 2k system."""
    rng = np.random.default_rng(4)
    for k in (1, 2, 3, 4):
        P = [rng.normal(size=(2, 2)) for _ in range(k)]
        Cu = [rng.normal(size=(2, 2)) + 3 * np.eye(2) for _ in range(k)]
        N = [rng.normal(size=(2, 2)) for _ in range(k)]
        C = [rng.normal(size=2) for _ in range(k)]
        A = np.zeros((2 * k, 2 * k))
        for i in range(k):
            A[2 * i:2 * i + 2, 2 * i:2 * i + 2] = Cu[i]
            if i > 0:
                A[2 * i:2 * i + 2, 2 * i - 2:2 * i] = P[i]
            if i < k - 1:
                A[2 * i:2 * i + 2, 2 * i + 2:2 * i + 4] = N[i]
        ref = np.linalg.solve(A, np.concatenate(C))
        tmp, il, dx = [None] * k, [None] * k, [None] * k
        tmp[0] = P[0]
        il[0] = np.linalg.inv(Cu[0])
        for i in range(1, k):
            tmp[i] = P[i] @ il[i - 1]
            il[i] = np.linalg.inv(Cu[i] - tmp[i] @ N[i - 1])
        dx[0] = C[0]
        for i in range(1, k):
            dx[i] = C[i] - tmp[i] @ dx[i - 1]
        dx[k - 1] = il[k - 1] @ dx[k - 1]
        for i in range(k - 2, -1, -1):
            dx[i] = il[i] @ (dx[i] - N[i] @ dx[i + 1])
        assert np.allclose(np.concatenate(dx), ref, atol=1e-10)


def test_slope_derivative_matches_finite_differences(sms, workloads, oracle):
    """NormalmapBSDF::slope_derivative (src/bsdfs/normalmap.cpp:318-336) is the
    analytic derivative of the bilinear slope lookup: compare with central
    differences inside a texel."""
    W = workloads
    d = W.glint_scene(slopes=W.glint_slopes(64))
    o = oracle.OracleScene(d)
    rng = np.random.default_rng(3)
    h = 1e-4
    for u, v in rng.uniform(0.05, 0.95, size=(20, 2)):
        a = o.slope(u, v)
        pu, mu = o.slope(u + h, v), o.slope(u - h, v)
        pv, mv = o.slope(u, v + h), o.slope(u, v - h)
        fd_u = (pu[:2] - mu[:2]) / (2 * h)
        fd_v = (pv[:2] - mv[:2]) / (2 * h)
        # the bilinear patch is smooth inside a texel; skip samples straddling an edge
        if np.abs(pu[2:4] - mu[2:4]).max() > 1e-3 * max(1.0, np.abs(a[2:4]).max()):
            continue
        np.testing.assert_allclose(a[2:4], fd_u, rtol=2e-2, atol=2e-2)
        np.testing.assert_allclose(a[4:6], fd_v, rtol=2e-2, atol=2e-2)


def test_glint_walks_reach_target_slope(sms, workloads, oracle):
    """Converged glint walks end at a uv whose slope equals the half-vector
    slope (manifold_glints.cpp:236-247) and inside the footprint."""
    W = workloads
    d = W.glint_scene(slopes=W.glint_slopes(256))
    o = oracle.OracleScene(d)
    q = W.glint_queries(64)
    n = q.shape[1]
    _, light = W.glint_camera()
    u = W.pcg32_streams_f32(5, np.arange(n, dtype=np.uint64), 2)
    w = np.zeros((5, n), np.float32)
    w[0:3] = np.asarray(light, np.float32)[:, None]
    w[3], w[4] = u[0], u[1]
    cfg = W.glint_config()
    out = o.glint_walk_batch(cfg, q, w)
    ok = out[0] > 0.5
    assert ok.sum() > 10
    for i in np.nonzero(ok)[0][:50]:
        p, sensor = q[0:3, i], q[18:21, i]
        wi = (sensor - p) / np.linalg.norm(sensor - p)
        wo = (np.asarray(light) - p) / np.linalg.norm(np.asarray(light) - p)
        h = (wi + wo) / np.linalg.norm(wi + wo)
        target = -h[:2] / h[2]
        s = o.slope(out[2, i], out[3, i])[:2]
        assert np.linalg.norm(s - target) < 1e-4


@pytest.mark.parametrize("halfvector", [False])
@pytest.mark.parametrize("conductor", [False, True])
def test_newton_jacobian_matches_finite_differences(sms, workloads, oracle, halfvector, conductor):
    """compute_step_anglediff / compute_step_halfvector (manifold_ss.cpp:410-636):
    the analytic 2x2 Jacobian of the constraint against central differences of
    the constraint along the sphere's (u, v) parametrization.  Points whose
    directions come within 25 degrees of the sphcoords pole (where the angle
    constraint is too nonlinear for a finite difference) are skipped."""
    W = workloads
    osc = oracle.OracleScene(W.sphere_scene(conductor=conductor))
    rng = np.random.default_rng(17 + 2 * halfvector + conductor)
    lp = np.array([4.0, -3.0, 2.5], np.float32)   # off-axis: directions away from the pole
    centre, radius, eta = np.array([0.0, 0.0, 1.5]), 1.0, (1.0 if conductor else 1.5)
    h = 2e-4
    checked = 0
    for _ in range(200):
        u, v = rng.uniform(0.05, 0.95), rng.uniform(0.1, 0.9)
        x = np.array([rng.uniform(-2, 2), rng.uniform(-2, 2), 0.0], np.float32)
        nrm = np.array([np.sin(np.pi * v) * np.cos(2 * np.pi * u), np.sin(np.pi * v) * np.sin(2 * np.pi * u),
                        np.cos(np.pi * v)])
        p = centre + radius * nrm
        wi, wo = (x - p) / np.linalg.norm(x - p), (lp - p) / np.linalg.norm(lp - p)
        if eta == 1.0:
            turned = [2 * (w @ nrm) * nrm - w for w in (wi, wo)]
        else:
            turned = []
            for w in (wi, wo):
                e, n = 1 / eta, nrm
                if w @ n < 0:
                    e, n = eta, -n
                root = 1 - e * e * (1 - (w @ n) ** 2)
                turned.append(-(w - n * (w @ n)) * e - n * np.sqrt(max(root, 0.0)))
        if max(abs(w[2]) for w in [wi, wo] + turned) > np.cos(np.radians(25)):
            continue
        c0 = osc.step_at(0, halfvector, u, v, x, lp)
        if not c0[0]:
            continue
        J = c0[3:7].reshape(2, 2).astype(np.float64)
        scale = max(1.0, np.abs(J).max())

        def fd(hh):
            cols = []
            for du, dv in ((hh, 0.0), (0.0, hh)):
                a = osc.step_at(0, halfvector, u + du, v + dv, x, lp)
                b = osc.step_at(0, halfvector, u - du, v - dv, x, lp)
                if not (a[0] and b[0]) or np.abs(a[1:3] - b[1:3]).max() > 1.0:   # failed or wrapped at +-pi
                    return None
                cols.append((a[1:3].astype(np.float64) - b[1:3]) / (2 * hh))
            return np.stack(cols, axis=1)
        d1, d2 = fd(2 * h), fd(h)
        if d1 is None or d2 is None or np.abs(d1 - d2).max() > 1e-2 * scale:
            continue   # too curved here for the difference to have converged
        assert np.abs(J - d2).max() < 2e-2 * scale, (u, v, x.tolist(), J, d2)
        checked += 1
    assert checked >= 20


@pytest.mark.parametrize("halfvector", [False, True])
@pytest.mark.parametrize("conductor", [False, True])
def test_newton_jacobian_on_a_curved_shading_mesh(sms, oracle, halfvector, conductor):
    """Both constraints on a flat quad with tilted vertex normals (curved
    shading, mesh.cpp:693-755 normal derivatives).  On a mesh the shading
    frame derivative of the reference (frame.h:224-242, which treats dp_du as
    constant) is exact, so the half-vector Jacobian is checked here; on a
    sphere only the angle-difference one is (the frame derivative there omits
    the parametrization's curvature, as in the reference)."""
    d = sms.SceneDesc()
    P = np.array([[-1, -1, 1.0], [1, -1, 1.0], [1, 1, 1.0], [-1, 1, 1.0]], np.float32)
    N = np.array([[-0.3, -0.2, 1], [0.25, -0.3, 1], [0.3, 0.2, 1], [-0.2, 0.3, 1]], np.float32)
    N /= np.linalg.norm(N, axis=1, keepdims=True)
    UV = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    F = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
    b = sms.Bsdf(sms.BSDF_CONDUCTOR, 0.2, 3.0) if conductor else sms.Bsdf(sms.BSDF_DIELECTRIC, 1.5)
    d.add_mesh(P, F, b, sms.SHAPE_CAUSTIC_CASTER_SINGLE, N=N, UV=UV)
    d.add_point_emitter((0.3, -0.2, 4.0), (100.0, 100.0, 100.0))
    osc = oracle.OracleScene(d)
    rng = np.random.default_rng(31 + 2 * halfvector + conductor)
    lp = np.array([0.3, -0.2, 4.0], np.float32)
    h = 2e-4
    checked = 0
    for _ in range(100):
        u, v = rng.uniform(0.05, 0.95), rng.uniform(0.05, 0.95)
        if abs(u - v) < 0.01:
            continue   # keep the differences inside one triangle
        x = np.array([rng.uniform(-1, 1), rng.uniform(-1, 1), 0.0], np.float32)
        c0 = osc.step_at(0, halfvector, u, v, x, lp)
        if not c0[0]:
            continue
        J = c0[3:7].reshape(2, 2).astype(np.float64)
        scale = max(1.0, np.abs(J).max())
        cols = []
        for du, dv in ((h, 0.0), (0.0, h)):
            a = osc.step_at(0, halfvector, u + du, v + dv, x, lp)
            bb = osc.step_at(0, halfvector, u - du, v - dv, x, lp)
            cols.append((a[1:3].astype(np.float64) - bb[1:3]) / (2 * h) if a[0] and bb[0] else None)
        if any(c is None for c in cols) or max(np.abs(c).max() for c in cols) > 1e3:
            continue
        fd = np.stack(cols, axis=1)
        assert np.abs(J - fd).max() < 2e-2 * scale, (u, v, x.tolist(), J, fd)
        checked += 1
    assert checked >= 20


@pytest.mark.parametrize("conductor", [False, True])
def test_mnee_init_ignores_the_random_seed(sms, workloads, oracle, conductor):
    """mnee_init (manifold_ss.cpp:229-241) replaces the sampled seed direction
    by the straight line to the light (real ior) or to the shape's bounding-box
    centre (complex ior): every walk of a query is the same walk."""
    W = workloads
    osc = oracle.OracleScene(W.sphere_scene(conductor=conductor))
    cfg = sms.SMSConfig(mnee_init=True)
    q = W.sphere_queries(16)
    n = q.shape[1]
    outs = []
    for seed in (3, 4):
        u = W.pcg32_streams_f32(seed, np.arange(n, dtype=np.uint64), 2)
        w = np.zeros((8, n), np.float32)
        w[2] = 5.0
        w[6], w[7] = u[0], u[1]
        outs.append(osc.walk_batch(cfg, 0, q, w))
    np.testing.assert_array_equal(outs[0], outs[1])
    if not conductor:
        # refraction: the straight line toward the light starts next to the solution
        assert outs[0][0].sum() > 10


def _nm_plane(sms, conductor, res=256):
    """Flat quad z = 1 with a smooth slope map (the reference's normalmap BSDF
    around a dielectric / conductor) flagged as a single-scatter caster."""
    d = sms.SceneDesc()
    P = np.array([[-1, -1, 1.0], [1, -1, 1.0], [1, 1, 1.0], [-1, 1, 1.0]], np.float32)
    UV = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    F = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
    b = sms.Bsdf(sms.BSDF_CONDUCTOR, 0.2, 3.0) if conductor else sms.Bsdf(sms.BSDF_DIELECTRIC, 1.5)
    sid = d.add_mesh(P, F, b, sms.SHAPE_CAUSTIC_CASTER_SINGLE, UV=UV)
    t = (np.arange(res) + 0.5) / res
    vv, uu = np.meshgrid(t, t, indexing="ij")
    sl = np.stack([0.15 * np.sin(2 * np.pi * (2 * uu + vv)), 0.1 * np.cos(2 * np.pi * (uu - 2 * vv))], axis=-1)
    d.normalmap = (sid, sl.astype(np.float16), 1.0)
    d.add_point_emitter((0.3, -0.2, 4.0), (100.0, 100.0, 100.0))
    return d


@pytest.mark.parametrize("halfvector", [False, True])
@pytest.mark.parametrize("conductor", [False, True])
def test_newton_jacobian_on_a_normal_mapped_caster(sms, oracle, halfvector, conductor):
    """Normal-mapped caster: the manifold vertex takes the normal-mapped frame
    and its derivative (normalmap.cpp:236-290, the bilinear slope derivative
    of normalmap.h:125-193).  Central differences of the constraint inside one
    bilinear cell of the slope map match the Newton Jacobian."""
    res = 256
    desc = _nm_plane(sms, conductor, res)
    osc = oracle.OracleScene(desc)
    rng = np.random.default_rng(41 + 2 * halfvector + conductor)
    lp = np.array([0.3, -0.2, 4.0], np.float32)
    # the map is in effect: the constraint differs from the bare plane's
    desc.normalmap = None
    bare = oracle.OracleScene(desc)
    x0 = np.array([0.2, 0.1, 0.0], np.float32)
    assert not np.allclose(osc.step_at(0, halfvector, 0.37, 0.61, x0, lp)[1:3],
                           bare.step_at(0, halfvector, 0.37, 0.61, x0, lp)[1:3], atol=1e-4)
    h = 2e-4
    checked = 0
    for _ in range(100):
        # cell centres of the bilinear interpolant sit at integer multiples of 1/res
        i, j = rng.integers(4, res - 4, size=2)
        u = (i + rng.uniform(-0.3, 0.3)) / res
        v = (j + rng.uniform(-0.3, 0.3)) / res
        if abs(u - v) < 0.01:
            continue   # keep the differences inside one triangle
        x = np.array([rng.uniform(-1, 1), rng.uniform(-1, 1), 0.0], np.float32)
        c0 = osc.step_at(0, halfvector, u, v, x, lp)
        if not c0[0]:
            continue
        J = c0[3:7].reshape(2, 2).astype(np.float64)
        scale = max(1.0, np.abs(J).max())
        cols = []
        for du, dv in ((h, 0.0), (0.0, h)):
            a = osc.step_at(0, halfvector, u + du, v + dv, x, lp)
            bb = osc.step_at(0, halfvector, u - du, v - dv, x, lp)
            cols.append((a[1:3].astype(np.float64) - bb[1:3]) / (2 * h) if a[0] and bb[0] else None)
        if any(c is None for c in cols) or max(np.abs(c).max() for c in cols) > 1e3:
            continue
        fd = np.stack(cols, axis=1)
        assert np.abs(J - fd).max() < 2e-2 * scale, (u, v, x.tolist(), J, fd)
        checked += 1
    assert checked >= 20


def test_two_stage_slope_gaussian_moments(oracle):
    """sample_gaussian (manifold.h:326-345): mean mu and covariance sigma for a
    correlated sigma, through square_to_std_normal (warp.h:184-190)."""
    from oracle import oracle as O
    mu, a, b, c = np.array([0.1, -0.2], np.float32), 0.04, 0.01, 0.012
    u = np.random.default_rng(5).random((20000, 2)).astype(np.float32)
    s = np.array([O.sample_slope_gaussian(mu, a, b, c, x) for x in u])
    assert np.allclose(s.mean(0), mu, atol=0.006)
    cov = np.cov(s.T)
    assert np.allclose(cov, [[a, c], [c, b]], rtol=0.06, atol=5e-4)


@pytest.mark.parametrize("conductor,freq", [(False, 4), (True, 1)])
def test_two_stage_solver_is_unbiased(sms, workloads, oracle, conductor, freq):
    """The two-stage solver (manifold_ss.cpp:253-270) only changes where walks
    start: the unbiased estimator gives the same expectation with and without
    it on a normal-mapped caster, and it converges more often on the bumpier
    map (its purpose)."""
    W = workloads
    osc = oracle.OracleScene(W.nm_plane_scene(conductor=conductor, freq=freq))
    q = W.nm_plane_queries(4096)
    res = {}
    for two in (False, True):
        cfg = sms.SMSConfig(biased=False, max_trials=-1, twostage=two)
        m, succ = [], 0.0
        for r in range(8):
            v, c, w, st = osc.connect_batch(cfg, q, seed=200 + r)
            m.append(float(v[0].mean()))
            succ += st["solver_succeeded"] / st["walks"]
        res[two] = (np.mean(m), np.std(m, ddof=1) / np.sqrt(len(m)), succ / 8)
    (a, sa, pa), (b, sb, pb) = res[False], res[True]
    assert a > 0.05
    assert abs(a - b) < 4.0 * np.hypot(sa, sb) + 0.02 * a, res
    assert pb > pa, res


def test_two_stage_walk_inputs(sms, workloads, oracle):
    """With twostage the per-walk harness takes two more rows (the smoothed
    solve's slope sample); the same walk with different slope samples can end
    on different solutions, and more walks converge than without it."""
    W = workloads
    osc = oracle.OracleScene(W.nm_plane_scene(freq=4))
    cfg = sms.SMSConfig(twostage=True)
    q = W.nm_plane_queries(256)
    w = np.zeros((10, 256), np.float32)
    w[0:3] = np.array([0.3, -0.2, 4.0], np.float32)[:, None]
    u = W.pcg32_streams_f32(3, np.arange(256, dtype=np.uint64), 4)
    w[6:10] = u
    with pytest.raises(ValueError):
        osc.walk_batch(cfg, 0, q, w[:8])
    a = osc.walk_batch(cfg, 0, q, w)
    w2 = w.copy()
    w2[8:10] = 1.0 - w[8:10]
    b = osc.walk_batch(cfg, 0, q, w2)
    assert a[0].mean() > 0.05
    both = (a[0] > 0.5) & (b[0] > 0.5)
    assert np.any(np.linalg.norm(a[2:5, both] - b[2:5, both], axis=0) > 1e-3)
    plain = osc.walk_batch(sms.SMSConfig(), 0, q, w[:8])
    assert a[0].mean() > plain[0].mean()


def test_normal_mapped_oracle_regression(sms, workloads, oracle):
    """Bit-exact regression of the oracle's normal-mapped caster restatement
    (two-stage walks, unbiased estimates with and without the two-stage
    solver) against tests/golden/oracle_nm.npz."""
    W = workloads
    ref = np.load(GOLDEN / "oracle_nm.npz")
    osc = oracle.OracleScene(W.nm_plane_scene(freq=4))
    n = 128
    q = W.nm_plane_queries(n)
    w = np.zeros((10, n), np.float32)
    w[0:3] = np.array([0.3, -0.2, 4.0], np.float32)[:, None]
    w[6:10] = W.pcg32_streams_f32(13, np.arange(n, dtype=np.uint64), 4)
    np.testing.assert_array_equal(osc.walk_batch(sms.SMSConfig(twostage=True), 0, q, w), ref["nm_walk_twostage"])
    for two in (False, True):
        cfg = sms.SMSConfig(biased=False, max_trials=64, twostage=two)
        v, c, wk, st = osc.connect_batch(cfg, W.nm_plane_queries(256), seed=9, nthreads=2)
        tag = "twostage" if two else "plain"
        assert np.array_equal(c, ref[f"nm_{tag}_count"]) and np.array_equal(wk, ref[f"nm_{tag}_walks"])
        np.testing.assert_allclose(v, ref[f"nm_{tag}_value"], rtol=1e-6, atol=1e-9)
