"""GPU parity of normal-mapped single-scatter casters against the oracle,
through the C ABI: manifold vertices with the normal map's frame and its
derivative (src/bsdfs/normalmap.cpp:236-290), the two-stage solver
(manifold_ss.cpp:253-270), rough normal-mapped casters, the refusals, and
path_sms_ss / path rendering through a normal-mapped dielectric.

Walks on a bumpy normal map are chaotic under rounding like the water
heightfields, so the yardstick is the oracle's disagreement with its own
FMA-contracted build (see test_gpu_ss_parity)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FLOOR_FACTOR = 1.5
FLOOR_SLACK = 0.005
POS_TOL = 1e-4
UNSUPPORTED = 4


def _walk_inputs(W, n, light, two, seed=11):
    u = W.pcg32_streams_f32(seed, np.arange(n, dtype=np.uint64), 4)
    w = np.zeros((10 if two else 8, n), np.float32)
    w[0:3] = np.asarray(light, np.float32)[:, None]
    w[6:8] = u[0:2]
    if two:
        w[8:10] = u[2:4]
    return w


def _walk_diff(a, b):
    """(flag mismatch fraction, fraction solved by both to different
    solutions, median |dp| over walks solved to the same solution, both)."""
    oka, okb = a[0] > 0.5, b[0] > 0.5
    both = oka & okb
    d = np.linalg.norm(a[2:5, both] - b[2:5, both], axis=0)
    same = d < POS_TOL
    med = float(np.median(d[same])) if same.any() else 0.0
    return float(np.mean(oka != okb)), float(np.sum(~same)) / len(oka), med, int(both.sum())


def _connect_diff(va, ca, wa, vb, cb, wb, rtol=1e-3):
    same_cw = (ca == cb) & (wa == wb)
    scale = np.maximum(np.abs(vb).max(axis=0), 1e-6)
    rel = np.abs(va - vb).max(axis=0) / scale
    nonzero = np.abs(vb).max(axis=0) > 1e-6
    differs = ~same_cw | (nonzero & (rel > rtol))
    agree = same_cw & nonzero & (rel <= rtol)
    med = float(np.median(rel[agree])) if agree.any() else 0.0
    return float(np.mean(ca != cb)), float(np.mean(differs)), med


@pytest.mark.parametrize("twostage", [False, True])
@pytest.mark.parametrize("conductor", [False, True])
def test_normal_mapped_walks(sms, workloads, oracle, gpu_lib, conductor, twostage):
    """Per-walk sample_path on the normal-mapped plane: converged flag,
    solution, initial hit and the solution's (normal-mapped) vertex normal."""
    W = workloads
    desc = W.nm_plane_scene(conductor=conductor, freq=4)
    cfg = sms.SMSConfig(twostage=twostage)
    ctx = sms.Context(sms.Scene(desc), cfg)
    n = 8192
    q = W.nm_plane_queries(n)
    light = (0.3, -0.2, -3.0) if conductor else (0.3, -0.2, 4.0)
    w = _walk_inputs(W, n, light, twostage)
    out_g = sms.SpecularManifoldSingleScatter(ctx).sample_path(0, q, w)
    out_o = oracle.OracleScene(desc).walk_batch(cfg, 0, q, w)
    out_f = oracle.OracleScene(desc, fma=True).walk_batch(cfg, 0, q, w)
    g_m, g_c, g_med, nboth = _walk_diff(out_g, out_o)
    f_m, f_c, _, _ = _walk_diff(out_f, out_o)
    print(f"nm conductor={conductor} twostage={twostage}: mismatch {g_m:.4f} crossed {g_c:.4f} | floor "
          f"{f_m:.4f} {f_c:.4f} | median|dp| {g_med:.1e} both {nboth}")
    assert nboth > 100
    assert g_m <= FLOOR_FACTOR * f_m + FLOOR_SLACK
    assert g_c <= FLOOR_FACTOR * f_c + FLOOR_SLACK
    assert g_med < 1e-5
    same = (out_g[0] > 0.5) & (out_o[0] > 0.5) & (np.linalg.norm(out_g[2:5] - out_o[2:5], axis=0) < POS_TOL)
    # the solution normal is the map's, not the plane's
    assert np.abs(out_g[8:11, same] - out_o[8:11, same]).max() < 1e-3
    assert np.mean(np.abs(out_g[10, same]) < 0.999) > 0.5
    ctx.close()


@pytest.mark.parametrize("alpha", [0.0, 0.2])
@pytest.mark.parametrize("twostage", [False, True])
@pytest.mark.parametrize("biased", [False, True])
def test_normal_mapped_connect(sms, workloads, oracle, gpu_lib, biased, twostage, alpha):
    """Estimators on the normal-mapped dielectric plane, smooth and rough
    (offset normals on top of the map), with and without the two-stage
    solver: GPU vs oracle on the same random streams against the FMA floor."""
    W = workloads
    desc = W.nm_plane_scene(conductor=False, freq=4, alpha=alpha)
    cfg = sms.SMSConfig(biased=biased, max_trials=16 if biased else 256, twostage=twostage)
    ctx = sms.Context(sms.Scene(desc), cfg)
    q = W.nm_plane_queries(4096)
    vg, cg, wg = sms.SpecularManifoldSingleScatter(ctx).specular_manifold_sampling(q, seed=3)
    vo, co, wo, st_o = oracle.OracleScene(desc).connect_batch(cfg, q, seed=3)
    vf, cf, wf, st_f = oracle.OracleScene(desc, fma=True).connect_batch(cfg, q, seed=3)
    g_cm, g_diff, g_med = _connect_diff(vg, cg, wg, vo, co, wo)
    f_cm, f_diff, _ = _connect_diff(vf, cf, wf, vo, co, wo)
    print(f"nm connect biased={biased} twostage={twostage} alpha={alpha}: count mismatch {g_cm:.4f} differs "
          f"{g_diff:.4f} (floor {f_cm:.4f}/{f_diff:.4f}) median rel {g_med:.1e} nonzero {np.mean(vo[0] > 0):.3f}")
    assert np.mean(vo[0] > 0) > 0.05
    assert g_cm <= FLOOR_FACTOR * f_cm + FLOOR_SLACK
    assert g_diff <= FLOOR_FACTOR * f_diff + FLOOR_SLACK
    assert g_med < 1e-3
    st = ctx.stats()
    # total walks: the queries whose outcome flips under rounding carry their
    # own trial counts, so the yardstick is again the oracle builds' difference
    assert abs(st["walks"] - st_o["walks"]) <= 3 * abs(st_f["walks"] - st_o["walks"]) + 0.02 * st_o["walks"] + 16
    ctx.close()


def test_normal_mapped_noalloc_matches_device_path(sms, workloads, gpu_lib):
    """The allocation-free entry point runs the normal-mapped kernels too; with
    twostage it needs the LEAN pyramid, which the first device call builds."""
    torch = pytest.importorskip("torch")
    W = workloads
    ctx = sms.Context(sms.Scene(W.nm_plane_scene(freq=4)), sms.SMSConfig(biased=False, max_trials=64, twostage=True))
    ss = sms.SpecularManifoldSingleScatter(ctx)
    n = 2048
    q = torch.from_numpy(np.ascontiguousarray(W.nm_plane_queries(n))).cuda()

    def run(fn):
        v = torch.zeros(3, n, device="cuda")
        c = torch.zeros(n, dtype=torch.int32, device="cuda")
        w = torch.zeros(n, dtype=torch.int32, device="cuda")
        fn(q.data_ptr(), n, v.data_ptr(), c.data_ptr(), w.data_ptr(), seed=4)
        torch.cuda.synchronize()
        return v.cpu().numpy(), c.cpu().numpy(), w.cpu().numpy()

    with pytest.raises(sms.SMSError) as e:
        run(ss.specular_manifold_sampling_noalloc)
    assert e.value.status == UNSUPPORTED
    a = run(ss.specular_manifold_sampling_device)
    b = run(ss.specular_manifold_sampling_noalloc)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    assert (a[0][0] > 0).mean() > 0.05
    ctx.close()


def test_normal_map_refusals(sms, workloads, gpu_lib):
    """twostage needs every single-scatter caster normal-mapped (the
    reference's lean() of a plain BSDF is zero: its slope draw is NaN and no
    walk converges); rough normal-mapped shapes in a render are not
    supported."""
    W = workloads
    ctx = sms.Context(sms.Scene(W.sphere_scene()), sms.SMSConfig(twostage=True))
    ss = sms.SpecularManifoldSingleScatter(ctx)
    q = W.sphere_queries(4)
    for call in (lambda: ss.specular_manifold_sampling(q),
                 lambda: ss.sample_path(0, q, np.zeros((10, q.shape[1]), np.float32))):
        with pytest.raises(sms.SMSError) as e:
            call()
        assert e.value.status == UNSUPPORTED
    ctx.close()
    ctx = sms.Context(sms.Scene(W.nm_plane_scene(alpha=0.2)), sms.SMSConfig())
    with pytest.raises(sms.SMSError) as e:
        ctx.render(W.pool_camera(8, 8), sms.RenderOptions(integrator="path_sms_ss", spp=1))
    assert e.value.status == UNSUPPORTED
    ctx.close()


def _nm_pool(W, freq=1, point_light=False):
    d = W.pool_scene(res=16, wave_scale=0.0, point_light=point_light)
    d.normalmap = (1, W.nm_plane_slopes(256, 0.15, freq), 1.0)
    return d


@pytest.mark.parametrize("twostage", [False, True])
def test_render_through_normal_mapped_caster_matches_oracle(sms, workloads, oracle, gpu_lib, twostage):
    """path_sms_ss over the pool floor under a normal-mapped flat water sheet:
    SMS on the normal-mapped caster and camera paths refracted by the
    normal-mapped dielectric (NormalmapBSDF::sample, normalmap.cpp:118-135)."""
    from test_gpu_render import _check_against_oracle
    W = workloads
    cfg = sms.SMSConfig(biased=False, max_trials=64, twostage=twostage)
    g, o, f = _check_against_oracle(sms, oracle, _nm_pool(W, 2), cfg, W.pool_camera(16, 16),
                                    sms.RenderOptions(integrator="path_sms_ss", spp=4, seed=13))
    assert o.mean() > 0.0


@pytest.mark.parametrize("twostage", [False, True])
def test_normal_mapped_caustic_is_unbiased_against_path(sms, workloads, gpu_lib, twostage):
    """Unbiased SMS on the normal-mapped sheet, with and without the two-stage
    solver, against plain path tracing through the same normal-mapped
    dielectric (which reaches the sphere light by BSDF sampling)."""
    from test_gpu_render import _compare_integrators
    W = workloads
    ctx = sms.Context(sms.Scene(_nm_pool(W, 1)), sms.SMSConfig(biased=False, max_trials=-1, twostage=twostage))
    _compare_integrators(sms, ctx, W.pool_camera(32, 32), "path_sms_ss", 4096, 512, 4)
    ctx.close()


def _nm_ms_scene(sms, W, conductor):
    """The normal-mapped plane as a one-vertex multi-scatter chain."""
    d = W.nm_plane_scene(conductor=conductor, freq=4)
    P, N, UV, F, b, _ = d.meshes[0]
    d.meshes[0] = (P, N, UV, F, b, sms.SHAPE_CAUSTIC_CASTER_MULTI)
    pos, inten, _ = d.point_emitters[0]
    d.point_emitters[0] = (pos, inten, sms.EMITTER_CAUSTIC_MULTI)
    return d


@pytest.mark.parametrize("conductor", [False, True])
def test_normal_mapped_multi_scatter(sms, workloads, oracle, gpu_lib, conductor):
    """Multi-scatter chains on a normal-mapped shape (the chain kernels built
    with the normal-mapped frames): per-walk and biased / unbiased estimates,
    GPU vs oracle against the FMA floor."""
    W = workloads
    desc = _nm_ms_scene(sms, W, conductor)
    light = (0.3, -0.2, -3.0) if conductor else (0.3, -0.2, 4.0)
    n = 4096
    q = W.nm_plane_queries(n)
    cfg = sms.SMSConfig(bounces=1)
    ctx = sms.Context(sms.Scene(desc), cfg)
    w = _walk_inputs(W, n, light, False)
    out_g = sms.SpecularManifoldMultiScatter(ctx).sample_path(0, q, w)
    out_o = oracle.OracleScene(desc).ms_walk_batch(cfg, 0, q, w)
    out_f = oracle.OracleScene(desc, fma=True).ms_walk_batch(cfg, 0, q, w)
    g = np.mean((out_g[0] > 0.5) != (out_o[0] > 0.5))
    f = np.mean((out_f[0] > 0.5) != (out_o[0] > 0.5))
    both = (out_g[0] > 0.5) & (out_o[0] > 0.5)
    print(f"nm ms walks conductor={conductor}: mismatch {g:.4f} floor {f:.4f} both {both.sum()}")
    assert both.sum() > 50
    assert g <= FLOOR_FACTOR * f + FLOOR_SLACK
    assert np.median(np.linalg.norm(out_g[2:5, both] - out_o[2:5, both], axis=0)) < 1e-5
    ctx.close()
    for biased in (True, False):
        cfg = sms.SMSConfig(bounces=1, biased=biased, max_trials=16 if biased else 256)
        ctx = sms.Context(sms.Scene(desc), cfg)
        vg, cg, wg = sms.SpecularManifoldMultiScatter(ctx).specular_manifold_sampling(q, seed=5)
        vo, co, wo, _ = oracle.OracleScene(desc).connect_batch(cfg, q, seed=5, multi=True)
        vf, cf, wf, _ = oracle.OracleScene(desc, fma=True).connect_batch(cfg, q, seed=5, multi=True)
        g_cm, g_diff, g_med = _connect_diff(vg, cg, wg, vo, co, wo)
        f_cm, f_diff, _ = _connect_diff(vf, cf, wf, vo, co, wo)
        print(f"nm ms connect conductor={conductor} biased={biased}: count mismatch {g_cm:.4f} differs {g_diff:.4f} "
              f"(floor {f_cm:.4f}/{f_diff:.4f}) median rel {g_med:.1e} nonzero {np.mean(vo[0] > 0):.3f}")
        assert np.mean(vo[0] > 0) > 0.02
        assert g_cm <= FLOOR_FACTOR * f_cm + FLOOR_SLACK
        assert g_diff <= FLOOR_FACTOR * f_diff + FLOOR_SLACK
        assert g_med < 1e-3
        ctx.close()
