"""GPU single-scatter parity against the CPU oracle, through the C ABI.

Per-walk parity follows the harness of the reference's figure scripts
(results/Figure_4_5_RingSolutions/generate_plots_simple.py:159-172: explicit
start points in, converged flag + solution out).

Tolerances (scene scale 1):
  * sphere scenes are well conditioned: the oracle agrees with its own
    FMA-contracted build on every walk, so GPU flag mismatches must stay below
    STRICT_MISMATCH and positions of the same solution within POS_TOL;
  * the water heightfields are chaotic under rounding: the oracle disagrees
    with its own FMA build on several percent of the walks (a one-rounding
    perturbation).  That measured floor f is the yardstick: the GPU may not
    disagree with the oracle more than FLOOR_FACTOR * f + FLOOR_SLACK;
  * biased unique-solution counts on the sphere are integers and must match on
    all but STRICT_MISMATCH of the queries; contributions of matching queries
    within VALUE_RTOL.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STRICT_MISMATCH = 0.005
POS_TOL = 1e-4
VALUE_RTOL = 2e-3
FLOOR_FACTOR = 1.5
FLOOR_SLACK = 0.005


def _walk_inputs(W, n, light, seed=11):
    u = W.pcg32_streams_f32(seed, np.arange(n, dtype=np.uint64), 2)
    w = np.zeros((8, n), np.float32)
    w[0], w[1], w[2] = light
    w[6], w[7] = u[0], u[1]
    return w


def _walk_diff(a, b):
    """(flag mismatch fraction, fraction solved by both to different solutions,
    median |dp| over walks solved to the same solution)."""
    oka, okb = a[0] > 0.5, b[0] > 0.5
    both = oka & okb
    d = np.linalg.norm(a[2:5, both] - b[2:5, both], axis=0)
    same = d < POS_TOL
    med = float(np.median(d[same])) if same.any() else 0.0
    return float(np.mean(oka != okb)), float(np.sum(~same)) / len(oka), med, int(both.sum())


@pytest.mark.parametrize("halfvector", [False, True])
@pytest.mark.parametrize("conductor", [False, True])
def test_sphere_walks(sms, workloads, oracle, gpu_lib, conductor, halfvector):
    W = workloads
    desc = W.sphere_scene(conductor=conductor)
    cfg = sms.SMSConfig(halfvector_constraints=halfvector)
    ctx = sms.Context(sms.Scene(desc), cfg)
    ss = sms.SpecularManifoldSingleScatter(ctx)
    q = W.sphere_queries(64)
    w = _walk_inputs(W, q.shape[1], (0.0, 0.0, 5.0))
    out_g = ss.sample_path(0, q, w)
    out_o = oracle.OracleScene(desc).walk_batch(cfg, 0, q, w)
    mism, crossed, med, nboth = _walk_diff(out_g, out_o)
    print(f"sphere conductor={conductor} halfvector={halfvector}: mismatch {mism:.5f} crossed {crossed:.5f} "
          f"median|dp| {med:.1e} both {nboth}")
    assert nboth > 20
    assert mism < STRICT_MISMATCH and crossed < STRICT_MISMATCH
    assert med < 1e-5
    hit = (np.abs(out_o[5:8]).sum(0) > 0) & (np.abs(out_g[5:8]).sum(0) > 0)
    assert np.abs(out_g[5:8, hit] - out_o[5:8, hit]).max() < 1e-4
    # iteration counts agree on walks with the same outcome
    same = (out_g[0] == out_o[0])
    assert np.mean(out_g[1, same] == out_o[1, same]) > 0.99


@pytest.mark.parametrize("res,halfvector", [(128, False), (512, False), (128, True)])
def test_water_walks_within_chaos_floor(sms, workloads, oracle, gpu_lib, res, halfvector):
    W = workloads
    desc = W.water_scene(res=res)
    cfg = sms.SMSConfig(halfvector_constraints=halfvector)
    ctx = sms.Context(sms.Scene(desc), cfg)
    ss = sms.SpecularManifoldSingleScatter(ctx)
    n = 16384
    q = W.water_queries(n)
    w = _walk_inputs(W, n, (0.0, 0.05, 10.0))
    out_g = ss.sample_path(0, q, w)
    out_o = oracle.OracleScene(desc).walk_batch(cfg, 0, q, w)
    out_f = oracle.OracleScene(desc, fma=True).walk_batch(cfg, 0, q, w)
    g_m, g_c, g_med, nboth = _walk_diff(out_g, out_o)
    f_m, f_c, f_med, _ = _walk_diff(out_f, out_o)
    print(f"water{res} halfvector={halfvector}: gpu mismatch {g_m:.4f} crossed {g_c:.4f} | floor mismatch {f_m:.4f} "
          f"crossed {f_c:.4f} | median|dp| {g_med:.1e} both {nboth}")
    assert nboth > 200
    assert g_m <= FLOOR_FACTOR * f_m + FLOOR_SLACK
    assert g_c <= FLOOR_FACTOR * f_c + FLOOR_SLACK
    assert g_med < 1e-5
    # converged fraction and iteration statistics agree
    assert abs(out_g[0].mean() - out_o[0].mean()) < 0.01
    assert abs(out_g[1].mean() - out_o[1].mean()) < 0.2


def _connect_diff(va, ca, wa, vb, cb, wb, rtol=1e-3):
    """(count mismatch fraction, fraction of queries whose estimate differs --
    count, walk count or value beyond rtol -- and the median relative value
    error over queries that agree)."""
    same_cw = (ca == cb) & (wa == wb)
    scale = np.maximum(np.abs(vb).max(axis=0), 1e-6)
    rel = (np.abs(va - vb).max(axis=0) / scale)
    nonzero = np.abs(vb).max(axis=0) > 1e-6
    differs = ~same_cw | (nonzero & (rel > rtol))
    agree = same_cw & nonzero & (rel <= rtol)
    med = float(np.median(rel[agree])) if agree.any() else 0.0
    return float(np.mean(ca != cb)), float(np.mean(differs)), med


@pytest.mark.parametrize("conductor", [False, True])
def test_sphere_connect_biased(sms, workloads, oracle, gpu_lib, conductor):
    W = workloads
    desc = W.sphere_scene(conductor=conductor)
    cfg = W.sphere_config()
    ctx = sms.Context(sms.Scene(desc), cfg)
    ss = sms.SpecularManifoldSingleScatter(ctx)
    q = W.sphere_queries(64)   # the full 64x64 benchmark grid
    vg, cg, wg = ss.specular_manifold_sampling(q, seed=1)
    vo, co, wo, st_o = oracle.OracleScene(desc).connect_batch(cfg, q, seed=1)
    vf, cf, wf, _ = oracle.OracleScene(desc, fma=True).connect_batch(cfg, q, seed=1)
    g_cm, g_diff, g_med = _connect_diff(vg, cg, wg, vo, co, wo)
    f_cm, f_diff, _ = _connect_diff(vf, cf, wf, vo, co, wo)
    print(f"sphere biased conductor={conductor}: count mismatch {g_cm:.5f} differs {g_diff:.5f} "
          f"(floor {f_cm:.5f}/{f_diff:.5f}) median rel {g_med:.1e} unique {co.sum()} vs {cg.sum()}")
    assert np.all(wg == 16) and np.all(wo == 16)
    assert g_cm < STRICT_MISMATCH
    assert g_diff <= FLOOR_FACTOR * f_diff + STRICT_MISMATCH
    assert g_med < 1e-4
    st = ctx.stats()
    assert st["walks"] == st_o["walks"] == 16 * q.shape[1]
    assert st["connections"] == q.shape[1]
    assert abs(st["solver_succeeded"] - st_o["solver_succeeded"]) <= 0.005 * st_o["solver_succeeded"] + 2
    if conductor:
        assert co.sum() > 100 and vo.sum() > 0
        assert abs(vg.sum() - vo.sum()) <= 0.01 * vo.sum()


def test_water_connect_unbiased(sms, workloads, oracle, gpu_lib):
    W = workloads
    desc = W.water_scene(res=128)
    cfg = W.water_config()
    ctx = sms.Context(sms.Scene(desc), cfg)
    ss = sms.SpecularManifoldSingleScatter(ctx)
    n = 8192
    q = W.water_queries(n)
    vg, cg, wg = ss.specular_manifold_sampling(q, seed=5)
    vo, co, wo, _ = oracle.OracleScene(desc).connect_batch(cfg, q, seed=5)
    vf, cf, wf, _ = oracle.OracleScene(desc, fma=True).connect_batch(cfg, q, seed=5)
    g_cm, g_diff, g_med = _connect_diff(vg, cg, wg, vo, co, wo)
    f_cm, f_diff, _ = _connect_diff(vf, cf, wf, vo, co, wo)
    print(f"water unbiased: gpu count mismatch {g_cm:.4f} differs {g_diff:.4f} "
          f"(floor {f_cm:.4f}/{f_diff:.4f}) median rel {g_med:.1e}")
    assert g_cm <= FLOOR_FACTOR * f_cm + FLOOR_SLACK
    assert g_diff <= FLOOR_FACTOR * f_diff + FLOOR_SLACK
    assert g_med < 1e-4
    # identical outcome classes in distribution
    for cls in (lambda c: c == 0, lambda c: c == -1, lambda c: c > 0):
        assert abs(cls(cg).mean() - cls(co).mean()) <= 2 * abs(cls(cf).mean() - cls(co).mean()) + 0.01


def test_water_full_size_invariants(sms, workloads, gpu_lib):
    """1M queries on the 512x512 water: exact bookkeeping identities of the
    unbiased estimator (manifold_ss.cpp:73-141)."""
    W = workloads
    cfg = W.water_config()
    ctx = sms.Context(sms.Scene(W.water_scene()), cfg)
    ss = sms.SpecularManifoldSingleScatter(ctx)
    n = 1 << 20
    q = W.water_queries(n)
    v, c, w = ss.specular_manifold_sampling(q, seed=1)
    st = ctx.stats()
    assert np.isfinite(v).all() and (v >= 0).all()
    assert np.all((c == -1) | (c == 0) | ((c >= 1) & (c <= cfg.max_trials)))
    assert np.all(v[:, c <= 0] == 0)
    assert np.all(w[c == 0] == 1)
    assert np.all(w[c > 0] == 1 + c[c > 0])
    assert np.all(w[c == -1] == 1 + cfg.max_trials)
    assert st["walks"] == w.sum()
    assert st["connections"] == n
    assert st["bernoulli_trial_iterations"] == c[c > 0].sum() + (cfg.max_trials + 1) * np.sum(c == -1)
    assert st["bernoulli_trial_calls"] == np.sum(c != 0)
    assert st["bernoulli_trial_iterations_max"] <= cfg.max_trials + 1


def test_results_independent_of_batching_and_launch(sms, workloads, gpu_lib):
    """Each query owns its RNG stream (seed, stream_offset + index): splitting a
    batch or changing the persistent grid gives bit-identical results."""
    W = workloads
    ctx = sms.Context(sms.Scene(W.water_scene(res=128)), W.water_config())
    ss = sms.SpecularManifoldSingleScatter(ctx)
    n = 20000
    q = W.water_queries(n)
    v, c, w = ss.specular_manifold_sampling(q, seed=9)
    a, b = 7000, 13000
    v2, c2, w2 = ss.specular_manifold_sampling(np.ascontiguousarray(q[:, a:b]), seed=9, stream_offset=a)
    assert np.array_equal(c[a:b], c2) and np.array_equal(w[a:b], w2) and np.array_equal(v[:, a:b], v2)
    ctx.set_launch(1)
    v3, c3, w3 = ss.specular_manifold_sampling(q, seed=9)
    assert np.array_equal(c, c3) and np.array_equal(v, v3)


def test_empty_and_single(sms, workloads, gpu_lib):
    W = workloads
    ctx = sms.Context(sms.Scene(W.sphere_scene()), W.sphere_config())
    ss = sms.SpecularManifoldSingleScatter(ctx)
    v, c, w = ss.specular_manifold_sampling(np.zeros((16, 0), np.float32))
    assert v.shape == (3, 0)
    v, c, w = ss.specular_manifold_sampling(W.sphere_queries(1), seed=3)
    assert w[0] == 16


def test_bad_arguments(sms, workloads, gpu_lib):
    W = workloads
    ctx = sms.Context(sms.Scene(W.sphere_scene()), W.sphere_config())
    ss = sms.SpecularManifoldSingleScatter(ctx)
    q = W.sphere_queries(2)
    with pytest.raises(sms.SMSError):
        ss.sample_path(7, q, np.zeros((8, q.shape[1]), np.float32))
    ctx.set_config(sms.SMSConfig(twostage=True))
    with pytest.raises(sms.SMSError):
        ss.specular_manifold_sampling(q)   # twostage on a caster without a normal map
    with pytest.raises(ValueError):
        ss.specular_manifold_sampling(np.zeros((15, 4), np.float32))


@pytest.mark.parametrize("conductor", [False, True])
def test_mnee_init_walks_and_connect(sms, workloads, oracle, gpu_lib, conductor):
    """mnee_init: deterministic straight-line seeds, GPU vs oracle per walk and
    for the biased estimator (every walk of a query finds the same solution,
    so at most one unique solution)."""
    W = workloads
    desc = W.sphere_scene(conductor=conductor)
    cfg = sms.SMSConfig(mnee_init=True)
    ctx = sms.Context(sms.Scene(desc), cfg)
    ss = sms.SpecularManifoldSingleScatter(ctx)
    q = W.sphere_queries(64)
    w = _walk_inputs(W, q.shape[1], (0.0, 0.0, 5.0))
    out_g = ss.sample_path(0, q, w)
    out_o = oracle.OracleScene(desc).walk_batch(cfg, 0, q, w)
    mism, crossed, med, nboth = _walk_diff(out_g, out_o)
    print(f"mnee conductor={conductor}: mismatch {mism:.5f} both {nboth}")
    assert mism < STRICT_MISMATCH and crossed < STRICT_MISMATCH
    if not conductor:
        assert nboth > 20
    bcfg = sms.SMSConfig(mnee_init=True, biased=True, max_trials=8)
    ctx.set_config(bcfg)
    vg, cg, wg = ss.specular_manifold_sampling(q, seed=2)
    vo, co, wo, _ = oracle.OracleScene(desc).connect_batch(bcfg, q, seed=2)
    assert np.all(cg <= 1) and np.mean(cg == co) > 1 - STRICT_MISMATCH
    ctx.close()


def _rough_scene(sms, W, conductor, alpha):
    """A rough caster over a point light's receiver plane: a flat Beckmann
    dielectric sheet (refraction) or a rough conductor sphere (reflection)."""
    d = sms.SceneDesc()
    if conductor:
        d.add_sphere((0.0, 0.0, 1.5), 1.0, sms.Bsdf(sms.BSDF_CONDUCTOR, 0.2, 3.0, alpha=alpha),
                     sms.SHAPE_CAUSTIC_CASTER_SINGLE)
        d.add_point_emitter((0.0, 0.0, 5.0), (100.0,) * 3, sms.EMITTER_CAUSTIC_SINGLE)
    else:
        P, N, UV, F = W.heightfield_mesh(16, 1.0, 1.3, [])
        d.add_mesh(P, F, sms.Bsdf(sms.BSDF_DIELECTRIC, 1.5, alpha=alpha), sms.SHAPE_CAUSTIC_CASTER_SINGLE,
                   N=N, UV=UV)
        d.add_point_emitter((0.3, 0.2, 4.0), (40.0,) * 3, sms.EMITTER_CAUSTIC_SINGLE)
    return d


@pytest.mark.parametrize("biased", [True, False])
@pytest.mark.parametrize("conductor", [False, True])
def test_rough_caster_connect(sms, workloads, oracle, gpu_lib, biased, conductor):
    """Rough casters: each query draws a Beckmann offset normal after its
    emitter sample (manifold_ss.cpp:60-70), walks to the offset-normal
    constraint and divides by the offset density; the glossy reflectance is
    the BSDF value in the half-vector domain (:648-669).  GPU vs oracle on the
    same random streams, against the oracle-vs-FMA floor."""
    W = workloads
    desc = _rough_scene(sms, W, conductor, 0.2)
    cfg = sms.SMSConfig(biased=True, max_trials=16) if biased else sms.SMSConfig(biased=False, max_trials=256)
    ctx = sms.Context(sms.Scene(desc), cfg)
    q = W.sphere_queries(48) if conductor else W.plane_queries(
        (W.pcg32_streams_f32(9, np.arange(4096, dtype=np.uint64), 2).T * 1.6 - 0.8).astype(np.float32))
    vg, cg, wg = sms.SpecularManifoldSingleScatter(ctx).specular_manifold_sampling(q, seed=3)
    vo, co, wo, _ = oracle.OracleScene(desc).connect_batch(cfg, q, seed=3)
    vf, cf, wf, _ = oracle.OracleScene(desc, fma=True).connect_batch(cfg, q, seed=3)
    g_cm, g_diff, g_med = _connect_diff(vg, cg, wg, vo, co, wo)
    f_cm, f_diff, _ = _connect_diff(vf, cf, wf, vo, co, wo)
    print(f"rough conductor={conductor} biased={biased}: count mismatch {g_cm:.4f} differs {g_diff:.4f} "
          f"(floor {f_cm:.4f}/{f_diff:.4f}) median rel {g_med:.1e} nonzero {np.mean(vo[0] > 0):.3f}")
    assert np.mean(vo[0] > 0) > 0.005                # the glossy caustic is there
    assert g_cm <= FLOOR_FACTOR * f_cm + FLOOR_SLACK
    assert g_diff <= FLOOR_FACTOR * f_diff + FLOOR_SLACK
    assert g_med < 1e-3
    ctx.close()


def test_rough_normal_mapped_chain_is_refused(sms, workloads, gpu_lib):
    """Rough chain shapes are supported (tests/test_gpu_ms_parity.py), rough
    normal-mapped chain shapes are not: SMS_ERR_UNSUPPORTED."""
    W = workloads
    d = sms.SceneDesc()
    P, N, UV, F = W.heightfield_mesh(8, 1.0, 1.3, [])
    sid = d.add_mesh(P, F, sms.Bsdf(sms.BSDF_DIELECTRIC, 1.5, alpha=0.1), sms.SHAPE_CAUSTIC_CASTER_MULTI, N=N, UV=UV)
    d.normalmap = (sid, W.nm_plane_slopes(64), 1.0)
    d.add_point_emitter((0.0, 0.0, 4.0), (40.0,) * 3, sms.EMITTER_CAUSTIC_MULTI)
    ctx = sms.Context(sms.Scene(d), sms.SMSConfig(bounces=1, biased=True, max_trials=4))
    with pytest.raises(sms.SMSError) as e:
        sms.SpecularManifoldMultiScatter(ctx).specular_manifold_sampling(W.sphere_queries(4))
    assert e.value.status == 4
    ctx.close()
