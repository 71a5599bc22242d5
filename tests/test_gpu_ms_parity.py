"""GPU multi-scatter parity against the oracle (manifold_ms.cpp), through the
C ABI.  Tolerances as in test_gpu_ss_parity: mismatches may not exceed 1.5x the
oracle-vs-FMA-oracle floor + 0.5%; positions of walks both sides solved to the
same solution agree to 1e-5 (median) at scene scale 1."""
import numpy as np
import pytest

from test_gpu_ss_parity import FLOOR_FACTOR, FLOOR_SLACK, _connect_diff

pytestmark = pytest.mark.gpu


def _ms_walk_diff(a, b, tol=1e-4):
    oka, okb = a[0] > 0.5, b[0] > 0.5
    both = oka & okb
    d = np.maximum(np.linalg.norm(a[2:5, both] - b[2:5, both], axis=0),
                   np.linalg.norm(a[5:8, both] - b[5:8, both], axis=0))
    same = d < tol
    return (float(np.mean(oka != okb)), float(np.sum(~same)) / len(oka),
            float(np.median(d[same])) if same.any() else 0.0, int(both.sum()))


@pytest.mark.parametrize("halfvector", [False, True])
def test_slab_walks(sms, workloads, oracle, gpu_lib, halfvector):
    W = workloads
    desc = W.slab_scene()
    cfg = sms.SMSConfig(bounces=2, max_iterations=30, halfvector_constraints=halfvector)
    ctx = sms.Context(sms.Scene(desc), cfg)
    ms = sms.SpecularManifoldMultiScatter(ctx)
    n = 8192
    q = W.slab_queries(n)
    u = W.pcg32_streams_f32(11, np.arange(n, dtype=np.uint64), 2)
    w = np.zeros((8, n), np.float32)
    w[2] = 5.0
    w[6], w[7] = u[0], u[1]
    out_g = ms.sample_path(0, q, w)
    out_o = oracle.OracleScene(desc).ms_walk_batch(cfg, 0, q, w)
    out_f = oracle.OracleScene(desc, fma=True).ms_walk_batch(cfg, 0, q, w)
    g_m, g_c, g_med, nboth = _ms_walk_diff(out_g, out_o)
    f_m, f_c, _, _ = _ms_walk_diff(out_f, out_o)
    print(f"slab walks halfvector={halfvector}: gpu mismatch {g_m:.4f} crossed {g_c:.4f} (floor {f_m:.4f}/{f_c:.4f}) "
          f"median|dp| {g_med:.1e} both {nboth}")
    assert nboth > n // 4
    assert np.mean(out_g[8] != out_o[8]) < 0.005          # seed paths
    assert g_m <= FLOOR_FACTOR * f_m + FLOOR_SLACK
    assert g_c <= FLOOR_FACTOR * f_c + FLOOR_SLACK
    assert g_med < 1e-5


@pytest.mark.parametrize("biased", [True, False])
def test_slab_connect(sms, workloads, oracle, gpu_lib, biased):
    W = workloads
    desc = W.slab_scene()
    cfg = W.slab_config() if biased else sms.SMSConfig(bounces=2, max_iterations=30, max_trials=64)
    ctx = sms.Context(sms.Scene(desc), cfg)
    ms = sms.SpecularManifoldMultiScatter(ctx)
    n = 4096 if biased else 8192
    q = W.slab_queries(n)
    vg, cg, wg = ms.specular_manifold_sampling(q, seed=2)
    vo, co, wo, st_o = oracle.OracleScene(desc).connect_batch(cfg, q, seed=2, multi=True)
    vf, cf, wf, _ = oracle.OracleScene(desc, fma=True).connect_batch(cfg, q, seed=2, multi=True)
    g_cm, g_diff, g_med = _connect_diff(vg, cg, wg, vo, co, wo)
    f_cm, f_diff, _ = _connect_diff(vf, cf, wf, vo, co, wo)
    print(f"slab {'biased' if biased else 'unbiased'}: count mismatch {g_cm:.4f} differs {g_diff:.4f} "
          f"(floor {f_cm:.4f}/{f_diff:.4f}) median rel {g_med:.1e}")
    assert g_cm <= FLOOR_FACTOR * f_cm + FLOOR_SLACK
    assert g_diff <= FLOOR_FACTOR * f_diff + FLOOR_SLACK
    assert g_med < 1e-4
    st = ctx.stats()
    assert st["connections"] == n
    if biased:
        assert np.all(wg == 32) and st["walks"] == st_o["walks"] == 32 * n
        assert abs(vg.mean() - vo.mean()) <= 0.01 * vo.mean()
    else:
        assert np.all(wg[cg > 0] == 1 + cg[cg > 0]) and np.all(wg[cg == 0] == 1)


def test_slab_full_size_invariants(sms, workloads, gpu_lib):
    """512k queries (the benchmark size of the two-bounce configuration)."""
    W = workloads
    cfg = W.slab_config()
    ctx = sms.Context(sms.Scene(W.slab_scene()), cfg)
    ms = sms.SpecularManifoldMultiScatter(ctx)
    n = 512 * 1024
    v, c, w = ms.specular_manifold_sampling(W.slab_queries(n), seed=1)
    st = ctx.stats()
    assert np.isfinite(v).all() and (v >= 0).all()
    assert np.all(w == 32) and np.all((c >= 0) & (c <= 32))
    assert np.all(v[:, c == 0] == 0)
    assert st["walks"] == 32 * n and st["solver_succeeded"] + st["solver_failed"] == 32 * n
    assert (c > 0).mean() > 0.9


def test_ms_bounce_validation(sms, workloads, gpu_lib):
    W = workloads
    ctx = sms.Context(sms.Scene(W.slab_scene(res=16)), sms.SMSConfig(bounces=5))
    ms = sms.SpecularManifoldMultiScatter(ctx)
    with pytest.raises(sms.SMSError) as e:
        ms.specular_manifold_sampling(W.slab_queries(4))
    assert e.value.status == 4


def test_slab_mnee_init_walks(sms, workloads, oracle, gpu_lib):
    """MNEE seed paths through the slab (manifold_ms.cpp:305-316, 377-397):
    straight line toward the light, no scattering at the seed vertices."""
    W = workloads
    desc = W.slab_scene(res=128)
    cfg = sms.SMSConfig(bounces=2, max_iterations=30, mnee_init=True)
    ctx = sms.Context(sms.Scene(desc), cfg)
    n = 4096
    q = W.slab_queries(n)
    u = W.pcg32_streams_f32(12, np.arange(n, dtype=np.uint64), 2)
    w = np.zeros((8, n), np.float32)
    w[2] = 5.0
    w[6], w[7] = u[0], u[1]
    out_g = sms.SpecularManifoldMultiScatter(ctx).sample_path(0, q, w)
    out_o = oracle.OracleScene(desc).ms_walk_batch(cfg, 0, q, w)
    out_f = oracle.OracleScene(desc, fma=True).ms_walk_batch(cfg, 0, q, w)
    g_m, g_c, g_med, nboth = _ms_walk_diff(out_g, out_o)
    f_m, f_c, _, _ = _ms_walk_diff(out_f, out_o)
    print(f"slab mnee walks: gpu mismatch {g_m:.4f} (floor {f_m:.4f}) both {nboth}")
    assert nboth > n // 4
    assert g_m <= FLOOR_FACTOR * f_m + FLOOR_SLACK and g_c <= FLOOR_FACTOR * f_c + FLOOR_SLACK


@pytest.mark.parametrize("biased", [True, False])
def test_rough_slab_connect(sms, workloads, oracle, gpu_lib, biased):
    """Rough chain shapes (manifold_ms.cpp:356-375): the first complete seed
    path samples a Beckmann offset normal at every rough vertex, later walks
    scatter about those offsets and must hit the same shapes, the Newton steps
    solve the offset constraints (:618-621, :707-717) and the estimate is
    divided by the offsets' density (:198).  Both slab faces rough (alpha 0.1);
    GPU vs oracle on the same random streams, against the oracle-vs-FMA floor."""
    W = workloads
    desc = W.slab_scene(alpha=0.1)
    cfg = W.slab_config() if biased else sms.SMSConfig(bounces=2, max_iterations=30, max_trials=64)
    ctx = sms.Context(sms.Scene(desc), cfg)
    ms = sms.SpecularManifoldMultiScatter(ctx)
    n = 4096 if biased else 8192
    q = W.slab_queries(n)
    vg, cg, wg = ms.specular_manifold_sampling(q, seed=2)
    vo, co, wo, st_o = oracle.OracleScene(desc).connect_batch(cfg, q, seed=2, multi=True)
    vf, cf, wf, _ = oracle.OracleScene(desc, fma=True).connect_batch(cfg, q, seed=2, multi=True)
    g_cm, g_diff, g_med = _connect_diff(vg, cg, wg, vo, co, wo)
    f_cm, f_diff, _ = _connect_diff(vf, cf, wf, vo, co, wo)
    print(f"rough slab {'biased' if biased else 'unbiased'}: count mismatch {g_cm:.4f} differs {g_diff:.4f} "
          f"(floor {f_cm:.4f}/{f_diff:.4f}) median rel {g_med:.1e} nonzero {np.mean(vo[0] > 0):.3f}")
    assert np.mean(vo[0] > 0) > 0.3
    assert g_cm <= FLOOR_FACTOR * f_cm + FLOOR_SLACK
    assert g_diff <= FLOOR_FACTOR * f_diff + FLOOR_SLACK
    assert g_med < 1e-4
    st = ctx.stats()
    assert st["connections"] == n and st["walks"] == wg.sum()
    if biased:
        assert np.all(wg == cfg.max_trials)
    ctx.close()
