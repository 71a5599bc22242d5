"""GPU glint parity against the oracle (manifold_glints.cpp), through the C
ABI.  Same floor-relative tolerances as the other parity tests; converged uv
positions of walks that agree match to 1e-6 (median, uv units)."""
import numpy as np
import pytest

from test_gpu_ss_parity import FLOOR_FACTOR, FLOOR_SLACK, _connect_diff

pytestmark = pytest.mark.gpu

_SLOPES = {}


def _slopes(W, res):
    if res not in _SLOPES:
        _SLOPES[res] = W.glint_slopes(res)
    return _SLOPES[res]


def _glint_walk_diff(a, b, tol=1e-4):
    oka, okb = a[0] > 0.5, b[0] > 0.5
    both = oka & okb
    d = np.linalg.norm(a[2:4, both] - b[2:4, both], axis=0)
    same = d < tol
    return (float(np.mean(oka != okb)), float(np.sum(~same)) / len(oka),
            float(np.median(d[same])) if same.any() else 0.0, int(both.sum()))


def test_glint_walks(sms, workloads, oracle, gpu_lib):
    W = workloads
    desc = W.glint_scene(slopes=_slopes(W, 1024))
    cfg = W.glint_config()
    ctx = sms.Context(sms.Scene(desc), cfg)
    gl = sms.SpecularManifoldGlints(ctx)
    q = W.glint_queries(128)
    n = q.shape[1]
    _, light = W.glint_camera()
    u = W.pcg32_streams_f32(5, np.arange(n, dtype=np.uint64), 2)
    w = np.zeros((5, n), np.float32)
    w[0:3] = np.asarray(light, np.float32)[:, None]
    w[3], w[4] = u[0], u[1]
    out_g = gl.sample_glint(q, w)
    out_o = oracle.OracleScene(desc).glint_walk_batch(cfg, q, w)
    out_f = oracle.OracleScene(desc, fma=True).glint_walk_batch(cfg, q, w)
    g_m, g_c, g_med, nboth = _glint_walk_diff(out_g, out_o)
    f_m, f_c, _, _ = _glint_walk_diff(out_f, out_o)
    print(f"glint walks: gpu mismatch {g_m:.4f} crossed {g_c:.4f} (floor {f_m:.4f}/{f_c:.4f}) "
          f"median|duv| {g_med:.1e} both {nboth}")
    assert nboth > 20
    assert g_m <= FLOOR_FACTOR * f_m + FLOOR_SLACK
    assert g_c <= FLOOR_FACTOR * f_c + FLOOR_SLACK
    assert g_med < 1e-6
    assert np.abs(out_g[4:6] - out_o[4:6]).max() < 1e-6   # seeds


@pytest.mark.parametrize("biased", [True, False])
def test_glint_connect(sms, workloads, oracle, gpu_lib, biased):
    W = workloads
    desc = W.glint_scene(slopes=_slopes(W, 1024))
    cfg = W.glint_config() if biased else sms.SMSConfig(max_iterations=10, max_trials=64)
    ctx = sms.Context(sms.Scene(desc), cfg)
    gl = sms.SpecularManifoldGlints(ctx)
    q = W.glint_queries(256)
    vg, cg, wg = gl.specular_manifold_sampling(q, seed=3)
    vo, co, wo, st_o = oracle.OracleScene(desc).connect_batch(cfg, q, seed=3, glints=True)
    vf, cf, wf, _ = oracle.OracleScene(desc, fma=True).connect_batch(cfg, q, seed=3, glints=True)
    g_cm, g_diff, g_med = _connect_diff(vg, cg, wg, vo, co, wo)
    f_cm, f_diff, _ = _connect_diff(vf, cf, wf, vo, co, wo)
    print(f"glints {'biased' if biased else 'unbiased'}: count mismatch {g_cm:.4f} differs {g_diff:.4f} "
          f"(floor {f_cm:.4f}/{f_diff:.4f}) median rel {g_med:.1e} nonzero {(vo[0] > 0).mean():.3f}")
    assert (co != 0).sum() > 50
    assert g_cm <= FLOOR_FACTOR * f_cm + FLOOR_SLACK
    assert g_diff <= FLOOR_FACTOR * f_diff + FLOOR_SLACK
    assert g_med < 1e-4
    st = ctx.stats()
    assert st["connections"] == st_o["connections"]


def test_glint_full_size(sms, workloads, gpu_lib):
    """The benchmark configuration: 8192^2 FP16 slope map, 1024^2 camera, 64
    seeds, 10 iterations, biased (vectorized) estimator."""
    W = workloads
    cfg = W.glint_config()
    ctx = sms.Context(sms.Scene(W.glint_scene(slopes=_slopes(W, 8192))), cfg)
    gl = sms.SpecularManifoldGlints(ctx)
    q = W.glint_queries(1024)
    v, c, w = gl.specular_manifold_sampling(q, seed=1)
    st = ctx.stats()
    assert np.isfinite(v).all() and (v >= 0).all()
    assert np.all((w == 64) | (w == 0)) and np.all((c >= 0) & (c <= 64))
    assert np.all(v[:, c == 0] == 0)
    assert st["walks"] == w.sum() and st["connections"] == q.shape[1]
    assert (c > 0).mean() > 0.01


@pytest.mark.parametrize("biased", [True, False])
def test_rough_glint_connect(sms, workloads, oracle, gpu_lib, biased):
    """Rough glinty surface (manifold_glints.cpp:56-64, :141, :383-393): a
    visible-normal Beckmann offset drawn after the emitter sample shifts the
    target slope, the glossy BSDF value of the normal-mapped rough conductor
    replaces the Fresnel factor, and the estimate is divided by the offset's
    density.  GPU vs oracle on the same random streams, against the
    oracle-vs-FMA floor; the offsets' inverse error function differs in the
    last bits between the two (CUDA's erfinvf, the oracle's own)."""
    W = workloads
    desc = W.glint_scene(slopes=_slopes(W, 1024), alpha=0.05)
    cfg = W.glint_config() if biased else sms.SMSConfig(max_iterations=10, max_trials=64)
    ctx = sms.Context(sms.Scene(desc), cfg)
    gl = sms.SpecularManifoldGlints(ctx)
    q = W.glint_queries(256)
    vg, cg, wg = gl.specular_manifold_sampling(q, seed=3)
    vo, co, wo, st_o = oracle.OracleScene(desc).connect_batch(cfg, q, seed=3, glints=True)
    vf, cf, wf, _ = oracle.OracleScene(desc, fma=True).connect_batch(cfg, q, seed=3, glints=True)
    g_cm, g_diff, g_med = _connect_diff(vg, cg, wg, vo, co, wo)
    f_cm, f_diff, _ = _connect_diff(vf, cf, wf, vo, co, wo)
    print(f"rough glints {'biased' if biased else 'unbiased'}: count mismatch {g_cm:.4f} differs {g_diff:.4f} "
          f"(floor {f_cm:.4f}/{f_diff:.4f}) median rel {g_med:.1e} nonzero {(vo[0] > 0).mean():.3f}")
    assert (co != 0).sum() > 50
    assert g_cm <= FLOOR_FACTOR * f_cm + FLOOR_SLACK
    assert g_diff <= FLOOR_FACTOR * f_diff + FLOOR_SLACK
    assert g_med < 1e-3
    st = ctx.stats()
    assert st["connections"] == st_o["connections"] and st["walks"] == wg.sum()
    ctx.close()
