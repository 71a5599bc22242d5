"""Caustic receivers with any BSDF (manifold_ss.cpp:109, 191; manifold_ms.cpp:
113, 190: the solver evaluates the shading point's own BSDF toward the first
specular vertex).  A query names its receiver shape by row 12 = -(1 + shape
id) and carries the incident direction in the frame built from its normal;
these tests run that form through the C ABI and the path tracer against the
oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

_FAR = np.array([[-1, -1, -10], [1, -1, -10], [1, 1, -10], [-1, 1, -10]], np.float32)
_TRI = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)


def _scene(sms, workloads, receiver_bsdf):
    """The mirror sphere under a point light, plus an unflagged quad far below
    that only lends its BSDF to the queries (shape id 1)."""
    d = workloads.sphere_scene(conductor=True)
    d.add_mesh(_FAR, _TRI, receiver_bsdf)
    return d


def _tagged(q, shape, wi_xy=(0.0, 0.0)):
    t = q.copy()
    t[12] = -1.0 - shape
    t[13], t[14] = wi_xy
    return t


def test_tagged_diffuse_receiver_equals_albedo_query(sms, workloads, gpu_lib):
    """A query naming a diffuse shape gives the albedo query's estimate."""
    W = workloads
    d = _scene(sms, W, sms.Bsdf(sms.BSDF_DIFFUSE, 1.0, 0.0, (0.5, 0.5, 0.5)))
    ss = sms.SpecularManifoldSingleScatter(sms.Context(sms.Scene(d), W.sphere_config()))
    q = W.sphere_queries(32)
    va, ca, _ = ss.specular_manifold_sampling(q, seed=4)
    vt, ct, _ = ss.specular_manifold_sampling(_tagged(q, 1), seed=4)
    assert va.sum() > 0
    np.testing.assert_array_equal(ca, ct)
    np.testing.assert_allclose(vt, va, rtol=1e-5, atol=1e-7)


@pytest.mark.parametrize("kind", ["roughplastic", "roughconductor"])
def test_glossy_receiver_connections_match_oracle(sms, workloads, oracle, gpu_lib, kind):
    """Biased connections at a glossy receiver, GPU vs the oracle, with the
    camera direction tilted off the normal."""
    W = workloads
    b = (sms.Bsdf(sms.BSDF_ROUGHPLASTIC, 1.5, 0.0, (0.3, 0.5, 0.7), alpha=0.3) if kind == "roughplastic"
         else sms.Bsdf(sms.BSDF_CONDUCTOR, 0.2, 3.0, alpha=0.3))
    d = _scene(sms, W, b)
    cfg = W.sphere_config()
    q = _tagged(W.sphere_queries(32), 1, (0.6, 0.0))
    q[15] = 0.8
    ss = sms.SpecularManifoldSingleScatter(sms.Context(sms.Scene(d), cfg))
    vg, cg, _ = ss.specular_manifold_sampling(q, seed=2)
    vo, co, _ = oracle.OracleScene(d).connect_batch(cfg, q, seed=2)[:3]
    assert vo.sum() > 0
    same = (cg == co)
    assert same.mean() > 0.95
    close = np.isclose(vg[:, same], vo[:, same], rtol=2e-3, atol=1e-6).all(0)
    assert close.mean() > 0.95, close.mean()
    assert abs(vg.sum() - vo.sum()) < 0.02 * vo.sum()


def test_glossy_receiver_chains_match_oracle(sms, workloads, oracle, gpu_lib):
    """Two-bounce chains through the slab ending at a rough-conductor
    receiver (manifold_ms.cpp:113, 190), biased, GPU vs the oracle with the
    oracle's FMA build as the floor."""
    from test_gpu_ss_parity import FLOOR_FACTOR, FLOOR_SLACK, _connect_diff
    W = workloads
    d = W.slab_scene()
    rid = d.add_mesh(_FAR, _TRI, sms.Bsdf(sms.BSDF_CONDUCTOR, 0.2, 3.0, alpha=0.3))
    cfg = W.slab_config()
    q = _tagged(W.slab_queries(2048), rid, (0.0, 0.6))
    q[15] = 0.8
    ms = sms.SpecularManifoldMultiScatter(sms.Context(sms.Scene(d), cfg))
    vg, cg, wg = ms.specular_manifold_sampling(q, seed=2)
    vo, co, wo, _ = oracle.OracleScene(d).connect_batch(cfg, q, seed=2, multi=True)
    vf, cf, wf, _ = oracle.OracleScene(d, fma=True).connect_batch(cfg, q, seed=2, multi=True)
    assert vo.sum() > 0
    g_cm, g_diff, g_med = _connect_diff(vg, cg, wg, vo, co, wo)
    f_cm, f_diff, _ = _connect_diff(vf, cf, wf, vo, co, wo)
    assert g_cm <= FLOOR_FACTOR * f_cm + FLOOR_SLACK
    assert g_diff <= FLOOR_FACTOR * f_diff + FLOOR_SLACK
    assert g_med < 1e-4
    assert abs(vg.mean() - vo.mean()) <= 0.01 * vo.mean()


def test_receiver_outside_the_scene_is_an_error(sms, workloads, gpu_lib):
    W = workloads
    d = _scene(sms, W, sms.Bsdf(sms.BSDF_DIFFUSE, 1.0, 0.0, (0.5, 0.5, 0.5)))
    ctx = sms.Context(sms.Scene(d), W.sphere_config())
    ss = sms.SpecularManifoldSingleScatter(ctx)
    q = W.sphere_queries(8)
    with pytest.raises(sms.SMSError, match="receiver shape"):
        ss.specular_manifold_sampling(_tagged(q, 7), seed=1)
    # the context stays usable
    v, c, _ = ss.specular_manifold_sampling(q, seed=1)
    assert c.sum() > 0


def test_glossy_floor_render_matches_oracle(sms, workloads, oracle, gpu_lib):
    """path_sms_ss over the water with a roughplastic floor: its caustics
    take the floor's BSDF; GPU image vs the oracle's."""
    from test_gpu_render import _check_against_oracle
    W = workloads
    fb = sms.Bsdf(sms.BSDF_ROUGHPLASTIC, 1.5, 0.0, (0.4, 0.5, 0.6), alpha=0.3)
    desc = W.pool_scene(res=32, floor_bsdf=fb)
    cfg = W.water_config()
    g, o, f = _check_against_oracle(sms, oracle, desc, cfg, W.pool_camera(24, 24),
                                    sms.RenderOptions(integrator="path_sms_ss", spp=4, seed=3))
    assert o.mean() > 0.01
