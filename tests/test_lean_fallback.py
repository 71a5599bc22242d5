"""The normal map's LEAN fallback BSDF (NormalmapBSDF with lean_fallback,
src/bsdfs/normalmap.cpp:80-112, 142-170, 187-203; include/mitsuba/render/
lean.h) in the oracle's restatement: sampling, evaluation and density agree
with each other, the density integrates to the visible share of the
distribution, and sampled directions follow it.  The reference ships no test
of this BSDF, so these are consistency checks of the restatement; the GPU
path tracer is compared with it in tests/test_gpu_render.py."""
import math

import numpy as np
import pytest


@pytest.fixture(scope="module")
def fb_scene(sms, workloads, oracle):
    return oracle.OracleScene(workloads.lean_fallback_scene(map_res=64))


def _hemisphere_dirs(n, rng, min_z=0.05):
    v = rng.standard_normal((3, n))
    v /= np.linalg.norm(v, axis=0, keepdims=True)
    v[2] = np.abs(v[2])
    return v[:, v[2] > min_z]


def test_sample_weight_is_eval_over_pdf(fb_scene):
    """bs.weight = F G / G1 of a visible-normal sample equals eval / pdf of
    the sampled pair, and the sample's density equals pdf()."""
    rng = np.random.default_rng(1)
    wi = _hemisphere_dirs(4000, rng, 0.1)
    u = rng.random((2, wi.shape[1])).astype(np.float32)
    s = fb_scene.lean_fb_sample(wi, u)
    ok = s[0] > 0
    assert ok.mean() > 0.5
    wo = s[1:4, ok]
    ev = fb_scene.lean_fb_eval(wi[:, ok], wo)
    assert (ev[1] > 0).all()
    np.testing.assert_allclose(s[5, ok], ev[1], rtol=2e-3)
    np.testing.assert_allclose(s[4, ok], ev[0] / ev[1], rtol=2e-3)
    np.testing.assert_allclose(np.linalg.norm(wo, axis=0), 1.0, atol=1e-5)
    assert (wo[2] > 0).all()


@pytest.mark.parametrize("theta_deg", [5.0, 40.0, 70.0])
def test_pdf_integrates_to_at_most_one(fb_scene, theta_deg):
    """The density over the upper hemisphere (midpoint rule on a fine grid)
    is at most 1 and, away from grazing, close to 1."""
    t = math.radians(theta_deg)
    n_t, n_p = 400, 800
    th = (np.arange(n_t) + 0.5) * (0.5 * math.pi / n_t)
    ph = (np.arange(n_p) + 0.5) * (2 * math.pi / n_p)
    T, P = np.meshgrid(th, ph, indexing="ij")
    wo = np.stack([np.sin(T) * np.cos(P), np.sin(T) * np.sin(P), np.cos(T)]).reshape(3, -1)
    wi = np.repeat(np.array([[math.sin(t)], [0.0], [math.cos(t)]]), wo.shape[1], axis=1)
    pdf = fb_scene.lean_fb_eval(wi, wo)[1].reshape(n_t, n_p)
    total = float((pdf * np.sin(T)).sum() * (0.5 * math.pi / n_t) * (2 * math.pi / n_p))
    assert total <= 1.02
    if theta_deg < 60:
        assert total > 0.95, total


def test_sampled_directions_follow_the_pdf(fb_scene):
    """Histogram of sampled wo over (cos theta, phi) bins against the pdf
    integrated over each bin, for the well-populated bins."""
    rng = np.random.default_rng(5)
    t = math.radians(30.0)
    n = 200000
    wi = np.repeat(np.array([[math.sin(t)], [0.0], [math.cos(t)]]), n, axis=1)
    s = fb_scene.lean_fb_sample(wi, rng.random((2, n)).astype(np.float32))
    ok = s[0] > 0
    wo = s[1:4, ok]
    nb_c, nb_p = 24, 24
    ct = np.clip(wo[2], 0, 1 - 1e-7)
    phi = np.mod(np.arctan2(wo[1], wo[0]), 2 * math.pi)
    hist, _, _ = np.histogram2d(ct, phi, bins=[nb_c, nb_p], range=[[0, 1], [0, 2 * math.pi]])
    # expected counts: pdf integrated over each (cos theta, phi) bin
    sub = 8
    cc = (np.arange(nb_c * sub) + 0.5) / (nb_c * sub)
    pp = (np.arange(nb_p * sub) + 0.5) * (2 * math.pi / (nb_p * sub))
    C, Pp = np.meshgrid(cc, pp, indexing="ij")
    st = np.sqrt(1 - C * C)
    d = np.stack([st * np.cos(Pp), st * np.sin(Pp), C]).reshape(3, -1)
    wi2 = np.repeat(wi[:, :1], d.shape[1], axis=1)
    pdf = fb_scene.lean_fb_eval(wi2, d)[1].reshape(nb_c * sub, nb_p * sub)
    area = (1.0 / (nb_c * sub)) * (2 * math.pi / (nb_p * sub))
    expect = (pdf * area).reshape(nb_c, sub, nb_p, sub).sum(axis=(1, 3)) * n
    big = expect > 200
    assert big.sum() > 10
    rel = np.abs(hist[big] - expect[big]) / expect[big]
    assert rel.max() < 0.15, rel.max()
    assert abs(hist.sum() - n * ok.mean()) < 1


def test_fallback_needs_a_normal_map(sms, workloads):
    """sms_scene_set_lean_fallback refuses a scene without a normal map and
    parameters out of range (host-side checks, no device needed)."""
    d = workloads.sphere_scene()
    d.lean_fallback = (1e-4, 0.0, 1.0)
    with pytest.raises(sms.SMSError):
        sms.Scene(d)
    d = workloads.lean_fallback_scene(map_res=16)
    sms.Scene(d)
    d.lean_fallback = (-1.0, 0.0, 1.0)
    with pytest.raises(sms.SMSError):
        sms.Scene(d)
    d.lean_fallback = (1e-4, 0.0, 0.0)
    with pytest.raises(sms.SMSError):
        sms.Scene(d)
