"""The roughplastic BSDF (src/bsdfs/roughplastic.cpp): a rough Beckmann
dielectric coating over a diffuse base.  The oracle's precomputed coating
terms (eval_transmittance / eval_reflectance, include/mitsuba/render/
microfacet.h:454-551, by visible-normal sampling at Gauss-Legendre nodes) are
pinned against a direct numerical integral written here; sampling, evaluation
and density agree with each other; the GPU path tracer is compared with the
oracle in tests/test_gpu_render.py."""
import math

import numpy as np
import pytest


def _roughplastic(sms, alpha=0.1, eta=1.49 / 1.000277, albedo=(0.5, 0.5, 0.5), nonlinear=False):
    return sms.Bsdf(sms.BSDF_ROUGHPLASTIC, eta, 0.0, albedo, alpha=alpha, nonlinear=nonlinear)


def _oracle_plane(sms, workloads, oracle, bsdf):
    d, cam = workloads.plane_light_scene(below=False, twosided=False, bsdf=bsdf)
    return oracle.OracleScene(d), d, cam


# ---- a direct integral of the coating terms over the microfacet normals

def _g1(v, m, alpha):
    """Smith G1 of the isotropic Beckmann distribution (microfacet.h:331-355,
    the rational approximation of Walter et al. 2007)"""
    xy = alpha * alpha * (v[0] ** 2 + v[1] ** 2)
    with np.errstate(divide="ignore", invalid="ignore"):
        a = np.where(xy > 0, 1.0 / np.sqrt(xy / (v[2] ** 2)), np.inf)
        r = np.where(a >= 1.6, 1.0, (3.535 * a + 2.181 * a * a) / (1.0 + 2.276 * a + 2.577 * a * a))
    return np.where((v * m).sum(0) * v[2] <= 0, 0.0, r)


def _fresnel(ci, eta):
    """Unpolarised dielectric Fresnel reflectance and cos theta_t (fresnel.h)"""
    outside = ci >= 0
    eta_it = np.where(outside, eta, 1.0 / eta)
    eta_ti = 1.0 / eta_it
    ct2 = 1.0 - (1.0 - ci * ci) * eta_ti * eta_ti
    ct = np.sqrt(np.maximum(ct2, 0.0))
    c = np.abs(ci)
    a_s = (c - eta_it * ct) / (c + eta_it * ct)
    a_p = (ct - eta_it * c) / (ct + eta_it * c)
    r = np.where(ct2 <= 0, 1.0, 0.5 * (a_s ** 2 + a_p ** 2))
    return r, np.where(outside, -ct, ct), eta_ti


def _coating_integral(alpha, eta, mu, transmit):
    """E over visible normals m of wi of G1(wo, m) (1 - F) (refraction) or
    G1(wo, m) F (reflection); theta_m by Gauss-Legendre, phi by midpoints"""
    wi = np.array([math.sqrt(1 - mu * mu), 0.0, mu])[:, None]
    x, w = np.polynomial.legendre.leggauss(200)
    tmax = math.atan(7.0 * alpha)
    th = 0.5 * tmax * (x + 1)
    wth = 0.5 * tmax * w
    n_phi = 256
    ph = 2 * math.pi * (np.arange(n_phi) + 0.5) / n_phi
    T, P = np.meshgrid(th, ph, indexing="ij")
    W = np.meshgrid(wth, ph, indexing="ij")[0] * (2 * math.pi / n_phi)
    st, ct = np.sin(T).ravel(), np.cos(T).ravel()
    m = np.stack([st * np.cos(P).ravel(), st * np.sin(P).ravel(), ct])
    D = np.exp(-(np.tan(T).ravel() ** 2) / alpha ** 2) / (math.pi * alpha ** 2 * ct ** 4)
    dm = (wi * m).sum(0)
    dvis = np.where(dm > 0, _g1(wi, m, alpha) * dm * D / mu, 0.0)
    F, cos_t, eta_ti = _fresnel(dm, eta)
    if transmit:
        wo = m * (dm * eta_ti + cos_t) - wi * eta_ti
        g = np.where(wo[2] * wi[2] >= 0, 0.0, _g1(wo, m, alpha) * (1 - F))
    else:
        wo = 2 * dm * m - wi
        g = np.where(wo[2] <= 0, 0.0, _g1(wo, m, alpha) * F)
    return float((dvis * g * st * W.ravel()).sum())


@pytest.mark.parametrize("alpha", [0.1, 0.3])
def test_tables_match_direct_integral(sms, workloads, oracle, alpha):
    """The external transmittance at 64 cosines, the internal diffuse
    reflectance 2 mean(mu R(mu, 1/eta)) and the specular sampling weight
    1 / (mean(diffuse) + 1) (roughplastic.cpp:364-396)."""
    eta = 1.49 / 1.000277
    O, _, _ = _oracle_plane(sms, workloads, oracle, _roughplastic(sms, alpha, eta, albedo=(0.2, 0.5, 0.8)))
    tab = O.roughplastic_tables(0)
    mus = [max(1e-6, i / 63) for i in range(64)]
    for i in (1, 5, 16, 32, 48, 63):
        ref = _coating_integral(alpha, eta, mus[i], True)
        assert abs(tab[i] - ref) < 4e-3, (i, tab[i], ref)
    assert 0.0 <= tab[0] < tab[63] < 1.0
    ref_r = [_coating_integral(alpha, 1.0 / eta, mu, False) * mu for mu in mus]
    fdr = 2.0 * float(np.mean(ref_r))
    assert abs(tab[64] - fdr) < 4e-3, (tab[64], fdr)
    assert 0.4 < tab[64] < 0.7
    assert tab[65] == pytest.approx(1.0 / (0.5 + 1.0), rel=1e-6)


def _hemisphere_dirs(n, rng, min_z=0.05):
    v = rng.standard_normal((3, n))
    v /= np.linalg.norm(v, axis=0, keepdims=True)
    v[2] = np.abs(v[2])
    return v[:, v[2] > min_z]


@pytest.mark.parametrize("alpha", [0.05, 0.3])
def test_sample_weight_is_eval_over_pdf(sms, workloads, oracle, alpha):
    """The sampled direction's weight is eval / pdf of the pair and its
    density equals pdf(); both lobes are drawn."""
    O, _, _ = _oracle_plane(sms, workloads, oracle, _roughplastic(sms, alpha))
    rng = np.random.default_rng(3)
    wi = _hemisphere_dirs(4000, rng, 0.1)
    u = rng.random((3, wi.shape[1])).astype(np.float32)
    s = O.shape_bsdf_sample(0, wi, u)
    ok = s[0] > 0
    assert ok.mean() > 0.8
    wo = s[1:4, ok]
    ev = O.shape_bsdf_eval(0, wi[:, ok], wo)
    np.testing.assert_allclose(s[7, ok], ev[3], rtol=2e-3)
    np.testing.assert_allclose(s[4:7, ok], ev[0:3] / ev[3], rtol=2e-3)
    assert (wo[2] > 0).all()
    # below the surface: no sample, zero value and density
    s = O.shape_bsdf_sample(0, -wi[:, :10], u[:, :10])
    assert not s[0].any()
    assert not O.shape_bsdf_eval(0, wi[:, :10], -wi[:, :10]).any()


def _sphere_grid(theta_deg, n_t=300, n_p=600):
    t = math.radians(theta_deg)
    th = (np.arange(n_t) + 0.5) * (0.5 * math.pi / n_t)
    ph = (np.arange(n_p) + 0.5) * (2 * math.pi / n_p)
    T, P = np.meshgrid(th, ph, indexing="ij")
    wo = np.stack([np.sin(T) * np.cos(P), np.sin(T) * np.sin(P), np.cos(T)]).reshape(3, -1)
    wi = np.repeat(np.array([[math.sin(t)], [0.0], [math.cos(t)]]), wo.shape[1], axis=1)
    dw = (np.sin(T) * (0.5 * math.pi / n_t) * (2 * math.pi / n_p)).ravel()
    return wi, wo, dw


@pytest.mark.parametrize("theta_deg", [10.0, 45.0, 70.0])
def test_pdf_integrates_to_one_and_energy_is_conserved(sms, workloads, oracle, theta_deg):
    """The density over the upper hemisphere is at most 1 (close to 1 away
    from grazing), and a white base reflects at most what arrives."""
    O, _, _ = _oracle_plane(sms, workloads, oracle, _roughplastic(sms, 0.2, albedo=(1.0, 1.0, 1.0)))
    wi, wo, dw = _sphere_grid(theta_deg)
    ev = O.shape_bsdf_eval(0, wi, wo)
    pdf_total = float((ev[3] * dw).sum())
    albedo = float((ev[0] * dw).sum())
    assert pdf_total <= 1.02
    assert albedo <= 1.03
    if theta_deg < 60:
        assert pdf_total > 0.95, pdf_total
        assert albedo > 0.85, albedo


def test_nonlinear_internal_scattering(sms, workloads, oracle):
    """nonlinear divides the base's albedo by 1 - albedo Fdr instead of
    1 - Fdr (roughplastic.cpp:288-291): away from the coating's lobe the
    ratio of the two is (1 - Fdr) / (1 - albedo Fdr) per channel."""
    albedo = (0.1, 0.5, 0.9)
    lin, _, _ = _oracle_plane(sms, workloads, oracle, _roughplastic(sms, 0.05, albedo=albedo))
    nl, _, _ = _oracle_plane(sms, workloads, oracle, _roughplastic(sms, 0.05, albedo=albedo, nonlinear=True))
    fdr = lin.roughplastic_tables(0)[64]
    wi = np.array([[0.5], [0.0], [math.sqrt(0.75)]])
    wo = np.array([[-0.1], [0.6], [math.sqrt(1 - 0.37)]])
    a, b = lin.shape_bsdf_eval(0, wi, wo)[:3, 0], nl.shape_bsdf_eval(0, wi, wo)[:3, 0]
    np.testing.assert_allclose(b / a, [(1 - fdr) / (1 - x * fdr) for x in albedo], rtol=1e-4)


def test_oracle_render_shows_coating_highlight(sms, workloads, oracle):
    """A black base leaves only the coating: the light's glossy highlight on
    the plane; a white base adds the diffuse light everywhere."""
    cfg = sms.SMSConfig()
    opt = sms.RenderOptions(integrator="path", spp=32, seed=5)
    O, _, cam = _oracle_plane(sms, workloads, oracle, _roughplastic(sms, 0.1, albedo=(0.0, 0.0, 0.0)))
    coat = O.render(cfg, cam, opt)
    O, _, cam = _oracle_plane(sms, workloads, oracle, _roughplastic(sms, 0.1, albedo=(0.8, 0.8, 0.8)))
    full = O.render(cfg, cam, opt)
    assert coat.max() > 0.1
    assert (coat[..., 0] > 1e-4).mean() < 0.5
    assert full.mean() > 2.0 * coat.mean()
    assert (full[..., 0] > 1e-4).mean() > 0.9


def test_library_refuses_bad_parameters(sms):
    """int_ior equal to ext_ior and a smooth coating are refused."""
    for b in (_roughplastic(sms, 0.1, eta=1.0), _roughplastic(sms, 0.0)):
        d = sms.SceneDesc()
        d.add_sphere((0, 0, 0), 1.0, b)
        with pytest.raises(sms.SMSError):
            sms.Scene(d)
    d = sms.SceneDesc()
    d.add_sphere((0, 0, 0), 1.0, _roughplastic(sms))
    sms.Scene(d)
