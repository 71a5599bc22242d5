"""CPU checks of the path-tracer restatement in the oracle (the checker of the
library's sms_render): integrator identities, unbiasedness of path_sms_ss
against plain path tracing on a scene where SMS finds every solution, and the
camera convention."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def O():
    from oracle import oracle
    return oracle


def _blocks(img, b):
    h, w = img.shape[:2]
    return img[..., 0].reshape(h // b, b, w // b, b).mean(axis=(1, 3))


def test_look_at_convention(sms):
    """Camera space x left, y up, z forward (the reference's look_at)."""
    cam = sms.Camera.look_at((1.0, 2.0, 3.0), (1.0, 2.0, 0.0), (0.0, 1.0, 0.0))
    M = cam.to_world
    assert np.allclose(M[:3, 3], [1, 2, 3])
    assert np.allclose(M[:3, 2], [0, 0, -1])          # forward
    assert np.allclose(M[:3, 1], [0, 1, 0])           # up
    assert np.allclose(M[:3, 0], [-1, 0, 0])          # left = up x forward


def test_unflagged_scene_sms_integrator_equals_path(sms, workloads, O):
    """Without caustic flags path_sms_ss never calls SMS and filters nothing;
    with disable_reflected_emitters it also skips the first-bounce emitter
    sample on delta BSDFs (path_sms_ss.cpp:150-151), so it draws the same
    random numbers as path and gives the same image."""
    W = workloads
    d = sms.SceneDesc()
    fl = np.array([[-2, -2, 0], [2, -2, 0], [2, 2, 0], [-2, 2, 0]], np.float32)
    d.add_mesh(fl, np.array([[0, 1, 2], [0, 2, 3]], np.uint32), sms.Bsdf(sms.BSDF_DIFFUSE, 1.0, 0.0, (0.5,) * 3))
    P, N, UV, F = W.heightfield_mesh(16, 1.0, 1.0, W.water_params())
    d.add_mesh(P, F, sms.Bsdf(sms.BSDF_DIELECTRIC, 1.33), 0, N=N, UV=UV)
    light = d.add_sphere((0.0, 0.0, 4.0), 0.5, sms.Bsdf(sms.BSDF_DIFFUSE, 1.0, 0.0, (0.0, 0.0, 0.0)), 0)
    d.add_area_emitter(light, (40.0,) * 3, 0)
    osc = O.OracleScene(d)
    cam = W.pool_camera(8, 8)
    a = osc.render(W.water_config(), cam, sms.RenderOptions(integrator="path", spp=4, seed=3, rr_depth=100))
    b = osc.render(W.water_config(), cam, sms.RenderOptions(integrator="path_sms_ss", spp=4, seed=3, rr_depth=100,
                                                            disable_reflected_emitters=True))
    assert np.array_equal(a, b)
    assert a.mean() > 0.0


@pytest.mark.parametrize("floor", ["diffuse", "roughplastic", "roughconductor"])
def test_path_sms_ss_matches_path_on_flat_water(sms, workloads, O, floor):
    """Flat water: SMS finds the one refraction solution of every receiver
    point, so path_sms_ss (unbiased) and plain path tracing estimate the same
    image; compare 3x3-pixel blocks against the sample spread of 4 runs.  A
    glossy floor evaluates its own BSDF toward the caster
    (manifold_ss.cpp:109, 191)."""
    W = workloads
    fb = {"diffuse": None,
          "roughplastic": sms.Bsdf(sms.BSDF_ROUGHPLASTIC, 1.5, 0.0, (0.4, 0.5, 0.6), alpha=0.3),
          "roughconductor": sms.Bsdf(sms.BSDF_CONDUCTOR, 0.2, 3.0, alpha=0.4)}[floor]
    osc = O.OracleScene(W.pool_scene(res=16, wave_scale=0.0, floor_bsdf=fb))
    cam = W.pool_camera(12, 12)
    cfg = W.water_config()
    cfg.max_trials = -1
    runs = {}
    for integ, spp in (("path", 2048), ("path_sms_ss", 256)):
        runs[integ] = np.stack([_blocks(osc.render(cfg, cam, sms.RenderOptions(integrator=integ, spp=spp,
                                                                                seed=50 + r)), 3)
                                for r in range(4)])
    a, b = runs["path"], runs["path_sms_ss"]
    se = np.sqrt(a.var(0, ddof=1) / 4 + b.var(0, ddof=1) / 4)
    diff = np.abs(a.mean(0) - b.mean(0))
    assert np.all(diff < 5.0 * se + 0.01 * a.mean(0) + 1e-3), (a.mean(0), b.mean(0), se)
    assert abs(a.mean() - b.mean()) < 0.03 * a.mean()


def test_sms_seed_matches_library(sms, O):
    """The oracle and the library derive the SMS state seed alike
    (SplitMix64); checked through the library's exported function."""
    def splitmix(seed):
        m = (1 << 64) - 1
        z = (seed + 0x9E3779B97F4A7C15) & m
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & m
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & m
        return z ^ (z >> 31)
    for seed in (0, 7, 123456789, (1 << 64) - 1):
        assert sms.sms_render_seed(seed) == splitmix(seed)


def _rough_sheet_scene(sms, W, bsdf):
    d = sms.SceneDesc()
    fl = np.array([[-2, -2, 0], [2, -2, 0], [2, 2, 0], [-2, 2, 0]], np.float32)
    d.add_mesh(fl, np.array([[0, 1, 2], [0, 2, 3]], np.uint32), sms.Bsdf(sms.BSDF_DIFFUSE, 1.0, 0.0, (0.5,) * 3),
               sms.SHAPE_CAUSTIC_RECEIVER, UV=np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32))
    P, N, UV, F = W.heightfield_mesh(16, 1.0, 1.3, [])
    d.add_mesh(P, F, bsdf, sms.SHAPE_CAUSTIC_CASTER_SINGLE, N=N, UV=UV)
    d.add_point_emitter((0.3, 0.2, 4.0), (40.0,) * 3, sms.EMITTER_CAUSTIC_SINGLE)
    return d


@pytest.mark.parametrize("alpha", [0.2, 0.5])
def test_rough_sms_matches_path_tracing(sms, workloads, O, alpha):
    """Glossy caustic through a rough dielectric sheet (Beckmann alpha) from a
    point light: path_sms_ss integrates the offset normal (manifold_ss.cpp:
    60-70, divided by its density, :199) where plain path tracing reaches the
    light by emitter sampling at the rough vertex; the two estimates agree.
    The camera sits under the sheet so every light path crosses it."""
    W = workloads
    d = _rough_sheet_scene(sms, W, sms.Bsdf(sms.BSDF_DIELECTRIC, 1.5, alpha=alpha))
    osc = O.OracleScene(d)
    cfg = sms.SMSConfig(biased=False, max_trials=-1, halfvector_constraints=True)
    cam = sms.Camera.look_at((0.0, 0.0, 0.9), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 60.0, 8, 8)
    means = {}
    for integ, spp in (("path", 8192), ("path_sms_ss", 256)):
        m = [osc.render(cfg, cam, sms.RenderOptions(integrator=integ, spp=spp, seed=60 + r, max_depth=4)).mean()
             for r in range(4)]
        means[integ] = (np.mean(m), np.std(m, ddof=1) / 2)
    (a, sa), (b, sb) = means["path"], means["path_sms_ss"]
    assert abs(a - b) < 4.0 * np.hypot(sa, sb) + 0.01 * a, means


def test_glint_lean_density_is_normalised(sms, workloads, O):
    """The LEAN density of the glints integrator's MIS (manifold_glints.cpp:
    557-579: the LEAN visible-normal density mapped to reflected directions)
    integrates to ~1 over the hemisphere: Monte Carlo over uniform directions."""
    osc = O.OracleScene(workloads.glint_scene(map_res=256))
    rng = np.random.default_rng(0)
    for theta in (0.3, 0.9):
        wi = np.array([np.sin(theta), 0.0, np.cos(theta)], np.float32)
        tot = 0.0
        n = 6000
        for _ in range(n):
            z, ph = rng.random(), 2 * np.pi * rng.random()
            r = np.sqrt(1 - z * z)
            wo = np.array([r * np.cos(ph), r * np.sin(ph), z], np.float32)
            tot += osc.glint_lean_pdf(0.3, 0.6, [0.05, 0.0, 0.0, 0.05], wi, wo)
        assert abs(2 * np.pi * tot / n - 1.0) < 0.12


def test_glints_integrator_oracle(sms, workloads, O):
    """path_sms_glints on the glint plane: finite, sparse positive glints, and
    the same image for a repeated seed; the BSDF-strategy-only and
    SMS-strategy-only switches split the estimate (a point light: the BSDF
    strategy cannot reach it, so it contributes nothing)."""
    W = workloads
    desc = W.glint_scene(map_res=256)
    osc = O.OracleScene(desc)
    cam = W.glint_render_camera(24, 24)
    opt = sms.RenderOptions(integrator="path_sms_glints", spp=4, seed=3)
    a = osc.render(W.glint_config(), cam, opt)
    b = osc.render(W.glint_config(), cam, opt)
    assert np.isfinite(a).all() and np.array_equal(a, b)
    assert 0.005 < (a[..., 0] > 0).mean() < 0.5
    cfg = W.glint_config()
    cfg.bsdf_strategy_only = True
    c = osc.render(cfg, cam, opt)
    assert c.max() == 0.0


def test_filtered_integrators_without_flags_equal_path(sms, workloads, O):
    """Without caustic flags the filtered path tracers filter nothing and draw
    the same random numbers as path: the same image."""
    W = workloads
    d = sms.SceneDesc()
    fl = np.array([[-2, -2, 0], [2, -2, 0], [2, 2, 0], [-2, 2, 0]], np.float32)
    d.add_mesh(fl, np.array([[0, 1, 2], [0, 2, 3]], np.uint32), sms.Bsdf(sms.BSDF_DIFFUSE, 1.0, 0.0, (0.5,) * 3))
    P, N, UV, F = W.heightfield_mesh(16, 1.0, 1.0, W.water_params())
    d.add_mesh(P, F, sms.Bsdf(sms.BSDF_DIELECTRIC, 1.33), 0, N=N, UV=UV)
    light = d.add_sphere((0.0, 0.0, 4.0), 0.5, sms.Bsdf(sms.BSDF_DIFFUSE, 1.0, 0.0, (0.0, 0.0, 0.0)), 0)
    d.add_area_emitter(light, (40.0,) * 3, 0)
    osc = O.OracleScene(d)
    cam = W.pool_camera(8, 8)
    a = osc.render(W.water_config(), cam, sms.RenderOptions(integrator="path", spp=4, seed=3, rr_depth=100))
    for integ in ("path_filtered_ss", "path_filtered_ms"):
        b = osc.render(sms.SMSConfig(bounces=2), cam, sms.RenderOptions(integrator=integ, spp=4, seed=3, rr_depth=100))
        assert np.array_equal(a, b), integ
    assert a.mean() > 0.0


def test_path_filtered_ss_matches_path_sms_ss_on_flat_water(sms, workloads, O):
    """The oracle's path_filtered_ss and unbiased path_sms_ss estimate the
    same image (path_filtered_ss.cpp:27-35) on flat water; plain path tracing
    also carries the caustics reflected off the water, which both filter."""
    W = workloads
    osc = O.OracleScene(W.pool_scene(res=16, wave_scale=0.0))
    cam = W.pool_camera(12, 12)
    cfg = W.water_config()
    cfg.max_trials = -1
    runs = {}
    for integ, spp in (("path_filtered_ss", 2048), ("path_sms_ss", 256)):
        runs[integ] = np.stack([_blocks(osc.render(cfg, cam, sms.RenderOptions(integrator=integ, spp=spp,
                                                                                seed=70 + r)), 3)
                                for r in range(4)])
    a, b = runs["path_filtered_ss"], runs["path_sms_ss"]
    se = np.sqrt(a.var(0, ddof=1) / 4 + b.var(0, ddof=1) / 4)
    assert np.all(np.abs(a.mean(0) - b.mean(0)) < 5.0 * se + 0.01 * a.mean(0) + 1e-3), (a.mean(0), b.mean(0), se)
    assert abs(a.mean() - b.mean()) < 0.03 * a.mean()


def test_gaussian_film_filter(sms, workloads, O):
    """The film's Gaussian reconstruction filter (gaussian.cpp, ImageBlock::put
    at imageblock.cpp:111-160): a pixel is the weighted mean of the samples
    within 2 pixels, so a constant image stays constant; an edge is blurred over
    about two pixels either side; stddev 0 is refused by the library."""
    cfg = sms.SMSConfig()

    def sphere_light(flip):
        d = sms.SceneDesc()
        light = d.add_sphere((0.0, 0.0, 0.0), 1.0, sms.Bsdf(sms.BSDF_DIFFUSE, 1.0, 0.0, (0.0, 0.0, 0.0)), 0,
                             flip=flip)
        d.add_area_emitter(light, (3.0, 2.0, 1.0), 0)
        return O.OracleScene(d)

    # inside an inward-facing sphere light: every camera ray sees the emitter
    inside = sms.Camera.look_at((0.0, 0.0, 0.0), (0.0, 0.0, 1.0), (0.0, 1.0, 0.0), 60.0, 12, 10)
    g = sphere_light(True).render(cfg, inside, sms.RenderOptions(integrator="path", spp=4, seed=1,
                                                                  rfilter="gaussian"))
    np.testing.assert_allclose(g.reshape(-1, 3), np.tile([3.0, 2.0, 1.0], (120, 1)), rtol=1e-5)
    osc = sphere_light(False)
    # from outside: the sphere's silhouette, box vs Gaussian
    cam = sms.Camera.look_at((0.0, 0.0, 6.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 30.0, 24, 24)
    box = osc.render(cfg, cam, sms.RenderOptions(integrator="path", spp=16, seed=2))
    gau = osc.render(cfg, cam, sms.RenderOptions(integrator="path", spp=16, seed=2, rfilter="gaussian"))
    assert abs(gau[..., 0].sum() - box[..., 0].sum()) < 0.02 * box[..., 0].sum()
    # the silhouette's interior keeps the emitter's radiance
    assert abs(gau[12, 12, 0] - 3.0) < 1e-4 and abs(box[12, 12, 0] - 3.0) < 1e-4
    # the Gaussian image varies more smoothly across the silhouette
    assert np.abs(np.diff(gau[..., 0], axis=1)).max() < np.abs(np.diff(box[..., 0], axis=1)).max()
    # a wider filter blurs more
    wide = osc.render(cfg, cam, sms.RenderOptions(integrator="path", spp=16, seed=2, rfilter="gaussian",
                                                  rfilter_stddev=1.0))
    assert np.abs(np.diff(wide[..., 0], axis=1)).max() < np.abs(np.diff(gau[..., 0], axis=1)).max()


def test_twosided_diffuse(sms, workloads, O):
    """twosided.cpp: a twosided diffuse plane lit and seen from its back
    renders like the same plane lit and seen from its front; one-sided, its
    back is black."""
    cfg = sms.SMSConfig()
    opt = sms.RenderOptions(integrator="path", spp=64, seed=4)
    d, cam = workloads.plane_light_scene(below=False, twosided=False)
    front = O.OracleScene(d).render(cfg, cam, opt)
    d, cam = workloads.plane_light_scene(below=True, twosided=True)
    back = O.OracleScene(d).render(cfg, cam, opt)
    d, cam = workloads.plane_light_scene(below=True, twosided=False)
    dark = O.OracleScene(d).render(cfg, cam, opt)
    assert front.mean() > 0.01
    assert abs(back.mean() - front.mean()) < 0.03 * front.mean()
    assert not dark.any()


def test_tagged_receiver_query(sms, workloads, O):
    """A query naming its receiver shape (row 12 = -(1 + id), rows 13-14 the
    incident direction in the frame of its normal) evaluates that shape's
    BSDF: a diffuse shape gives the albedo query's estimate, a rough
    conductor its own glossy value, an id outside the scene nothing."""
    W = workloads
    far = np.array([[-1, -1, -10], [1, -1, -10], [1, 1, -10], [-1, 1, -10]], np.float32)
    tri = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
    cfg = W.sphere_config()
    q = W.sphere_queries(16)
    t = q.copy()
    t[12], t[13], t[14] = -2.0, 0.0, 0.0
    d = W.sphere_scene(conductor=True)
    d.add_mesh(far, tri, sms.Bsdf(sms.BSDF_DIFFUSE, 1.0, 0.0, (0.5, 0.5, 0.5)))
    osc = O.OracleScene(d)
    va, ca, _ = osc.connect_batch(cfg, q, seed=4)[:3]
    vt, ct, _ = osc.connect_batch(cfg, t, seed=4)[:3]
    assert va.sum() > 0
    np.testing.assert_array_equal(ca, ct)
    np.testing.assert_allclose(vt, va, rtol=1e-5, atol=1e-7)
    d = W.sphere_scene(conductor=True)
    d.add_mesh(far, tri, sms.Bsdf(sms.BSDF_CONDUCTOR, 0.2, 3.0, alpha=0.3))
    osc = O.OracleScene(d)
    vg = osc.connect_batch(cfg, t, seed=4)[0]
    np.testing.assert_array_equal(osc.connect_batch(cfg, t, seed=4)[1], ca)
    assert vg.sum() > 0 and not np.allclose(vg, va)
    t[12] = -9.0
    assert not osc.connect_batch(cfg, t, seed=4)[0].any()
