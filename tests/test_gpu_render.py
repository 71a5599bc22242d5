"""GPU path tracer (sms_render) against the oracle's restatement and against
plain path tracing.  Both implementations draw every random number from the
same PCG32 streams (keyed by path index), so most pixels agree to float
rounding; paths whose discrete choices (Russian roulette, Fresnel lobe, Newton
basin, duplicate merging) flip under FP32 rounding differences make the rest,
measured against the same statistic between the oracle's plain and
FMA-contracted builds."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PIXEL_RTOL = 1e-3   # per-pixel relative tolerance of "agreeing" pixels


def _blocks(img, b):
    h, w = img.shape[:2]
    return img[..., 0].reshape(h // b, b, w // b, b).mean(axis=(1, 3))


def _agree(a, b):
    return np.mean(np.abs(a - b) <= PIXEL_RTOL * np.maximum(np.abs(b), 1e-3))


def _far(a, b):
    return np.mean(np.abs(a - b) > 0.5 * np.maximum(np.abs(b), 1e-2))


def _check_against_oracle(sms, oracle, desc, cfg, cam, opt):
    """GPU image vs the oracle's, with the oracle's FMA-contracted build as
    the yardstick: the share of pixels that disagree (and that disagree by
    more than half) may exceed the oracle-vs-oracle floor by a small margin
    only.  Sample-level divergence from FP rounding (a flipped Fresnel choice,
    a Newton walk ending in another basin, a duplicate merged differently) is
    what the floor measures."""
    ctx = sms.Context(sms.Scene(desc), cfg)
    g = ctx.render(cam, opt)
    ctx.close()
    o = oracle.OracleScene(desc).render(cfg, cam, opt)
    f = oracle.OracleScene(desc, fma=True).render(cfg, cam, opt)
    assert np.isfinite(g).all()
    floor_mis, floor_far = 1.0 - _agree(f, o), _far(f, o)
    mis, far = 1.0 - _agree(g, o), _far(g, o)
    assert mis <= 1.5 * floor_mis + 0.05, (mis, floor_mis)
    assert far <= 1.5 * floor_far + 0.03, (far, floor_far)
    return g, o, f


@pytest.mark.parametrize("integrator", ["path", "path_sms_ss"])
def test_render_matches_oracle(sms, workloads, oracle, gpu_lib, integrator):
    W = workloads
    g, o, f = _check_against_oracle(sms, oracle, W.pool_scene(res=32), W.water_config(), W.pool_camera(16, 16),
                                    sms.RenderOptions(integrator=integrator, spp=8, seed=11))
    if integrator == "path":
        assert _agree(g, o) > 0.97


def test_render_biased_and_point_light_match_oracle(sms, workloads, oracle, gpu_lib):
    W = workloads
    g, o, f = _check_against_oracle(sms, oracle, W.pool_scene(res=32, point_light=True),
                                    sms.SMSConfig(biased=True, max_trials=16), W.pool_camera(16, 16),
                                    sms.RenderOptions(integrator="path_sms_ss", spp=4, seed=5))
    # bounded (biased) weights: the image means agree like the oracle builds do
    assert abs(g.mean() - o.mean()) <= 3.0 * abs(f.mean() - o.mean()) + 0.01 * o.mean()


def test_render_is_deterministic_and_wavefront_invariant(sms, workloads, gpu_lib):
    """Random numbers are keyed by path index: the same image from two runs,
    and (up to the order of the per-pixel sums) from a wavefront size that
    splits the samples of a pixel across launches."""
    W = workloads
    ctx = sms.Context(sms.Scene(W.pool_scene(res=32)), W.water_config())
    cam = W.pool_camera(24, 16)
    a = ctx.render(cam, sms.RenderOptions(spp=6, seed=2))
    b = ctx.render(cam, sms.RenderOptions(spp=6, seed=2))
    c = ctx.render(cam, sms.RenderOptions(spp=6, seed=2, max_paths=1000))
    assert np.array_equal(a, b)
    assert np.allclose(a, c, rtol=1e-5, atol=1e-6)
    d = ctx.render(cam, sms.RenderOptions(spp=6, seed=3))
    assert not np.array_equal(a, d)
    ctx.close()


def _compare_integrators(sms, ctx, cam, integ, spp_path, spp_sms, reps, block=4, rel=0.02, base="path"):
    """Integrator `base` (plain path tracing by default) vs integrator `integ`
    on 4x4-pixel blocks: the difference of the means must lie within 5
    standard errors (from the spread of `reps` independent runs) plus `rel` of
    the value."""
    runs = {}
    for name, spp in ((base, spp_path), (integ, spp_sms)):
        runs[name] = np.stack([_blocks(ctx.render(cam, sms.RenderOptions(integrator=name, spp=spp, seed=900 + r)),
                                       block) for r in range(reps)])
    a, b = runs[base], runs[integ]
    se = np.sqrt(a.var(0, ddof=1) / reps + b.var(0, ddof=1) / reps)
    diff = np.abs(a.mean(0) - b.mean(0))
    assert np.all(diff < 5.0 * se + rel * a.mean(0) + 1e-3), (a.mean(0), b.mean(0), se)
    assert abs(a.mean() - b.mean()) < rel * a.mean()


def test_path_sms_ss_is_unbiased_against_path(sms, workloads, gpu_lib):
    """Flat water: unbiased SMS + the integrator's path filtering estimate the
    same image as plain path tracing."""
    W = workloads
    cfg = W.water_config()
    cfg.max_trials = -1
    ctx = sms.Context(sms.Scene(W.pool_scene(res=32, wave_scale=0.0)), cfg)
    _compare_integrators(sms, ctx, W.pool_camera(32, 32), "path_sms_ss", 4096, 512, 4)
    ctx.close()


def test_unbiased_mnee_is_unbiased_against_path(sms, workloads, gpu_lib):
    """mnee_init without biased_mnee (path_sms_ss.cpp:207-241): paths the
    deterministic MNEE walk cannot find are added from BSDF sampling."""
    W = workloads
    cfg = W.water_config()
    cfg.mnee_init = True
    ctx = sms.Context(sms.Scene(W.pool_scene(res=32, wave_scale=0.0)), cfg)
    _compare_integrators(sms, ctx, W.pool_camera(32, 32), "path_sms_ss", 4096, 512, 4)
    ctx.close()


def _slab_desc(sms, W, caster_below=False):
    """Flat glass slab (caster_multi top sheet z = 1.3, bouncer bottom sheet
    z = 1, or the other way round) over the diffuse floor, sphere light above
    (caustic_emitter_multi)."""
    d = sms.SceneDesc()
    fl = np.array([[-2, -2, 0], [2, -2, 0], [2, 2, 0], [-2, 2, 0]], np.float32)
    d.add_mesh(fl, np.array([[0, 1, 2], [0, 2, 3]], np.uint32), sms.Bsdf(sms.BSDF_DIFFUSE, 1.0, 0.0, (0.5,) * 3),
               sms.SHAPE_CAUSTIC_RECEIVER, UV=np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32))
    glass = sms.Bsdf(sms.BSDF_DIELECTRIC, 1.5)
    top, bottom = sms.SHAPE_CAUSTIC_CASTER_MULTI, sms.SHAPE_CAUSTIC_BOUNCER
    if caster_below:
        top, bottom = bottom, top
    P, N, UV, F = W.heightfield_mesh(16, 1.0, 1.3, [])
    d.add_mesh(P, F, glass, top, N=N, UV=UV)
    P, N, UV, F = W.heightfield_mesh(16, 1.0, 1.0, [], flip_normals=True)
    d.add_mesh(P, F, glass, bottom, N=N, UV=UV)
    light = d.add_sphere((0.0, 0.0, 4.0), 0.5, sms.Bsdf(sms.BSDF_DIFFUSE, 1.0, 0.0, (0.0, 0.0, 0.0)), 0)
    d.add_area_emitter(light, (40.0,) * 3, sms.EMITTER_CAUSTIC_MULTI)
    return d


def test_path_sms_ms_matches_path_on_flat_slab(sms, workloads, gpu_lib):
    """Two-bounce chains through a flat glass slab over the floor: path_sms_ms
    (bounces = 2, unbiased, half-vector constraints) against plain path
    tracing, seen by a camera under the slab, where every light path to the
    visible floor crosses both faces.  (The slab's faces are two open sheets:
    light that enters one face and leaves through the open side is a
    one-vertex chain, which path_sms_ms filters and bounces = 2 cannot
    sample, as in the reference.)  Paths that reflect inside the slab are
    filtered and not re-sampled either, a loss below 1% here, inside the 2%
    tolerance.  With the light straight above, the angle-difference
    constraints sit at their pole: walks rarely converge and the unbiased
    estimate, while still unbiased, is too heavy-tailed for a 4-run test."""
    W = workloads
    d = _slab_desc(sms, W)
    cfg = sms.SMSConfig(biased=False, max_trials=-1, bounces=2, halfvector_constraints=True)
    ctx = sms.Context(sms.Scene(d), cfg)
    cam = sms.Camera.look_at((0.0, 0.0, 0.9), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 60.0, 32, 32)
    _compare_integrators(sms, ctx, cam, "path_sms_ms", 4096, 512, 4)
    ctx.close()


def test_render_with_learned_proposal(sms, workloads, gpu_lib):
    """A bound learned proposal seeds the SMS calls of the path tracer."""
    import torch
    W = workloads
    ctx = sms.Context(sms.Scene(W.pool_scene(res=32)), W.water_config())
    q = torch.from_numpy(W.water_queries(8192, seed=4)).cuda()
    torch.cuda.synchronize()
    prop = sms.SeedProposal(ctx, 1, seed=1, capacity=1 << 15)
    assert prop.collect(q.data_ptr(), 8192, seed=4, walks_per_query=4) > 0
    prop.normalize()
    prop.train(steps=50, batch=1024)
    ctx.set_proposal(prop, 0.1)
    img = ctx.render(W.pool_camera(16, 16), sms.RenderOptions(spp=4, seed=1))
    assert np.isfinite(img).all() and img.mean() > 0.0
    ctx.set_proposal(None)
    prop.close()
    ctx.close()


def test_render_argument_errors(sms, workloads, gpu_lib):
    W = workloads
    ctx = sms.Context(sms.Scene(W.pool_scene(res=16)), sms.SMSConfig(mnee_init=True, bounces=5))
    with pytest.raises(sms.SMSError) as e:   # chains of 1..4 vertices
        ctx.render(W.pool_camera(8, 8), sms.RenderOptions(integrator="path_filtered_ms"))
    assert e.value.status == 4
    with pytest.raises(sms.SMSError) as e:
        ctx.render(W.pool_camera(8, 8), sms.RenderOptions(spp=0))
    assert e.value.status == 1
    cam = W.pool_camera(8, 8)
    cam.fov = 0.0
    with pytest.raises(sms.SMSError):
        ctx.render(cam, sms.RenderOptions())
    ctx.close()


@pytest.mark.parametrize("alpha", [0.2, 0.5])
def test_rough_caustic_is_unbiased_against_path(sms, workloads, gpu_lib, alpha):
    """Glossy caustic through a rough dielectric sheet from a point light:
    path_sms_ss (offset normals, half-vector constraints) against plain path
    tracing, which reaches the light by emitter sampling at the rough vertex.
    Camera under the sheet: every light path crosses it."""
    W = workloads
    d = sms.SceneDesc()
    fl = np.array([[-2, -2, 0], [2, -2, 0], [2, 2, 0], [-2, 2, 0]], np.float32)
    d.add_mesh(fl, np.array([[0, 1, 2], [0, 2, 3]], np.uint32), sms.Bsdf(sms.BSDF_DIFFUSE, 1.0, 0.0, (0.5,) * 3),
               sms.SHAPE_CAUSTIC_RECEIVER, UV=np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32))
    P, N, UV, F = W.heightfield_mesh(16, 1.0, 1.3, [])
    d.add_mesh(P, F, sms.Bsdf(sms.BSDF_DIELECTRIC, 1.5, alpha=alpha), sms.SHAPE_CAUSTIC_CASTER_SINGLE, N=N, UV=UV)
    d.add_point_emitter((0.3, 0.2, 4.0), (40.0,) * 3, sms.EMITTER_CAUSTIC_SINGLE)
    ctx = sms.Context(sms.Scene(d), sms.SMSConfig(biased=False, max_trials=-1, halfvector_constraints=True))
    cam = sms.Camera.look_at((0.0, 0.0, 0.9), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 60.0, 32, 32)
    _compare_integrators(sms, ctx, cam, "path_sms_ss", 8192, 256, 4)
    ctx.close()


@pytest.mark.parametrize("biased", [True, False])
def test_glints_integrator_matches_oracle(sms, workloads, oracle, gpu_lib, biased):
    """path_sms_glints (manifold_glints.cpp:28-223 inside path_sms_glints.cpp):
    glint SMS over each camera footprint with sensor importance and LEAN-MIS,
    on the GPU against the oracle (LEAN pyramid built on the device), against
    the oracle-vs-FMA floor."""
    W = workloads
    desc = W.glint_scene(map_res=512)
    cfg = W.glint_config()
    if not biased:
        cfg = sms.SMSConfig(biased=False, max_trials=64, max_iterations=10)
    g, o, f = _check_against_oracle(sms, oracle, desc, cfg, W.glint_render_camera(32, 32),
                                    sms.RenderOptions(integrator="path_sms_glints", spp=4, seed=7))
    assert (o[..., 0] > 0).mean() > 0.005
    assert abs(g.mean() - o.mean()) <= 3.0 * abs(f.mean() - o.mean()) + 0.02 * o.mean()


@pytest.mark.parametrize("integrator", ["path", "path_sms_glints"])
def test_lean_fallback_matches_oracle(sms, workloads, oracle, gpu_lib, integrator):
    """The normal map's LEAN fallback BSDF (normalmap.cpp:80-112, 142-170,
    187-203): paths that reach the normal-mapped plane after a bounce off the
    diffuse wall reflect like the map's top LEAN level (emitter sampling with
    the LEAN eval and density, BSDF sampling of visible normals); GPU vs the
    oracle within the oracle-vs-FMA floor, and the fallback changes the
    image."""
    W = workloads
    desc = W.lean_fallback_scene(map_res=256)
    cfg = W.glint_config()
    cam = W.lean_fallback_camera(24, 24)
    opt = sms.RenderOptions(integrator=integrator, spp=8, seed=3)
    g, o, f = _check_against_oracle(sms, oracle, desc, cfg, cam, opt)
    assert abs(g.mean() - o.mean()) <= 3.0 * abs(f.mean() - o.mean()) + 0.01 * o.mean()
    desc.lean_fallback = None
    ctx = sms.Context(sms.Scene(desc), cfg)
    plain = ctx.render(cam, opt)
    ctx.close()
    assert abs(plain.mean() - g.mean()) > 0.005 * g.mean()


def test_gaussian_film_filter_matches_oracle(sms, workloads, oracle, gpu_lib):
    """The film's Gaussian reconstruction filter (gaussian.cpp; ImageBlock::put,
    imageblock.cpp:111-160): the GPU gathers each pixel's weighted samples in a
    fixed order, chunk by chunk; the oracle splats sample by sample.  Checked
    with the whole image in one wavefront and with wavefronts smaller than the
    image (the splat crosses chunk boundaries)."""
    W = workloads
    desc, cfg = W.pool_scene(res=32), W.water_config()
    cam = W.pool_camera(20, 16)
    for max_paths in (0, 97):
        opt = sms.RenderOptions(integrator="path_sms_ss", spp=4, seed=11, rfilter="gaussian", max_paths=max_paths)
        g, o, f = _check_against_oracle(sms, oracle, desc, cfg, cam, opt)
        assert abs(g.mean() - o.mean()) <= 3.0 * abs(f.mean() - o.mean()) + 0.01 * o.mean()
    ctx = sms.Context(sms.Scene(desc), cfg)
    box = ctx.render(cam, sms.RenderOptions(integrator="path_sms_ss", spp=4, seed=11))
    with pytest.raises(sms.SMSError):
        ctx.render(cam, sms.RenderOptions(integrator="path_sms_ss", spp=4, seed=11, rfilter="gaussian",
                                          rfilter_stddev=0.0))
    ctx.close()
    assert not np.array_equal(box, g)


def test_twosided_matches_oracle(sms, workloads, oracle, gpu_lib):
    """A twosided diffuse plane lit and seen from its back (twosided.cpp: the
    local frame's normal reflected), GPU vs the oracle; one-sided it is black
    on the GPU too."""
    W = workloads
    cfg = sms.SMSConfig()
    opt = sms.RenderOptions(integrator="path", spp=16, seed=4)
    d, cam = W.plane_light_scene(below=True, twosided=True)
    g, o, f = _check_against_oracle(sms, oracle, d, cfg, cam, opt)
    assert o.mean() > 0.01
    d, cam = W.plane_light_scene(below=True, twosided=False)
    ctx = sms.Context(sms.Scene(d), cfg)
    assert not ctx.render(cam, opt).any()
    ctx.close()


@pytest.mark.parametrize("nonlinear", [False, True])
def test_roughplastic_matches_oracle(sms, workloads, oracle, gpu_lib, nonlinear):
    """A roughplastic plane (roughplastic.cpp: Beckmann coating over a diffuse
    base) lit by a sphere light in view of its glossy lobe, GPU vs the oracle.
    The library tabulates the coating's transmittance by its own quadrature,
    the oracle by the reference's; they agree to about 1e-3."""
    b = sms.Bsdf(sms.BSDF_ROUGHPLASTIC, 1.49 / 1.000277, 0.0, (0.2, 0.5, 0.8), alpha=0.15, nonlinear=nonlinear)
    d, cam = workloads.plane_light_scene(below=False, twosided=False, width=24, height=24, bsdf=b)
    g, o, f = _check_against_oracle(sms, oracle, d, sms.SMSConfig(), cam,
                                    sms.RenderOptions(integrator="path", spp=16, seed=6))
    assert o.mean() > 0.01
    assert abs(g.mean() - o.mean()) < 0.02 * o.mean()


def test_roughplastic_refused_on_the_caustic_path(sms, gpu_lib):
    """A roughplastic shape cannot be a caustic caster (the manifold walks
    need a smooth dielectric or conductor)."""
    def scene(caster_bsdf):
        d = sms.SceneDesc()
        q = np.array([[-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], np.float32)
        d.add_mesh(q, np.array([[0, 1, 2], [0, 2, 3]], np.uint32), caster_bsdf, sms.SHAPE_CAUSTIC_CASTER_SINGLE)
        d.add_mesh(q * np.float32([3, 3, 0]), np.array([[0, 1, 2], [0, 2, 3]], np.uint32),
                   sms.Bsdf(sms.BSDF_DIFFUSE, 1.0, 0.0, (0.5,) * 3), sms.SHAPE_CAUSTIC_RECEIVER)
        light = d.add_sphere((0, 0, 5), 0.3, sms.Bsdf(sms.BSDF_DIFFUSE, 1.0, 0.0, (0.0,) * 3), 0)
        d.add_area_emitter(light, (10.0,) * 3, sms.EMITTER_CAUSTIC_SINGLE)
        return sms.Scene(d)

    sms.Context(scene(sms.Bsdf(sms.BSDF_DIELECTRIC, 1.5)), sms.SMSConfig()).close()
    with pytest.raises(sms.SMSError, match="roughplastic"):
        sms.Context(scene(sms.Bsdf(sms.BSDF_ROUGHPLASTIC, 1.5, 0.0, (0.5,) * 3, alpha=0.1)), sms.SMSConfig())


def _teaser_area_light(sms, W):
    """The teaser stand-in with its point light replaced by a sphere area light
    flagged for single- and multi-scatter caustics, so that path tracing can
    reach the caustics it filters."""
    desc = W.teaser_scene()
    desc.point_emitters.clear()
    light = desc.add_sphere((0.0, 0.5, 4.0), 0.4, sms.Bsdf(sms.BSDF_DIFFUSE, 1.0, 0.0, (0.0, 0.0, 0.0)), 0)
    desc.add_area_emitter(light, (40.0, 40.0, 40.0), sms.EMITTER_CAUSTIC_SINGLE | sms.EMITTER_CAUSTIC_MULTI)
    return desc


def test_filtered_teaser_matches_oracle(sms, workloads, oracle, gpu_lib):
    """path_filtered_teaser (path_filtered_teaser.cpp:56-226, 331-410): path
    tracing with the teaser's caustic filter (single- and multi-scatter chains
    tracked by the path record, caustic-only emitter samples on casters) on the
    teaser stand-in with an area light, GPU vs the oracle within the
    oracle-vs-FMA floor."""
    W = workloads
    desc = _teaser_area_light(sms, W)
    cfg = sms.SMSConfig(bounces=2)
    cam = W.teaser_camera(16, 16)
    opt = sms.RenderOptions(integrator="path_filtered_teaser", spp=8, seed=5)
    g, o, f = _check_against_oracle(sms, oracle, desc, cfg, cam, opt)
    assert abs(g.mean() - o.mean()) <= 3.0 * abs(f.mean() - o.mean()) + 0.02 * o.mean()


def test_filtered_teaser_caustics_only(sms, workloads, oracle, gpu_lib):
    """Without the non-SMS paths only the filtered caustics remain.  With the
    teaser's point light none can be found by path tracing (its casters are
    smooth, so they take no emitter samples, and no ray hits a point light):
    the image is zero, and no SMS query is made.  With an area light the
    sparse caustic image (a few paths per pixel that reach the light through
    the chains) matches the oracle's."""
    W = workloads
    cfg = sms.SMSConfig(bounces=2)
    ctx = sms.Context(sms.Scene(W.teaser_scene()), cfg)
    img = ctx.render(W.teaser_camera(16, 16), sms.RenderOptions(integrator="path_filtered_teaser", spp=8, seed=5,
                                                                non_sms_paths_enabled=False))
    assert ctx.stats()["connections"] == 0
    ctx.close()
    assert not img.any()
    desc = _teaser_area_light(sms, W)
    cam = W.teaser_camera(24, 24)
    opt = sms.RenderOptions(integrator="path_filtered_teaser", spp=256, seed=5, non_sms_paths_enabled=False)
    ctx = sms.Context(sms.Scene(desc), cfg)
    g = ctx.render(cam, opt)
    ctx.close()
    o = oracle.OracleScene(desc).render(cfg, cam, opt)
    nz_g, nz_o = g[..., 0] > 0, o[..., 0] > 0
    print(f"filtered teaser caustics: mean gpu {g.mean():.5g} oracle {o.mean():.5g}, "
          f"pixels {nz_g.sum()} / {nz_o.sum()}, shared {(nz_g & nz_o).sum()}")
    assert nz_o.sum() > 10
    assert (nz_g & nz_o).sum() >= 0.7 * nz_o.sum()
    assert abs(g.mean() - o.mean()) <= 0.25 * o.mean()


@pytest.mark.parametrize("integrator", ["path_filtered_ss", "path_filtered_ms"])
def test_filtered_integrators_match_oracle(sms, workloads, oracle, gpu_lib, integrator):
    """path_filtered_ss / path_filtered_ms (plain path tracing restricted to
    the paths the SMS integrators account for) on the GPU against the oracle,
    against the oracle-vs-FMA floor."""
    W = workloads
    if integrator == "path_filtered_ss":
        desc, cfg, cam = W.pool_scene(res=32), W.water_config(), W.pool_camera(16, 16)
    else:
        desc = _slab_desc(sms, W, caster_below=True)
        cfg = sms.SMSConfig(bounces=2)
        cam = sms.Camera.look_at((0.0, 0.0, 0.9), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 60.0, 16, 16)
    g, o, f = _check_against_oracle(sms, oracle, desc, cfg, cam, sms.RenderOptions(integrator=integrator, spp=8,
                                                                                   seed=21))
    assert o.mean() > 0.0


def test_path_filtered_ss_matches_path_sms_ss(sms, workloads, gpu_lib):
    """Flat water: path_filtered_ss finds by BSDF and emitter sampling exactly
    the light paths unbiased path_sms_ss accounts for (path_filtered_ss.cpp:
    27-35), so the two estimate the same image."""
    W = workloads
    cfg = W.water_config()
    cfg.max_trials = -1
    ctx = sms.Context(sms.Scene(W.pool_scene(res=32, wave_scale=0.0)), cfg)
    _compare_integrators(sms, ctx, W.pool_camera(32, 32), "path_sms_ss", 4096, 512, 4, base="path_filtered_ss")
    ctx.close()


def test_path_filtered_ms_matches_path_sms_ms(sms, workloads, gpu_lib):
    """The flat slab seen from under it: path_filtered_ms (its path record
    keeps exactly the receiver -> caster -> bouncer -> light chains of
    path_filtered_ms.cpp:219-301) against unbiased path_sms_ms.  The record
    wants the first specular vertex after the receiver to be a
    caustic_caster_multi shape, so the caster is the slab's lower sheet here
    (path_sms_ms's seed paths may start on either, manifold_ms.cpp:351)."""
    W = workloads
    cfg = sms.SMSConfig(biased=False, max_trials=-1, bounces=2, halfvector_constraints=True)
    ctx = sms.Context(sms.Scene(_slab_desc(sms, W, caster_below=True)), cfg)
    cam = sms.Camera.look_at((0.0, 0.0, 0.9), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 60.0, 32, 32)
    _compare_integrators(sms, ctx, cam, "path_sms_ms", 4096, 512, 4, base="path_filtered_ms")
    ctx.close()


def test_render_passes_and_timeout(sms, workloads, gpu_lib):
    """samples_per_pass / timeout (integrator.cpp:35-36, 61-68, 143-146):
    passes change nothing but the summation order; a timeout that has run
    out after the first pass leaves its mean (spp_done = samples_per_pass,
    the same paths as a 1-pass render); spp must be a multiple of the pass."""
    W = workloads
    ctx = sms.Context(sms.Scene(W.pool_scene(res=32)), W.water_config())
    cam = W.pool_camera(24, 16)
    a = ctx.render(cam, sms.RenderOptions(spp=8, seed=4))
    assert ctx.render_spp_done() == 8
    b = ctx.render(cam, sms.RenderOptions(spp=8, seed=4, samples_per_pass=2))
    assert np.allclose(a, b, rtol=1e-5, atol=1e-6)
    c = ctx.render(cam, sms.RenderOptions(spp=64, seed=4, samples_per_pass=1, timeout=1e-6))
    assert ctx.render_spp_done() == 1
    d = ctx.render(cam, sms.RenderOptions(spp=1, seed=4))
    assert np.array_equal(c, d)
    with pytest.raises(sms.SMSError):
        ctx.render(cam, sms.RenderOptions(spp=8, samples_per_pass=3))
    ctx.close()


def test_unbiased_mnee_multi_scatter(sms, workloads, oracle, gpu_lib):
    """path_sms_ms with mnee_init and without biased_mnee (MNEEHelper,
    path_sms_ms.cpp:54-142, 323-360): the deterministic MNEE chain plus the
    BSDF-sampled chains MNEE does not reproduce.  GPU vs oracle within the
    FMA floor, and unbiased against plain path tracing under the slab."""
    W = workloads
    desc = _slab_desc(sms, W, caster_below=True)
    cfg = sms.SMSConfig(biased=True, max_trials=1, mnee_init=True, bounces=2, halfvector_constraints=True)
    cam = sms.Camera.look_at((0.0, 0.0, 0.9), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 60.0, 16, 16)
    g, o, f = _check_against_oracle(sms, oracle, desc, cfg, cam,
                                    sms.RenderOptions(integrator="path_sms_ms", spp=8, seed=17))
    assert o.mean() > 0.0
    ctx = sms.Context(sms.Scene(desc), cfg)
    cam = sms.Camera.look_at((0.0, 0.0, 0.9), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 60.0, 32, 32)
    _compare_integrators(sms, ctx, cam, "path_sms_ms", 4096, 512, 4)
    ctx.close()


def test_teaser_matches_oracle(sms, workloads, oracle, gpu_lib):
    """path_sms_teaser (path_sms_teaser.cpp:120-320) on a small stand-in for its
    scene: single-scatter caustics of a mirror sphere and two-bounce caustics of
    a glass sphere on a diffuse floor (the caustics_* config), biased glints on
    a normal-mapped tile seen from the camera (the glints_* config), and the
    filtered path tracing around them; GPU vs the oracle's restatement, path by
    path, within the oracle-vs-FMA floor.  Each part also contributes alone."""
    W = workloads
    desc = W.teaser_scene()
    cfg = sms.SMSConfig(biased=True, max_trials=16, bounces=2)
    cam = W.teaser_camera(16, 16)
    gcfg = sms.SMSConfig(max_trials=16, max_iterations=10)
    opt = sms.RenderOptions(integrator="path_sms_teaser", spp=4, seed=3, glints=gcfg)
    g, o, f = _check_against_oracle(sms, oracle, desc, cfg, cam, opt)
    print(f"teaser: mean gpu {g.mean():.5g} oracle {o.mean():.5g} fma {f.mean():.5g}")
    assert abs(g.mean() - o.mean()) <= 3.0 * abs(f.mean() - o.mean()) + 0.02 * o.mean()
    ctx = sms.Context(sms.Scene(desc), cfg)
    parts = {}
    for name, kw in (("caustics", dict(glints_enabled=False, non_sms_paths_enabled=False)),
                     ("glints", dict(caustics_enabled=False, non_sms_paths_enabled=False)),
                     ("paths", dict(caustics_enabled=False, glints_enabled=False))):
        parts[name] = ctx.render(cam, sms.RenderOptions(integrator="path_sms_teaser", spp=4, seed=3, glints=gcfg,
                                                        **kw))
        assert np.isfinite(parts[name]).all() and parts[name].max() > 0, name
    # the image is deterministic
    np.testing.assert_array_equal(ctx.render(cam, opt), g)
    ctx.close()
