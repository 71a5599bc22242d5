"""Edge cases of the C ABI on the GPU: empty batches, scenes without casters
or emitters, unbounded Bernoulli trials, and misuse of the learned-proposal
API.  Every error is an sms_status (SMSError in Python), never a crash; per-walk
failures are data."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _plane_only(sms):
    d = sms.SceneDesc()
    P = np.array([[-2, -2, 0], [2, -2, 0], [2, 2, 0], [-2, 2, 0]], np.float32)
    F = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
    d.add_mesh(P, F, sms.Bsdf(sms.BSDF_DIFFUSE, 1.0, 0.0, (0.5, 0.5, 0.5)), sms.SHAPE_CAUSTIC_RECEIVER)
    return d


def test_empty_batches_for_every_estimator(sms, workloads, gpu_lib):
    W = workloads
    ctx = sms.Context(sms.Scene(W.slab_scene(res=32)), W.slab_config())
    v, c, w = sms.SpecularManifoldMultiScatter(ctx).specular_manifold_sampling(np.zeros((16, 0), np.float32))
    assert v.shape == (3, 0) and c.shape == (0,)
    ctx = sms.Context(sms.Scene(W.glint_scene(map_res=64)), W.glint_config())
    v, c, w = sms.SpecularManifoldGlints(ctx).specular_manifold_sampling(
        np.zeros((sms.GLINT_QUERY_FIELDS, 0), np.float32))
    assert v.shape == (3, 0)
    ctx = sms.Context(sms.Scene(W.water_scene(res=32)), W.water_config())
    v, c, w = sms.SpecularManifoldSingleScatter(ctx).specular_manifold_sampling(np.zeros((16, 0), np.float32))
    assert v.shape == (3, 0)


@pytest.mark.parametrize("biased", [True, False])
def test_no_caster_gives_zero(sms, workloads, gpu_lib, biased):
    """manifold_ss.cpp:53-55: without caustic casters every query gets zero."""
    d = _plane_only(sms)
    d.add_point_emitter((0.0, 0.0, 5.0), (100.0, 100.0, 100.0))
    ctx = sms.Context(sms.Scene(d), sms.SMSConfig(biased=biased, max_trials=16 if biased else 64))
    v, c, w = sms.SpecularManifoldSingleScatter(ctx).specular_manifold_sampling(workloads.sphere_queries(8), seed=1)
    assert np.all(v == 0) and np.all(c == 0)


def test_no_emitter_gives_zero(sms, workloads, gpu_lib):
    """No caustic emitter: the emitter sample fails and nothing is walked."""
    d = sms.SceneDesc()
    d.add_sphere((0.0, 0.0, 1.5), 1.0, sms.Bsdf(sms.BSDF_DIELECTRIC, 1.5), sms.SHAPE_CAUSTIC_CASTER_SINGLE)
    ctx = sms.Context(sms.Scene(d), workloads.sphere_config())
    v, c, w = sms.SpecularManifoldSingleScatter(ctx).specular_manifold_sampling(workloads.sphere_queries(8), seed=1)
    assert np.all(v == 0) and np.all(w == 0)
    st = ctx.stats()
    assert st["walks"] == 0 and st["connections"] == 0


def test_unbounded_trials_finish_or_report_the_limit(sms, workloads, gpu_lib):
    """max_trials <= 0 is unbounded in the reference (manifold_ss.cpp:127); the
    device stops at 65,536 trials and returns SMS_ERR_DEVICE_LIMIT instead of
    looping forever.  On the sphere every query finishes well below that."""
    W = workloads
    ctx = sms.Context(sms.Scene(W.sphere_scene()), sms.SMSConfig(biased=False, max_trials=-1))
    v, c, w = sms.SpecularManifoldSingleScatter(ctx).specular_manifold_sampling(W.sphere_queries(16), seed=2)
    assert np.all(c >= 0) and np.isfinite(v).all()


def test_proposal_api_misuse_is_reported(sms, workloads, gpu_lib):
    W = workloads
    desc = W.water_scene(res=32)
    ctx = sms.Context(sms.Scene(desc), W.water_config())
    with pytest.raises(sms.SMSError) as e:
        sms.SeedProposal(ctx, 5, capacity=16)          # not a caster shape
    assert e.value.status == 1
    prop = sms.SeedProposal(ctx, 0, capacity=64)
    with pytest.raises(sms.SMSError):
        prop.train(steps=1, batch=256)                  # empty training set
    rng = np.random.default_rng(0)
    prop.set_data(rng.normal(size=(9, 64)).astype(np.float32), rng.uniform(size=(2, 64)).astype(np.float32))
    with pytest.raises(sms.SMSError):
        prop.train(steps=1, batch=24)                   # not a multiple of 16
    with pytest.raises(sms.SMSError):
        prop.loss_grad(128)                             # more rows than the data set
    with pytest.raises(sms.SMSError):
        prop.set_data(np.zeros((9, 65), np.float32), np.zeros((2, 65), np.float32))   # over capacity
    with pytest.raises(sms.SMSError):
        ctx.set_proposal(prop, 0.0)                     # defensive share must be > 0
    ctx.set_proposal(prop, 0.1)
    ctx.set_config(sms.SMSConfig(biased=True, max_trials=16))
    with pytest.raises(sms.SMSError) as e:
        sms.SpecularManifoldSingleScatter(ctx).specular_manifold_sampling(W.water_queries(16))
    assert e.value.status == 4                          # unsupported: learned seeds need the unbiased estimator
    ctx.set_config(W.water_config())
    import torch
    q = torch.from_numpy(W.water_queries(64)).cuda()
    out = torch.zeros((5, 64), dtype=torch.float32, device="cuda")
    with pytest.raises(sms.SMSError) as e:
        sms.SpecularManifoldSingleScatter(ctx).specular_manifold_sampling_noalloc(
            q.data_ptr(), 64, out[0].data_ptr(), out[3].data_ptr(), out[4].data_ptr())
    assert e.value.status == 4
    ctx.set_proposal(None)
    v, c, w = sms.SpecularManifoldSingleScatter(ctx).specular_manifold_sampling(W.water_queries(16), seed=1)
    assert np.isfinite(v).all()


def test_context_destroyed_before_its_proposal(sms, workloads, gpu_lib):
    """Destroying a context detaches its proposals; destroying them afterwards
    is safe, and they refuse work."""
    W = workloads
    ctx = sms.Context(sms.Scene(W.water_scene(res=32)), W.water_config())
    prop = sms.SeedProposal(ctx, 0, capacity=64)
    ctx.set_proposal(prop, 0.1)
    ctx.close()
    with pytest.raises(sms.SMSError):
        prop.normalize()
    prop.close()


def test_context_destroyed_before_unbound_proposals(sms, workloads, gpu_lib):
    W = workloads
    ctx = sms.Context(sms.Scene(W.water_scene(res=32)), W.water_config())
    a = sms.SeedProposal(ctx, 0, capacity=64)
    b = sms.SeedProposal(ctx, 0, capacity=64)
    ctx.set_proposal(a, 0.1)
    ctx.close()
    for p in (a, b):
        with pytest.raises(sms.SMSError):
            p.train(steps=1, batch=16)
        p.close()
