"""The allocation-free connection entry point (sms_ss_connect_batch_noalloc).

It serves callers that cannot allocate device memory during a render:
fixed-budget real-time loops, or hosts that own every device allocation and
forbid libraries from calling cudaMalloc.  It must give the same results as the regular device
entry point, call after call, even though its scratch array keeps the previous
call's contents.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(fn, ctx, q_dev, n, seed, stream_offset=0):
    import torch
    dev = q_dev.device
    val = torch.full((3, n), -1.0, dtype=torch.float32, device=dev)
    cnt = torch.full((n,), -7, dtype=torch.int32, device=dev)
    wlk = torch.full((n,), -7, dtype=torch.int32, device=dev)
    fn(q_dev.data_ptr(), n, val.data_ptr(), cnt.data_ptr(), wlk.data_ptr(), seed=seed, stream_offset=stream_offset)
    torch.cuda.synchronize()
    stream = torch.cuda.ExternalStream(ctx.stream)
    stream.synchronize()
    return val.cpu().numpy(), cnt.cpu().numpy(), wlk.cpu().numpy()


def test_noalloc_matches_device_entry_point(sms, workloads, gpu_lib):
    import torch
    W = workloads
    ctx = sms.Context(sms.Scene(W.water_scene(res=128)), W.water_config())
    ss = sms.SpecularManifoldSingleScatter(ctx)
    n = 6000
    q_dev = torch.from_numpy(W.water_queries(n)).cuda()
    # two calls in a row with different seeds and offsets: the second call must
    # not see anything the first one left in the shared scratch array
    for seed, off in ((3, 0), (4, 1000)):
        v_ref, c_ref, w_ref = _run(ss.specular_manifold_sampling_device, ctx, q_dev, n, seed, off)
        v, c, w = _run(ss.specular_manifold_sampling_noalloc, ctx, q_dev, n, seed, off)
        assert np.array_equal(c, c_ref) and np.array_equal(w, w_ref)
        np.testing.assert_allclose(v, v_ref, rtol=1e-6, atol=0)
        assert (c > 0).sum() > 0 and (w >= 1).all()
    ctx.close()


def test_noalloc_rejects_oversized_batch(sms, workloads, gpu_lib):
    import torch
    W = workloads
    ctx = sms.Context(sms.Scene(W.water_scene(res=64)), W.water_config())
    ss = sms.SpecularManifoldSingleScatter(ctx)
    n = sms.NOALLOC_MAX_QUERIES + 1
    q_dev = torch.zeros((16, n), dtype=torch.float32, device="cuda")
    out = torch.zeros((5, n), dtype=torch.float32, device="cuda")
    with pytest.raises(sms.SMSError) as e:
        ss.specular_manifold_sampling_noalloc(q_dev.data_ptr(), n, out[0].data_ptr(), out[3].data_ptr(),
                                              out[4].data_ptr())
    assert e.value.status == 1 and "exceed" in str(e.value)
    ctx.close()


def test_noalloc_biased_matches_device_and_shares_its_checks(sms, workloads, gpu_lib):
    """The biased estimator through the allocation-free call gives the device
    entry point's results, and a configuration the device entry point refuses
    (a biased max_trials above 2^24) is refused here too."""
    import dataclasses

    import torch
    W = workloads
    scene = sms.Scene(W.sphere_scene(conductor=True))
    ctx = sms.Context(scene, W.sphere_config())
    ss = sms.SpecularManifoldSingleScatter(ctx)
    n = 4096
    q_dev = torch.from_numpy(W.sphere_queries(64)).cuda()
    for seed in (1, 2):
        v_ref, c_ref, w_ref = _run(ss.specular_manifold_sampling_device, ctx, q_dev, n, seed)
        v, c, w = _run(ss.specular_manifold_sampling_noalloc, ctx, q_dev, n, seed)
        assert np.array_equal(c, c_ref) and np.array_equal(w, w_ref)
        np.testing.assert_allclose(v, v_ref, rtol=1e-6, atol=0)
        assert (c > 0).sum() > 0
    ctx.close()
    bad = dataclasses.replace(W.sphere_config(), max_trials=(1 << 24) + 1)
    ctx = sms.Context(scene, bad)
    ss = sms.SpecularManifoldSingleScatter(ctx)
    out = torch.zeros((5, n), dtype=torch.float32, device="cuda")
    for fn in (ss.specular_manifold_sampling_device, ss.specular_manifold_sampling_noalloc):
        with pytest.raises(sms.SMSError) as e:
            fn(q_dev.data_ptr(), n, out[0].data_ptr(), out[3].data_ptr(), out[4].data_ptr(), seed=1)
        assert e.value.status == 1 and "max_trials" in str(e.value)
    ctx.close()


def test_noalloc_device_limit_reported_by_next_call(sms, workloads, gpu_lib):
    """A device limit hit inside an allocation-free call (here a query naming
    a receiver shape outside the scene) is not returned by that asynchronous
    call; the context's next synchronous call reports it, and the one after
    that runs clean."""
    import torch
    W = workloads
    ctx = sms.Context(sms.Scene(W.sphere_scene(conductor=True)), W.sphere_config())
    ss = sms.SpecularManifoldSingleScatter(ctx)
    q = W.sphere_queries(16)
    bad = q.copy()
    bad[12] = -9.0
    n = q.shape[1]
    _run(ss.specular_manifold_sampling_noalloc, ctx, torch.from_numpy(bad).cuda(), n, 1)
    with pytest.raises(sms.SMSError, match="receiver shape"):
        ss.specular_manifold_sampling(q, seed=1)
    v, c, _ = ss.specular_manifold_sampling(q, seed=1)
    assert c.sum() > 0
    ctx.close()
