"""The oracle's other builds (oracle/Makefile): the counting build gives
results identical to the FP32 oracle, the FP64 build agrees on well-conditioned
scenes, and the operation counts behind the FLOP/s figures are stable.  CPU
only."""
import numpy as np
import pytest


def _connect(oracle, variant, desc, cfg, q, **kw):
    return oracle.OracleScene(desc, variant=variant).connect_batch(cfg, q, seed=1, nthreads=4, **kw)


@pytest.mark.parametrize("case", ["sphere", "water", "slab", "glints"])
def test_counting_build_is_bit_identical(workloads, oracle, case):
    W = workloads
    if case == "sphere":
        args, kw = (W.sphere_scene(conductor=True), W.sphere_config(), W.sphere_queries(16)), {}
    elif case == "water":
        args, kw = (W.water_scene(res=64), W.water_config(), W.water_queries(512)), {}
    elif case == "slab":
        args, kw = (W.slab_scene(res=32), W.slab_config(), W.slab_queries(128)), {"multi": True}
    else:
        args, kw = (W.glint_scene(map_res=256), W.glint_config(), W.glint_queries(32)), {"glints": True}
    a = _connect(oracle, "f32", *args, **kw)
    b = _connect(oracle, "ops", *args, **kw)
    for x, y in zip(a[:3], b[:3]):
        assert np.array_equal(x, y)
    assert a[3] == b[3]


def test_double_build_agrees_on_the_sphere(workloads, oracle):
    W = workloads
    desc, cfg, q = W.sphere_scene(conductor=True), W.sphere_config(), W.sphere_queries(32)
    a = _connect(oracle, "f32", desc, cfg, q)
    b = _connect(oracle, "f64", desc, cfg, q)
    assert oracle.load(variant="f64").oracle_build_kind() == 1
    assert np.mean(a[1] == b[1]) > 0.99
    both = (a[1] == b[1]) & (a[1] > 0)
    assert both.sum() > 20
    assert np.abs(a[0][:, both] - b[0][:, both]).max() <= 1e-3 * np.abs(b[0]).max()


def test_operation_counts(workloads, oracle):
    """FLOPs per Newton iteration on the sphere (analytic intersection), and per
    box / triangle test on the water mesh, in the ranges the per-unit table of
    the measurement uses."""
    W = workloads
    s = oracle.flops_per_unit(W.sphere_scene(conductor=True), W.sphere_config(), W.sphere_queries(16), nthreads=4)
    assert 300 < s["flops_per_newton_iteration"] < 600
    assert s["counts"]["box_tests"] == 0 and s["counts"]["rays"] > 0
    assert 4 <= s["transcendentals_per_newton_iteration"] <= 6
    w = oracle.flops_per_unit(W.water_scene(res=64), W.water_config(), W.water_queries(512), nthreads=4)
    assert 9 <= w["flops_per_box"] <= 15          # 5 per axis, early exit on a miss
    assert 20 <= w["flops_per_triangle"] <= 60    # Moller-Trumbore with its divisions
    assert w["flops_per_ray"] > 300
    # the counts do not depend on the thread split
    w2 = oracle.flops_per_unit(W.water_scene(res=64), W.water_config(), W.water_queries(512), nthreads=1)
    assert w2["counts"] == w["counts"]
