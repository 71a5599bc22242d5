"""The oracle pinned against known answers (no GPU).

* PCG32 against O'Neill's published demo stream (the reference's sampler RNG,
  include/mitsuba/core/random.h:50-52);
* Fresnel against the values the reference's own test asserts
  (src/librender/tests/test_fresnel.py:7-39) and the conductor/dielectric
  agreement of test03 there;
* the uniform-sphere warp (include/mitsuba/core/warp.h:262-267);
* converged walks against specular solutions derived independently in FP64
  (tests/golden/sphere_analytic.json), tolerance 1e-5 at scene scale 1;
* bit-exact regression of small estimator runs (tests/golden/oracle_small.npz).
"""
import ctypes as C
import json
import math
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def kat():
    return json.loads((GOLDEN / "kat.json").read_text())


def test_pcg32_reference_stream(oracle, workloads, kat):
    lib = oracle.load()
    out = np.zeros(6, np.uint32)
    lib.oracle_pcg32(42, 54, 6, out.ctypes.data)
    assert out.tolist() == kat["pcg32_42_54_u32"]
    r = workloads.Pcg32(42, 54)
    assert [r.next_u32() for _ in range(6)] == kat["pcg32_42_54_u32"]


def test_pcg32_float_streams_agree(oracle, workloads):
    lib = oracle.load()
    f = np.zeros(5, np.float32)
    lib.oracle_pcg32_f32(7, 3, 5, f.ctypes.data)
    v = workloads.pcg32_streams_f32(7, np.array([3], np.uint64), 5).ravel()
    assert np.array_equal(f, v)
    r = workloads.Pcg32(7, 3)
    assert np.array_equal(np.float32([r.next_f32() for _ in range(5)]), f)
    assert np.all((f >= 0) & (f < 1))


def test_fresnel_reference_values(oracle, kat):
    lib = oracle.load()
    ct = C.c_float()
    for cos_i, eta, F_ref, ct_ref in kat["fresnel"]:
        F = lib.oracle_fresnel(cos_i, eta, C.byref(ct))
        assert F == pytest.approx(F_ref, abs=1e-5), (cos_i, eta)
        assert ct.value == pytest.approx(ct_ref, abs=1e-5), (cos_i, eta)


def test_fresnel_conductor_matches_dielectric_for_real_ior(oracle):
    # test_fresnel.py:60-72 (test03_fresnel_conductor)
    lib = oracle.load()
    for th in np.linspace(0, math.pi / 2, 20):
        c = math.cos(th)
        for eta in (1.5, 1 / 1.5):
            a = lib.oracle_fresnel(c, eta, None)
            b = lib.oracle_fresnel_conductor(c, eta, 0.0)
            assert a == pytest.approx(b, abs=1e-5)


def test_snell(oracle):
    # test_fresnel.py:75-83 (test04_snell)
    lib = oracle.load()
    ct = C.c_float()
    for th in np.linspace(0, math.pi / 2, 20):
        lib.oracle_fresnel(math.cos(th), 1.5, C.byref(ct))
        assert math.sin(th) - 1.5 * math.sin(math.acos(ct.value)) == pytest.approx(0, abs=1e-5)


def test_uniform_sphere(oracle, kat):
    lib = oracle.load()
    out = (C.c_float * 3)()
    for u, v, x, y, z in kat["uniform_sphere"]:
        lib.oracle_uniform_sphere(u, v, out)
        assert list(out) == pytest.approx([x, y, z], abs=1e-6)


@pytest.mark.parametrize("mode", ["reflect", "refract"])
def test_walks_converge_to_analytic_solutions(sms, workloads, oracle, mode):
    W = workloads
    cases = [c for c in json.loads((GOLDEN / "sphere_analytic.json").read_text()) if c["mode"] == mode]
    assert cases
    desc = W.sphere_scene(conductor=(mode == "reflect"))
    o = oracle.OracleScene(desc)
    xy = np.array([[c["x"][0], 0.0] for c in cases for _ in (1, -1)], np.float32)
    q = W.plane_queries(xy)
    n = q.shape[1]
    w = np.zeros((8, n), np.float32)
    w[2] = 5.0
    for i, c in enumerate(cases):
        for j, s in enumerate((1, -1)):
            th = c["theta"] + 0.03 * s
            w[3:6, 2 * i + j] = [math.sin(th), 0.0, 1.5 - math.cos(th)]
    out = o.walk_batch(sms.SMSConfig(), 0, q, w)
    sol = np.array([c["solution"] for c in cases for _ in (1, -1)]).T
    ok = out[0] > 0.5
    assert ok.mean() >= 0.9
    err = np.linalg.norm(out[2:5, ok] - sol[:, ok], axis=0)
    assert err.max() < 1e-5


def test_oracle_regression(sms, workloads, oracle):
    W = workloads
    ref = np.load(GOLDEN / "oracle_small.npz")
    for cond in (False, True):
        tag = "cond" if cond else "glass"
        v, c, w, st = oracle.OracleScene(W.sphere_scene(conductor=cond)).connect_batch(
            W.sphere_config(), W.sphere_queries(16), seed=1, nthreads=2)
        assert np.array_equal(c, ref[f"sphere_{tag}_count"])
        np.testing.assert_allclose(v, ref[f"sphere_{tag}_value"], rtol=1e-6, atol=1e-9)
    v, c, w, st = oracle.OracleScene(W.water_scene(res=64)).connect_batch(
        W.water_config(), W.water_queries(256), seed=5, nthreads=2)
    assert np.array_equal(c, ref["water64_count"])
    assert np.array_equal(w, ref["water64_walks"])
    np.testing.assert_allclose(v, ref["water64_value"], rtol=1e-6, atol=1e-9)


def test_nan_walks_are_misses(sms, workloads, oracle):
    """A start point at the shading point gives a NaN direction: the walk fails."""
    W = workloads
    o = oracle.OracleScene(W.sphere_scene())
    q = W.sphere_queries(1)
    w = np.zeros((8, 1), np.float32)
    w[2] = 5.0
    w[3:6, 0] = q[0:3, 0]
    w[3:6, 0][2] = 1e-30  # non-zero so it counts as an explicit start, ~ the shading point
    out = o.walk_batch(sms.SMSConfig(), 0, q, w)
    assert out[0, 0] == 0.0
