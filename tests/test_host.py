"""Host-side logic of the library (no GPU): ABI exports, config parsing, scene
validation, workload generators."""
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_library_exports_every_declared_symbol(sms):
    lib = sms.load_library()
    header = (ROOT / "include" / "sms_gb300.h").read_text()
    names = set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(sms_[a-z_0-9]+)\s*\(", header, re.M))
    assert len(names) >= 40
    for n in sorted(names):
        assert hasattr(lib, n), n


def test_config_defaults_match_reference(sms):
    c = sms.default_config()
    # include/mitsuba/render/manifold.h:11-45
    assert (c.biased, c.twostage, c.halfvector_constraints, c.mnee_init) == (False,) * 4
    assert c.step_scale == 1.0 and c.max_iterations == 20 and c.max_trials == -1
    assert c.solver_threshold == pytest.approx(1e-5) and c.uniqueness_threshold == pytest.approx(1e-4)
    assert c.bounces == 1


def test_parse_integrator_xml(sms):
    xml = """<scene><integrator type="path_sms_ss">
        <integer name="max_depth" value="6"/>
        <boolean name="biased" value="true"/>
        <boolean name="halfvector_constraints" value="false"/>
        <integer name="max_iterations" value="30"/>
        <float name="solver_threshold" value="0.00001"/>
        <float name="uniqueness_threshold" value="0.00002"/>
        <integer name="max_trials" value="16"/>
        <float name="step_scale" value="0.5"/>
    </integrator></scene>"""
    c, t = sms.SMSConfig.from_xml(xml)
    assert t == "path_sms_ss"
    assert c.biased and c.max_iterations == 30 and c.max_trials == 16
    assert c.uniqueness_threshold == pytest.approx(2e-5) and c.step_scale == 0.5
    c, t = sms.SMSConfig.from_xml('<integrator type="path_sms_ms"></integrator>')
    assert t == "path_sms_ms" and c.bounces == 2
    c, t = sms.SMSConfig.from_xml(
        '<integrator type="path_sms_glints"><boolean name="glints_vectorized" value="true"/>'
        '<boolean name="sms_strategy_only" value="true"/></integrator>')
    assert c.glints_vectorized and c.sms_strategy_only and not c.bsdf_strategy_only


@pytest.mark.parametrize("xml", [
    "<scene/>",
    '<integrator><boolean name="biased" value="true"/></integrator>',
    '<integrator type="path_sms_ss"><boolean name="biased" value="maybe"/></integrator>',
    '<integrator type="path_sms_ss"><integer name="max_trials" value="1.5"/></integrator>',
])
def test_parse_errors(sms, xml):
    with pytest.raises(sms.SMSError) as e:
        sms.SMSConfig.from_xml(xml)
    assert e.value.status == 5


def test_scene_validation(sms):
    d = sms.SceneDesc()
    d.add_mesh(np.zeros((3, 3)), np.array([[0, 1, 5]]), sms.Bsdf(sms.BSDF_DIELECTRIC, 1.5))
    with pytest.raises(sms.SMSError):
        sms.Scene(d)
    d = sms.SceneDesc()
    m = d.add_mesh(np.eye(3), np.array([[0, 1, 2]]), sms.Bsdf())
    d.add_area_emitter(m, (1, 1, 1))
    with pytest.raises(sms.SMSError) as e:
        sms.Scene(d)
    assert e.value.status == 4
    d = sms.SceneDesc()
    d.add_sphere((0, 0, 0), 1.0, sms.Bsdf(7))
    with pytest.raises(sms.SMSError):
        sms.Scene(d)


def test_context_without_device_fails_loudly(sms, workloads):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is visible")
    with pytest.raises(sms.SMSError) as e:
        sms.Context(sms.Scene(workloads.sphere_scene()), sms.SMSConfig())
    assert e.value.status in (2, 6)


def test_water_workload_shapes(workloads):
    W = workloads
    d = W.water_scene()
    P, N, UV, F, b, flags = d.meshes[0]
    assert P.shape == (512 * 512, 3) and F.shape == (2 * 511 * 511, 3)
    assert np.allclose(np.linalg.norm(N, axis=1), 1, atol=1e-5)
    waves = W.water_params()
    assert len(waves) == 32
    for a, kx, ky, ph in waves:
        assert 0.002 <= a <= 0.02 and 2 <= np.hypot(kx, ky) <= 40 and 0 <= ph <= 2 * np.pi
    q = W.water_queries(1000)
    assert q.shape == (16, 1000) and np.all(np.abs(q[:2]) <= 1)
    q2 = W.water_queries(10, first=990)
    assert np.array_equal(q2, q[:, 990:])
