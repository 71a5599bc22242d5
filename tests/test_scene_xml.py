"""Scene XML loading (the reference's scene format, subset in scene_xml.py):
a file describing the benchmark sphere scene must give the same scene as the
built-in description -- checked through the CPU oracle, bit for bit -- and
unsupported content must be refused, never dropped."""
import numpy as np
import pytest

SPHERE_XML = """<scene version="2.0.0">
  <integrator type="path_sms_ss">
    <boolean name="biased" value="true"/>
    <integer name="max_trials" value="16"/>
    <integer name="max_iterations" value="20"/>
    <float name="solver_threshold" value="1e-5"/>
  </integrator>
  <sensor type="perspective"><float name="fov" value="30"/></sensor>
  <shape type="sphere">
    <point name="center" x="0" y="0" z="0"/>
    <float name="radius" value="0.5"/>
    <transform name="to_world">
      <scale value="2"/>
      <translate x="0" y="0" z="1.5"/>
    </transform>
    <bsdf type="conductor">
      <float name="eta" value="0.2"/>
      <float name="k" value="3"/>
    </bsdf>
    <boolean name="caustic_caster_single" value="true"/>
  </shape>
  <shape type="sphere">
    <point name="center" x="5" y="5" z="-3"/>
    <float name="radius" value="0.5"/>
    <bsdf type="dielectric">
      <float name="int_ior" value="1.5"/>
      <string name="ext_ior" value="vacuum"/>
    </bsdf>
  </shape>
  <shape type="rectangle">
    <transform name="to_world"><scale value="4"/></transform>
    <bsdf type="diffuse"><rgb name="reflectance" value="0.5, 0.5, 0.5"/></bsdf>
    <boolean name="caustic_receiver" value="true"/>
  </shape>
  <emitter type="point">
    <point name="position" value="0, 0, 5"/>
    <spectrum name="intensity" value="100"/>
    <boolean name="caustic_emitter_single" value="true"/>
  </emitter>
</scene>
"""


def test_sphere_scene_from_xml_matches_builtin(sms, workloads, oracle, tmp_path):
    path = tmp_path / "sphere.xml"
    path.write_text(SPHERE_XML)
    desc, cfg, kind = sms.load_scene(path)
    assert kind == "path_sms_ss" and cfg.biased and cfg.max_trials == 16
    c, r, flip, b, flags = desc.spheres[0]
    np.testing.assert_allclose(c, (0, 0, 1.5))
    assert r == pytest.approx(1.0) and b.type == sms.BSDF_CONDUCTOR and b.k == pytest.approx(3.0)
    assert flags == sms.SHAPE_CAUSTIC_CASTER_SINGLE
    b2 = desc.spheres[1][3]
    assert b2.type == sms.BSDF_DIELECTRIC and b2.eta == pytest.approx(1.5) and desc.spheres[1][4] == 0
    P = desc.meshes[0][0]
    np.testing.assert_allclose(np.abs(P[:, :2]), 4.0)
    q = workloads.sphere_queries(16)
    ref = oracle.OracleScene(workloads.sphere_scene(conductor=True)).connect_batch(workloads.sphere_config(), q,
                                                                                  seed=3)
    got = oracle.OracleScene(desc).connect_batch(cfg, q, seed=3)
    for a, b_ in zip(ref[:3], got[:3]):
        np.testing.assert_array_equal(a, b_)
    assert (ref[1] > 0).sum() > 10


def test_obj_shape_and_area_emitter(sms, tmp_path):
    (tmp_path / "quad.obj").write_text("v -1 -1 0\nv 1 -1 0\nv 1 1 0\nv -1 1 0\nf 1 2 3 4\n")
    (tmp_path / "s.xml").write_text("""<scene version="2.0.0">
  <shape type="obj">
    <string name="filename" value="quad.obj"/>
    <transform name="to_world"><translate x="0" y="0" z="1"/></transform>
    <bsdf type="conductor"><rgb name="eta" value="0.2, 0.2, 0.2"/><rgb name="k" value="3, 3, 3"/></bsdf>
    <boolean name="caustic_caster_single" value="true"/>
  </shape>
  <shape type="sphere">
    <point name="center" x="0" y="0" z="10"/><float name="radius" value="0.1"/>
    <emitter type="area">
      <rgb name="radiance" value="1000, 1000, 1000"/>
      <boolean name="caustic_emitter_single" value="true"/>
    </emitter>
  </shape>
</scene>""")
    desc, cfg, kind = sms.load_scene(tmp_path / "s.xml")
    assert cfg is None and kind is None
    P, N, UV, F, b, flags = desc.meshes[0]
    np.testing.assert_allclose(P[:, 2], 1.0)
    assert b.type == sms.BSDF_CONDUCTOR and b.k == pytest.approx(3.0)
    assert np.allclose(N[:, 2], 1.0)              # recomputed normals of the quad
    assert len(desc.area_emitters) == 1 and desc.area_emitters[0][0] == 1


@pytest.mark.parametrize("body,what", [
    ('<shape type="cylinder"/>', "cylinder"),
    ('<shape type="sphere"><bsdf type="roughconductor"><string name="distribution" value="ggx"/></bsdf></shape>',
     "ggx"),
    ('<shape type="sphere"><bsdf type="plastic"/></shape>', "plastic"),
    ('<emitter type="envmap"/>', "envmap"),
    ('<shape type="sphere"><transform name="to_world"><rotate x="1" angle="3"/></transform></shape>',
     "translation and a uniform scale"),
    ('<shape type="sphere"><transform name="to_world"><shear value="1"/></transform></shape>', "shear"),
    ('<shape type="sphere"><bsdf type="dielectric"><string name="int_ior" value="unobtainium"/></bsdf></shape>',
     "unobtainium"),
])
def test_unsupported_content_is_refused(sms, tmp_path, body, what):
    (tmp_path / "bad.xml").write_text(f'<scene version="2.0.0">{body}</scene>')
    with pytest.raises(ValueError) as e:
        sms.load_scene(tmp_path / "bad.xml")
    assert what in str(e.value)


RENDER_XML = """<scene version="2.0.0">
  <integrator type="path_sms_ss">
    <integer name="max_depth" value="8"/>
    <integer name="rr_depth" value="3"/>
    <boolean name="biased_mnee" value="true"/>
    <boolean name="disable_reflected_emitters" value="true"/>
  </integrator>
  <sensor type="perspective">
    <float name="fov" value="40"/>
    <string name="fov_axis" value="y"/>
    <transform name="to_world">
      <lookat origin="0, -3.2, 3.6" target="0, 0, 0.4" up="0, 0, 1"/>
    </transform>
    <sampler type="independent"><integer name="sample_count" value="32"/></sampler>
    <film type="hdrfilm">
      <integer name="width" value="40"/><integer name="height" value="30"/>
      <rfilter type="box"/>
    </film>
  </sensor>
</scene>
"""


def test_render_setup_from_xml(sms, workloads, tmp_path):
    """Sensor, film, sampler and integrator parameters of a scene file."""
    path = tmp_path / "render.xml"
    path.write_text(RENDER_XML)
    cam, opt = sms.load_render_setup(path)
    ref = workloads.pool_camera(40, 30)
    np.testing.assert_allclose(cam.to_world, ref.to_world, atol=1e-6)
    assert (cam.width, cam.height, cam.fov, cam.fov_axis) == (40, 30, 40.0, "y")
    assert (opt.integrator, opt.max_depth, opt.rr_depth, opt.spp) == ("path_sms_ss", 8, 3, 32)
    assert opt.biased_mnee and opt.disable_reflected_emitters
    assert opt.rfilter == "box"
    # the film's filter: gaussian by default (the reference's), with its stddev
    path.write_text(RENDER_XML.replace('<rfilter type="box"/>', ''))
    assert sms.load_render_setup(path)[1].rfilter == "gaussian"
    path.write_text(RENDER_XML.replace('<rfilter type="box"/>',
                                       '<rfilter type="gaussian"><float name="stddev" value="0.3"/></rfilter>'))
    opt = sms.load_render_setup(path)[1]
    assert opt.rfilter == "gaussian" and abs(opt.rfilter_stddev - 0.3) < 1e-7
    assert opt.to_c().rfilter == 1
    path.write_text(RENDER_XML.replace('<rfilter type="box"/>', '<rfilter type="tent"/>'))
    with pytest.raises(ValueError):
        sms.load_render_setup(path)
    path.write_text(RENDER_XML.replace('type="path_sms_ss"', 'type="bdpt"'))
    with pytest.raises(ValueError):
        sms.load_render_setup(path)
    # the filtered comparison integrators; path_filtered_ms defaults to 2 bounces
    path.write_text(RENDER_XML.replace('type="path_sms_ss"', 'type="path_filtered_ms"'))
    cam, opt = sms.load_render_setup(path)
    assert opt.integrator == "path_filtered_ms"
    _, cfg, kind = sms.load_scene(path)
    assert kind == "path_filtered_ms" and cfg.bounces == 2
    # equal-time rendering parameters of the integrator (integrator.cpp:35-41)
    path.write_text(RENDER_XML.replace('<integer name="rr_depth" value="3"/>',
                                       '<integer name="rr_depth" value="3"/><float name="timeout" value="2.5"/>'
                                       '<integer name="samples_per_pass" value="4"/>'))
    cam, opt = sms.load_render_setup(path)
    assert (opt.timeout, opt.samples_per_pass) == (2.5, 4)


TEASER_INTEGRATOR = """<integrator type="path_sms_teaser">
    <integer name="max_depth" value="6"/>
    <boolean name="caustics_biased" value="true"/>
    <integer name="caustics_max_trials" value="24"/>
    <integer name="caustics_bounces" value="3"/>
    <float name="caustics_solver_threshold" value="2e-5"/>
    <boolean name="glints_biased" value="false"/>
    <integer name="glints_max_trials" value="48"/>
    <integer name="glints_max_iterations" value="12"/>
    <boolean name="non_sms_paths_enabled" value="false"/>
    <boolean name="glints_enabled" value="false"/>
  </integrator>"""


def test_teaser_integrator_from_xml(sms, tmp_path):
    """path_sms_teaser (path_sms_teaser.cpp:60-81): the caustics_* block is the
    context's SMSConfig (bounces default 2), the glints_* block and the
    switches are render options."""
    path = tmp_path / "teaser.xml"
    i0, i1 = RENDER_XML.index("<integrator"), RENDER_XML.index("</integrator>") + len("</integrator>")
    path.write_text(RENDER_XML[:i0] + TEASER_INTEGRATOR + RENDER_XML[i1:])
    _, cfg, kind = sms.load_scene(path)
    assert kind == "path_sms_teaser"
    assert cfg.biased and cfg.max_trials == 24 and cfg.bounces == 3 and abs(cfg.solver_threshold - 2e-5) < 1e-12
    assert cfg.max_iterations == 20     # glints_max_iterations is not a caustics parameter
    cam, opt = sms.load_render_setup(path)
    assert opt.integrator == "path_sms_teaser" and opt.max_depth == 6
    assert opt.caustics_enabled and not opt.glints_enabled and not opt.non_sms_paths_enabled
    assert opt.glints.max_trials == 48 and opt.glints.max_iterations == 12 and not opt.glints.biased
    c = opt.to_c()
    assert c.integrator == 6 and c.glints.max_trials == 48 and c.non_sms_paths_enabled == 0
    # defaults: bounces 2 for the caustics block
    path.write_text(RENDER_XML[:i0] + '<integrator type="path_sms_teaser"/>' + RENDER_XML[i1:])
    _, cfg, _ = sms.load_scene(path)
    assert cfg.bounces == 2 and not cfg.biased and cfg.max_trials == -1


def test_filtered_teaser_integrator_from_xml(sms, tmp_path):
    """path_filtered_teaser (path_filtered_teaser.cpp:45-48): the filter's
    chain length multi_caustic_bounces (default 2) is the SMSConfig's bounces;
    non_sms_paths_enabled is a render option."""
    path = tmp_path / "ft.xml"
    i0, i1 = RENDER_XML.index("<integrator"), RENDER_XML.index("</integrator>") + len("</integrator>")
    body = """<integrator type="path_filtered_teaser">
    <integer name="max_depth" value="7"/>
    <integer name="multi_caustic_bounces" value="3"/>
    <boolean name="non_sms_paths_enabled" value="false"/>
  </integrator>"""
    path.write_text(RENDER_XML[:i0] + body + RENDER_XML[i1:])
    _, cfg, kind = sms.load_scene(path)
    assert kind == "path_filtered_teaser" and cfg.bounces == 3
    cam, opt = sms.load_render_setup(path)
    assert opt.integrator == "path_filtered_teaser" and opt.max_depth == 7 and not opt.non_sms_paths_enabled
    assert opt.to_c().integrator == 7
    path.write_text(RENDER_XML[:i0] + '<integrator type="path_filtered_teaser"/>' + RENDER_XML[i1:])
    _, cfg, _ = sms.load_scene(path)
    assert cfg.bounces == 2
    assert sms.load_render_setup(path)[1].non_sms_paths_enabled


def test_twosided_bsdf_from_xml(sms, tmp_path):
    """<bsdf type="twosided"> around a diffuse or conductor bsdf sets the
    twosided flag (twosided.cpp); around a dielectric it is refused."""
    body = '''<scene version="2.0.0">
      <shape type="rectangle"><bsdf type="twosided"><bsdf type="diffuse">
        <rgb name="reflectance" value="0.2, 0.3, 0.4"/></bsdf></bsdf></shape>
      <shape type="rectangle"><bsdf type="conductor"/></shape>
    </scene>'''
    (tmp_path / "t.xml").write_text(body)
    desc, _, _ = sms.load_scene(tmp_path / "t.xml")
    b0, b1 = desc.meshes[0][4], desc.meshes[1][4]
    assert b0.twosided and b0.type == sms.BSDF_DIFFUSE and b0.albedo == (0.2, 0.3, 0.4)
    assert not b1.twosided
    assert b0.to_c().twosided == 1
    sms.Scene(desc)
    (tmp_path / "d.xml").write_text(body.replace('<bsdf type="diffuse">', '<bsdf type="dielectric">'))
    with pytest.raises(ValueError, match="dielectric"):
        sms.load_scene(tmp_path / "d.xml")
    d = sms.SceneDesc()
    d.add_sphere((0, 0, 0), 1.0, sms.Bsdf(sms.BSDF_DIELECTRIC, 1.5, twosided=True))
    with pytest.raises(sms.SMSError):
        sms.Scene(d)


def test_rough_bsdfs_from_xml(sms, tmp_path):
    body = """<scene version="2.0.0">
      <shape type="sphere"><float name="radius" value="1"/>
        <bsdf type="roughdielectric"><float name="alpha" value="0.3"/><float name="int_ior" value="1.5"/>
          <float name="ext_ior" value="1.0"/></bsdf></shape>
      <shape type="sphere"><float name="radius" value="1"/>
        <bsdf type="roughconductor"><float name="alpha" value="0.05"/></bsdf></shape>
    </scene>"""
    (tmp_path / "rough.xml").write_text(body)
    desc, _, _ = sms.load_scene(tmp_path / "rough.xml")
    b0, b1 = desc.spheres[0][3], desc.spheres[1][3]
    assert b0.type == sms.BSDF_DIELECTRIC and b0.alpha == pytest.approx(0.3) and b0.eta == pytest.approx(1.5)
    assert b1.type == sms.BSDF_CONDUCTOR and b1.alpha == pytest.approx(0.05)


def test_roughplastic_bsdf_from_xml(sms, tmp_path):
    """<bsdf type="roughplastic"> (roughplastic.cpp:148-183): defaults
    polypropylene in air, alpha 0.1, diffuse_reflectance 0.5; Beckmann only;
    twosided may wrap it."""
    body = '''<scene version="2.0.0">
      <shape type="rectangle"><bsdf type="roughplastic"/></shape>
      <shape type="rectangle"><bsdf type="twosided"><bsdf type="roughplastic">
        <float name="alpha" value="0.3"/><float name="int_ior" value="1.5"/><float name="ext_ior" value="1.0"/>
        <rgb name="diffuse_reflectance" value="0.1, 0.2, 0.3"/><boolean name="nonlinear" value="true"/>
      </bsdf></bsdf></shape>
    </scene>'''
    (tmp_path / "t.xml").write_text(body)
    desc, _, _ = sms.load_scene(tmp_path / "t.xml")
    b0, b1 = desc.meshes[0][4], desc.meshes[1][4]
    assert b0.type == sms.BSDF_ROUGHPLASTIC and b0.alpha == pytest.approx(0.1)
    assert b0.eta == pytest.approx(1.49 / 1.000277) and b0.albedo == (0.5, 0.5, 0.5) and not b0.nonlinear
    assert b1.twosided and b1.nonlinear and b1.alpha == pytest.approx(0.3) and b1.eta == pytest.approx(1.5)
    assert b1.albedo == (0.1, 0.2, 0.3)
    sms.Scene(desc)
    (tmp_path / "g.xml").write_text(body.replace('<bsdf type="roughplastic"/>',
                                                 '<bsdf type="roughplastic"><string name="distribution" '
                                                 'value="ggx"/></bsdf>'))
    with pytest.raises(ValueError, match="beckmann"):
        sms.load_scene(tmp_path / "g.xml")
