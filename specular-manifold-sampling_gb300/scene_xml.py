"""Scene loader for the subset of the reference's XML scene format the SMS path
needs (Mitsuba 2 scene files, as the paper's scenes are written).

Recognised elements (everything else raises ValueError, so a scene is never
silently half-loaded):

  <shape type="sphere">   center (point), radius (float), flip_normals
  <shape type="obj">      filename (relative to the XML file), face_normals,
                          flip_tex_coords (src/shapes/obj.cpp:90-110)
  <shape type="rectangle"> the two triangles of [-1,1]^2 at z = 0 with uv
                          (src/shapes/rectangle.cpp)
      shape flags: caustic_caster_single, caustic_caster_multi,
      caustic_bouncer, caustic_receiver, glinty (src/librender/shape.cpp:78-82);
      <transform name="to_world"> with translate / scale / matrix children
      (spheres: translate and uniform scale only);
      nested <bsdf>: dielectric (int_ior / ext_ior, names from
      include/mitsuba/render/ior.h), conductor (eta, k), diffuse (reflectance),
      roughdielectric / roughconductor (isotropic Beckmann alpha),
      roughplastic (int_ior / ext_ior, diffuse_reflectance, Beckmann alpha,
      nonlinear), twosided around one diffuse, conductor or roughplastic bsdf
      (src/bsdfs/twosided.cpp),
      normalmap around any of these (filename of an OpenEXR or PNG RGB normal
      map, tiles, lean_fallback with lean_fallback_alpha and grey eta / k;
      src/bsdfs/normalmap.cpp:24-58; one normal-mapped shape per scene); a
      top-level <bsdf id="..."> referenced by <ref id="..."/>;
      no bsdf -> diffuse (shape.cpp:73-74);
      nested <emitter type="area"> with radiance (spheres only)
  <emitter type="point">  position (point), intensity (spectrum / rgb / float)
      emitter flags: caustic_emitter_single, caustic_emitter_multi
      (src/librender/emitter.cpp:9-10)
  <integrator type="path_sms_*"> -> SMSConfig (sms_config_parse_xml)
  <sensor>, <film>, <sampler> are accepted and ignored (not on this path).

Returns (SceneDesc, SMSConfig or None, integrator type or None).

load_render_setup reads the rendering side of the same file:
  <sensor type="perspective">  fov, fov_axis, near_clip, far_clip,
      <transform name="to_world"> (lookat / translate / scale / rotate / matrix),
      <film> width, height (hdrfilm defaults 768 x 576) and its <rfilter> (box,
      or gaussian with stddev: the default), <sampler> sample_count
      (independent sampler default 4)   (src/sensors/perspective.cpp)
  <integrator type="path|path_sms_ss|path_sms_ms|path_sms_glints|path_filtered_ss|path_filtered_ms|
                    path_sms_teaser|path_filtered_teaser">  max_depth, rr_depth
      (src/librender/integrator.cpp:300-320), samples_per_pass, timeout,
      glint_diff_scale_factor_clamp (:35-41), disable_reflected_emitters,
      biased_mnee (path_sms_ss.cpp:59-60); path_sms_teaser's caustics_enabled,
      glints_enabled, non_sms_paths_enabled and glints_* block
      (path_sms_teaser.cpp:60-81; its caustics_* block is the SMSConfig);
      path_filtered_teaser's non_sms_paths_enabled and multi_caustic_bounces
      (the SMSConfig's bounces; path_filtered_teaser.cpp:45-48)
and returns (Camera, RenderOptions).
"""
from __future__ import annotations

import math
import xml.etree.ElementTree as ET
from pathlib import Path

import numpy as np

# include/mitsuba/render/ior.h:22-49
IOR = {"vacuum": 1.0, "helium": 1.000036, "hydrogen": 1.000132, "air": 1.000277, "carbon dioxide": 1.00045,
       "water": 1.3330, "acetone": 1.36, "ethanol": 1.361, "carbon tetrachloride": 1.461, "glycerol": 1.4729,
       "benzene": 1.501, "silicone oil": 1.52045, "bromine": 1.661, "water ice": 1.31, "fused quartz": 1.458,
       "pyrex": 1.470, "acrylic glass": 1.49, "polypropylene": 1.49, "bk7": 1.5046, "sodium chloride": 1.544,
       "amber": 1.55, "pet": 1.5750, "diamond": 2.419}

_IGNORED = {"sensor", "film", "sampler", "default"}
_INTEGRATOR_TYPES = {"path", "path_sms_ss", "path_sms_ms", "path_filtered_ss", "path_filtered_ms", "path_sms_glints",
                     "path_sms_teaser", "path_filtered_teaser"}


def _props(el):
    """name -> (tag, element) of the direct property children."""
    return {c.get("name"): (c.tag, c) for c in el if c.get("name") is not None}


def _bool(p, name, default=False):
    if name not in p:
        return default
    return p[name][1].get("value", "false").strip().lower() == "true"


def _float(p, name, default):
    if name not in p:
        return default
    tag, el = p[name]
    v = el.get("value")
    if tag == "string":
        if v.lower() not in IOR:
            raise ValueError(f"unknown index of refraction name '{v}'")
        return IOR[v.lower()]
    return float(v)


def _spectrum(p, name, default):
    """rgb / spectrum / float -> 3 floats (a single value is grey)."""
    if name not in p:
        return default
    tag, el = p[name]
    v = el.get("value")
    if tag in ("float", "spectrum") and v is not None and "," not in v and len(v.split()) == 1:
        x = float(v)
        return (x, x, x)
    vals = [float(x) for x in v.replace(",", " ").split()]
    if len(vals) != 3:
        raise ValueError(f"'{name}': expected 1 or 3 values")
    return tuple(vals)


def _point(p, name, default):
    if name not in p:
        return default
    el = p[name][1]
    if el.get("value") is not None:
        return tuple(float(x) for x in el.get("value").replace(",", " ").split())
    return (float(el.get("x", 0)), float(el.get("y", 0)), float(el.get("z", 0)))


def _transform(el):
    """4x4 matrix of a <transform> element (translate, scale, matrix)."""
    M = np.eye(4)
    for c in el:
        if c.tag == "translate":
            T = np.eye(4)
            if c.get("value"):
                T[:3, 3] = [float(x) for x in c.get("value").replace(",", " ").split()]
            else:
                T[:3, 3] = [float(c.get(k, 0)) for k in "xyz"]
            M = T @ M
        elif c.tag == "scale":
            S = np.eye(4)
            if c.get("value") and len(c.get("value").replace(",", " ").split()) == 1:
                S[:3, :3] *= float(c.get("value"))
            elif c.get("value"):
                S[np.arange(3), np.arange(3)] = [float(x) for x in c.get("value").replace(",", " ").split()]
            else:
                S[np.arange(3), np.arange(3)] = [float(c.get(k, 1)) for k in "xyz"]
            M = S @ M
        elif c.tag == "matrix":
            A = np.array([float(x) for x in c.get("value").replace(",", " ").split()]).reshape(4, 4)
            M = A @ M
        elif c.tag == "rotate":
            # rotation by `angle` degrees about the axis (x, y, z) (Rodrigues)
            if c.get("value"):
                ax = np.array([float(x) for x in c.get("value").replace(",", " ").split()])
            else:
                ax = np.array([float(c.get(k, 0)) for k in "xyz"])
            ax = ax / np.linalg.norm(ax)
            a = math.radians(float(c.get("angle", 0)))
            K = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]])
            R = np.eye(4)
            R[:3, :3] = np.eye(3) + math.sin(a) * K + (1 - math.cos(a)) * (K @ K)
            M = R @ M
        elif c.tag == "lookat":
            # include/mitsuba/core/transform.h look_at: columns left, up, forward, origin
            vec = lambda k: np.array([float(x) for x in c.get(k).replace(",", " ").split()])
            o, t = vec("origin"), vec("target")
            up = vec("up") if c.get("up") else np.array([0.0, 1.0, 0.0])
            d = (t - o) / np.linalg.norm(t - o)
            left = np.cross(up, d)
            left /= np.linalg.norm(left)
            new_up = np.cross(d, left)
            L = np.eye(4)
            L[:3, 0], L[:3, 1], L[:3, 2], L[:3, 3] = left, new_up, d, o
            M = L @ M
        else:
            raise ValueError(f"unsupported transform operation <{c.tag}>")
    return M


def _bsdf_nm(sms, el, refs, base):
    """(Bsdf, normal map or None) of a <bsdf> element; the normal map is
    (float16 slopes (res, res, 2), tiles) of a normalmap BSDF."""
    if el is not None and el.get("type") == "normalmap":
        p = _props(el)
        if not _bool(p, "use_slopes", True):
            raise ValueError("normalmap with use_slopes = false is not supported")
        lean_fb = None
        if _bool(p, "lean_fallback"):
            # normalmap.cpp:46-55: base roughness and the fallback's complex IOR
            mat = p.get("lean_fallback_material", (None, None))[1]
            if mat is not None and mat.get("value", "none").lower() != "none":
                raise ValueError("named lean_fallback_material is not supported; give eta and k")
            eta, k = _spectrum(p, "eta", (0.0,) * 3), _spectrum(p, "k", (1.0,) * 3)
            if len(set(eta)) != 1 or len(set(k)) != 1:
                raise ValueError("lean_fallback: eta and k must be grey (one value)")
            lean_fb = (_float(p, "lean_fallback_alpha", 0.0001), eta[0], k[0])
        if "filename" not in p:
            raise ValueError("normalmap without a filename")
        from .image_io import normalmap_slopes
        inner = [c for c in el if c.tag in ("bsdf", "ref")]
        if len(inner) != 1:
            raise ValueError("normalmap needs exactly one nested bsdf")
        b, nm = _bsdf_nm(sms, _deref(inner[0], refs), refs, base)
        if nm is not None:
            raise ValueError("nested normal maps are not supported")
        return b, (normalmap_slopes(base / p["filename"][1].get("value")), _float(p, "tiles", 1.0), lean_fb)
    return _bsdf(sms, el, refs), None


def _deref(el, refs):
    if el is not None and el.tag == "ref":
        rid = el.get("id")
        if rid not in refs:
            raise ValueError(f"unknown bsdf reference '{rid}'")
        return refs[rid]
    return el


def _bsdf(sms, el, refs=None):
    el = _deref(el, refs or {})
    if el is None:
        return sms.Bsdf(sms.BSDF_DIFFUSE, 1.0, 0.0, (0.5, 0.5, 0.5))
    t = el.get("type")
    p = _props(el)
    if t == "normalmap":
        raise ValueError("a normalmap bsdf is only supported directly on a shape")
    if t == "twosided":
        # twosided.cpp: one nested BSDF for both sides (two different ones are
        # not supported), no transmission
        inner = [c for c in el if c.tag in ("bsdf", "ref")]
        if len(inner) > 1:
            raise ValueError("twosided with two different nested bsdfs is not supported")
        b = _bsdf(sms, inner[0] if inner else None, refs)
        if b.type == sms.BSDF_DIELECTRIC:
            raise ValueError("twosided cannot wrap a dielectric (transmission)")
        b.twosided = True
        return b
    if t == "dielectric":
        # dielectric.cpp:177-186: eta = int_ior / ext_ior, defaults bk7 / air
        return sms.Bsdf(sms.BSDF_DIELECTRIC, _float(p, "int_ior", 1.5046) / _float(p, "ext_ior", 1.000277))
    if t in ("conductor", "roughconductor") and p.get("material", (None, None))[1] is not None:
        if p["material"][1].get("value", "none").lower() != "none":
            raise ValueError("named conductor materials are not supported; give eta and k")
    if t == "conductor":
        eta, k = _spectrum(p, "eta", (0.0,) * 3), _spectrum(p, "k", (1.0,) * 3)
        return sms.Bsdf(sms.BSDF_CONDUCTOR, float(np.mean(eta)), float(np.mean(k)))
    if t in ("roughdielectric", "roughconductor"):
        # roughdielectric.cpp / roughconductor.cpp: isotropic Beckmann only
        dist = p["distribution"][1].get("value").lower() if "distribution" in p else "beckmann"
        if dist != "beckmann":
            raise ValueError(f"microfacet distribution '{dist}' is not supported (beckmann only)")
        if "alpha_u" in p or "alpha_v" in p:
            raise ValueError("anisotropic roughness (alpha_u / alpha_v) is not supported")
        alpha = _float(p, "alpha", 0.1)
        if t == "roughdielectric":
            return sms.Bsdf(sms.BSDF_DIELECTRIC, _float(p, "int_ior", 1.5046) / _float(p, "ext_ior", 1.000277),
                            alpha=alpha)
        eta, k = _spectrum(p, "eta", (0.0,) * 3), _spectrum(p, "k", (1.0,) * 3)
        return sms.Bsdf(sms.BSDF_CONDUCTOR, float(np.mean(eta)), float(np.mean(k)), alpha=alpha)
    if t == "diffuse":
        return sms.Bsdf(sms.BSDF_DIFFUSE, 1.0, 0.0, _spectrum(p, "reflectance", (0.5,) * 3))
    if t == "roughplastic":
        # roughplastic.cpp:148-183: isotropic Beckmann coating over a diffuse base
        dist = p["distribution"][1].get("value").lower() if "distribution" in p else "beckmann"
        if dist != "beckmann":
            raise ValueError(f"microfacet distribution '{dist}' is not supported (beckmann only)")
        if "alpha_u" in p or "alpha_v" in p:
            raise ValueError("anisotropic roughness (alpha_u / alpha_v) is not supported")
        if "specular_reflectance" in p and _spectrum(p, "specular_reflectance", (1.0,) * 3) != (1.0, 1.0, 1.0):
            raise ValueError("roughplastic specular_reflectance other than 1 is not supported")
        eta = _float(p, "int_ior", 1.49) / _float(p, "ext_ior", 1.000277)
        return sms.Bsdf(sms.BSDF_ROUGHPLASTIC, eta, 0.0, _spectrum(p, "diffuse_reflectance", (0.5,) * 3),
                        alpha=_float(p, "alpha", 0.1), nonlinear=_bool(p, "nonlinear"))
    raise ValueError(f"unsupported bsdf type '{t}'")


def _flags(sms, p):
    f = 0
    for name, bit in (("caustic_receiver", sms.SHAPE_CAUSTIC_RECEIVER),
                      ("caustic_caster_single", sms.SHAPE_CAUSTIC_CASTER_SINGLE),
                      ("caustic_caster_multi", sms.SHAPE_CAUSTIC_CASTER_MULTI),
                      ("caustic_bouncer", sms.SHAPE_CAUSTIC_BOUNCER), ("glinty", sms.SHAPE_GLINTY)):
        if _bool(p, name):
            f |= bit
    return f


def _emitter_flags(sms, p):
    f = 0
    if _bool(p, "caustic_emitter_single"):
        f |= sms.EMITTER_CAUSTIC_SINGLE
    if _bool(p, "caustic_emitter_multi"):
        f |= sms.EMITTER_CAUSTIC_MULTI
    return f


def load_scene_xml(sms, path):
    path = Path(path)
    root = ET.parse(path).getroot()
    if root.tag != "scene":
        raise ValueError("not a <scene> document")
    desc = sms.SceneDesc()
    config, itype = None, None
    refs = {c.get("id"): c for c in root if c.tag == "bsdf" and c.get("id") is not None}
    for el in root:
        if el.tag in _IGNORED:
            continue
        if el.tag == "integrator":
            config, itype = sms.SMSConfig.from_xml(ET.tostring(el, encoding="unicode"))
            continue
        if el.tag == "bsdf":
            if el.get("id") is None:
                raise ValueError("a top-level <bsdf> needs an id")
            continue
        p = _props(el)
        if el.tag == "emitter":
            if el.get("type") != "point":
                raise ValueError(f"unsupported top-level emitter type '{el.get('type')}'")
            desc.add_point_emitter(_point(p, "position", (0.0, 0.0, 0.0)), _spectrum(p, "intensity", (1.0,) * 3),
                                   _emitter_flags(sms, p))
            continue
        if el.tag != "shape":
            raise ValueError(f"unsupported element <{el.tag}>")
        t = el.get("type")
        bsdf_el = next((c for c in el if c.tag in ("bsdf", "ref")), None)
        tr_el = next((c for c in el if c.tag == "transform" and c.get("name") == "to_world"), None)
        M = _transform(tr_el) if tr_el is not None else np.eye(4)
        flags = _flags(sms, p)
        b, nm = _bsdf_nm(sms, _deref(bsdf_el, refs), refs, path.parent)
        if t == "sphere":
            c = np.array(_point(p, "center", (0.0, 0.0, 0.0)), np.float64)
            r = _float(p, "radius", 1.0)
            A = M[:3, :3]
            s = np.cbrt(abs(np.linalg.det(A)))
            if not np.allclose(A, s * np.eye(3), atol=1e-6 * max(1.0, s)):
                raise ValueError("sphere to_world must be a translation and a uniform scale")
            centre = A @ c + M[:3, 3]
            sid = desc.add_sphere(tuple(centre), r * s, b, flags, flip=_bool(p, "flip_normals"))
        elif t in ("obj", "rectangle"):
            if t == "obj":
                P, F, N, UV = sms.load_obj(path.parent / p["filename"][1].get("value"),
                                           _bool(p, "face_normals"), _bool(p, "flip_tex_coords", True))
            else:
                P = np.array([[-1, -1, 0], [1, -1, 0], [1, 1, 0], [-1, 1, 0]], np.float32)
                F = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
                UV = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
                N = None
            Ph = np.concatenate([P.astype(np.float64), np.ones((P.shape[0], 1))], axis=1) @ M.T
            P = Ph[:, :3].astype(np.float32)
            if N is not None:
                Nw = N.astype(np.float64) @ np.linalg.inv(M[:3, :3])
                N = (Nw / np.linalg.norm(Nw, axis=1, keepdims=True)).astype(np.float32)
            if _bool(p, "flip_normals") and N is not None:
                N = -N
            sid = desc.add_mesh(P, F, b, flags, N=N, UV=UV)
        else:
            raise ValueError(f"unsupported shape type '{t}'")
        if nm is not None:
            if desc.normalmap is not None:
                raise ValueError("more than one normal-mapped shape (one normal map per scene)")
            desc.normalmap = (sid, nm[0], nm[1])
            desc.lean_fallback = nm[2]
        for em in (c for c in el if c.tag == "emitter"):
            if em.get("type") != "area":
                raise ValueError("only area emitters may be nested in a shape")
            if t != "sphere":
                raise ValueError("area emitters are supported on spheres only")
            ep = _props(em)
            desc.add_area_emitter(sid, _spectrum(ep, "radiance", (1.0,) * 3), _emitter_flags(sms, ep))
    return desc, config, itype


def _int(p, name, default):
    return int(p[name][1].get("value")) if name in p else default


def load_render_setup(sms, path):
    """(Camera, RenderOptions) of the scene file's sensor and integrator."""
    root = ET.parse(Path(path)).getroot()
    sensor = next((c for c in root if c.tag == "sensor"), None)
    if sensor is None:
        raise ValueError("the scene has no <sensor>")
    if sensor.get("type") != "perspective":
        raise ValueError(f"unsupported sensor type '{sensor.get('type')}'")
    p = _props(sensor)
    if "focal_length" in p:
        raise ValueError("focal_length is not supported; give the sensor a fov")
    tr = next((c for c in sensor if c.tag == "transform" and c.get("name") == "to_world"), None)
    M = _transform(tr) if tr is not None else np.eye(4)
    film = next((c for c in sensor if c.tag == "film"), None)
    fp = _props(film) if film is not None else {}
    smp = next((c for c in sensor if c.tag == "sampler"), None)
    sp = _props(smp) if smp is not None else {}
    # the film's reconstruction filter: gaussian (stddev 0.5) unless the film
    # names one (src/rfilters/gaussian.cpp: the reference's default), or box
    rf = next((c for c in film if c.tag == "rfilter"), None) if film is not None else None
    rf_type = "gaussian" if rf is None else rf.get("type")
    if rf_type not in ("box", "gaussian"):
        raise ValueError(f"reconstruction filter '{rf_type}' is not supported (box or gaussian)")
    rf_stddev = _float(_props(rf), "stddev", 0.5) if rf is not None else 0.5
    axis = p["fov_axis"][1].get("value").lower() if "fov_axis" in p else "x"
    cam = sms.Camera(M.astype(np.float32), _float(p, "fov", 45.0), _int(fp, "width", 768), _int(fp, "height", 576),
                     axis, _float(p, "near_clip", 1e-2), _float(p, "far_clip", 1e4))
    opt = sms.RenderOptions(spp=_int(sp, "sample_count", 4), rfilter=rf_type, rfilter_stddev=rf_stddev)
    integ = next((c for c in root if c.tag == "integrator"), None)
    if integ is not None:
        t = integ.get("type")
        if t not in _INTEGRATOR_TYPES:
            raise ValueError(f"unsupported integrator type '{t}'")
        ip = _props(integ)
        opt.integrator = t
        opt.max_depth = _int(ip, "max_depth", -1)
        opt.rr_depth = _int(ip, "rr_depth", 5)
        opt.disable_reflected_emitters = _bool(ip, "disable_reflected_emitters")
        opt.biased_mnee = _bool(ip, "biased_mnee")
        opt.samples_per_pass = _int(ip, "samples_per_pass", 0)
        opt.timeout = _float(ip, "timeout", -1.0)
        opt.glint_diff_scale_factor_clamp = _float(ip, "glint_diff_scale_factor_clamp", 0.0)
        if t == "path_filtered_teaser":
            opt.non_sms_paths_enabled = _bool(ip, "non_sms_paths_enabled", True)
        if t == "path_sms_teaser":
            # path_sms_teaser.cpp:60-81: the switches and the glints_* block
            opt.caustics_enabled = _bool(ip, "caustics_enabled", True)
            opt.glints_enabled = _bool(ip, "glints_enabled", True)
            opt.non_sms_paths_enabled = _bool(ip, "non_sms_paths_enabled", True)
            g = sms.SMSConfig()
            g.biased = _bool(ip, "glints_biased")
            g.step_scale = _float(ip, "glints_step_scale", 1.0)
            g.max_iterations = _int(ip, "glints_max_iterations", 20)
            g.solver_threshold = _float(ip, "glints_solver_threshold", 1e-5)
            g.uniqueness_threshold = _float(ip, "glints_uniqueness_threshold", 1e-4)
            g.max_trials = _int(ip, "glints_max_trials", -1)
            opt.glints = g
    return cam, opt
