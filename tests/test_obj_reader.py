"""Wavefront OBJ reader (sms_obj_load), the reference's obj shape plugin
(src/shapes/obj.cpp:90-330) restated: vertex de-duplication by (v, vt, vn),
fan triangulation, texture-v flip, angle-weighted vertex normals
(src/librender/mesh.cpp:420-470) when the file has none.  Host code only."""
import numpy as np
import pytest


def _write(tmp_path, text, name="m.obj"):
    p = tmp_path / name
    p.write_text(text)
    return p


def test_quad_and_triangle_with_all_reference_forms(sms, tmp_path):
    text = """# test mesh
mtllib none.mtl
o thing
v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
v 0.5 0.5 1
vt 0 0
vt 1 0
vt 1 1
vt 0 1
vn 0 0 1
vn 0 1 0
g quad
usemtl x
f 1/1/1 2/2/1 3/3/1 4/4/1
f 1//2 2//2 5//2
f 3 4 5
"""
    P, F, N, UV = sms.load_obj(_write(tmp_path, text))
    # distinct (v, vt, vn): 4 for the quad, 3 for the v//vn triangle, 3 for the v-only one
    assert P.shape == (10, 3) and F.shape == (4, 3)
    # fan triangulation of the quad: (0,1,2), (0,2,3)
    np.testing.assert_array_equal(F[:2], [[0, 1, 2], [0, 2, 3]])
    np.testing.assert_array_equal(F[2], [4, 5, 6])
    # texture v flipped (flip_tex_coords default true)
    np.testing.assert_allclose(UV[:4], [[0, 1], [1, 1], [1, 0], [0, 0]])
    np.testing.assert_allclose(N[:4], [[0, 0, 1]] * 4)
    np.testing.assert_allclose(N[4:7], [[0, 1, 0]] * 3)
    # a vertex without a vn reference in a file with normals gets a zero normal
    np.testing.assert_allclose(N[7:], 0.0)
    P2, F2, N2, UV2 = sms.load_obj(_write(tmp_path, text), face_normals=True, flip_tex_coords=False)
    assert N2 is None
    np.testing.assert_allclose(UV2[:4], [[0, 0], [1, 0], [1, 1], [0, 1]])


def _angle_weighted_normals(P, F):
    acc = np.zeros_like(P, dtype=np.float64)
    for f in F:
        v = P[f].astype(np.float64)
        n = np.cross(v[1] - v[0], v[2] - v[0])
        if np.linalg.norm(n) == 0:
            continue
        n /= np.linalg.norm(n)
        for j in range(3):
            e1 = v[(j + 1) % 3] - v[j]
            e2 = v[(j + 2) % 3] - v[j]
            a = np.arccos(np.clip(e1 @ e2 / np.linalg.norm(e1) / np.linalg.norm(e2), -1, 1))
            acc[f[j]] += n * a
    return acc / np.linalg.norm(acc, axis=1, keepdims=True)


def test_recomputed_normals_are_angle_weighted(sms, workloads, tmp_path):
    # a small heightfield written as OBJ without normals
    P, N, UV, F = workloads.heightfield_mesh(9, 1.0, 1.0, workloads.water_params(4))
    lines = [f"v {x:.7f} {y:.7f} {z:.7f}" for x, y, z in P] + [f"f {a + 1} {b + 1} {c + 1}" for a, b, c in F]
    P2, F2, N2, UV2 = sms.load_obj(_write(tmp_path, "\n".join(lines) + "\n"))
    # vertices are renumbered in order of first use; the triangles are the same
    assert UV2 is None and P2.shape == P.shape
    np.testing.assert_allclose(P2[F2], P[F], atol=1e-6)
    np.testing.assert_allclose(N2, _angle_weighted_normals(P2, F2), atol=2e-6)
    assert np.all(N2[:, 2] > 0)   # the surface faces up


@pytest.mark.parametrize("bad,what", [("v 0 0 0\nv 1 0 0\nf 1 2 3\n", "invalid vertex"),
                                      ("v 0 0\n", "could not parse"),
                                      ("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1/4 2 3\n", "texture coordinate"),
                                      ("# nothing\n", "no faces")])
def test_errors_are_reported(sms, tmp_path, bad, what):
    with pytest.raises(sms.SMSError) as e:
        sms.load_obj(_write(tmp_path, bad))
    assert e.value.status == 5 and what in str(e.value)


def test_missing_file(sms, tmp_path):
    with pytest.raises(sms.SMSError) as e:
        sms.load_obj(tmp_path / "absent.obj")
    assert "cannot open" in str(e.value)


def test_scene_desc_add_obj(sms, tmp_path):
    text = "v -1 -1 1\nv 1 -1 1\nv 1 1 1\nv -1 1 1\nvt 0 0\nvt 1 0\nvt 1 1\nvt 0 1\nf 1/1 2/2 3/3 4/4\n"
    d = sms.SceneDesc()
    sid = d.add_obj(_write(tmp_path, text), sms.Bsdf(sms.BSDF_DIELECTRIC, 1.33), sms.SHAPE_CAUSTIC_CASTER_SINGLE)
    assert sid == 0
    P, F, b, flags = d.meshes[0][0], d.meshes[0][3], d.meshes[0][4], d.meshes[0][5]
    assert P.shape == (4, 3) and F.shape == (2, 3) and flags == sms.SHAPE_CAUSTIC_CASTER_SINGLE
