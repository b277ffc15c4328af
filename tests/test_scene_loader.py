"""Scene-file loader (CS123 XML + OBJ/MTL), host side."""

import os

import numpy as np
import pytest

from path_gb300 import api, capi

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "scenes", "room.xml")
# the reference's own scenes/ folder (CS123 XML + OBJ/MTL), when a checkout of
# the reference is at hand; the test that loads them skips otherwise
REFERENCE_SCENES = os.environ.get("PATH_REFERENCE_SCENES", "")


def test_fixture_scene(lib):
    sc, f2w = api.Scene.load_xml(FIXTURE, 1.0)
    z = sc.sizes()
    assert z == {"triangles": 13, "meshes": 1, "instances": 2, "clusters": 2, "materials": 6}
    ex = sc.export()
    types = [ex["materials"][i].type for i in range(6)]
    B = capi.BSDF
    assert types == [B["Diffuse"], B["Diffuse"], B["Diffuse"], B["DiffuseGlossy"], B["Mirror"],
                     B["DielectricRefractive"]]
    lamp = ex["materials"][2]
    assert list(lamp.emission) == [10, 8, 6]
    shiny = ex["materials"][3]
    wd = 0.9 / (0.9 + 1.2)
    assert abs(shiny.diffuse_weight - wd) < 1e-6 and abs(shiny.shininess - 30) < 1e-6
    assert abs(ex["materials"][5].ior - 1.45) < 1e-6
    # emissive clusters: the lamp quad (triangles 4, 5) and the lamp triangle (10)
    assert ex["clusters"].tolist() == [[2, 4, 6], [2, 10, 11]]
    # the concave hexagon is cut into 4 triangles covering its 0.2 area
    t = ex["triangles"].reshape(-1, 3, 3)
    hexa = t[6:10]
    areas = 0.5 * np.linalg.norm(np.cross(hexa[:, 1] - hexa[:, 0], hexa[:, 2] - hexa[:, 0]), axis=1)
    assert abs(areas.sum() - 0.2) < 1e-6
    # normals from vn for the lamp quad, face normals elsewhere
    n = ex["normals"].reshape(-1, 3, 3)
    np.testing.assert_allclose(n[4:6].reshape(-1, 3), np.tile([0, -1, 0], (6, 1)))
    # second instance: translate (3, 0, 0) then rotate 90 degrees about y
    x = ex["instance_xforms"][1].reshape(3, 4)
    np.testing.assert_allclose(x[:, :3], [[0, 0, 1], [0, 1, 0], [-1, 0, 0]], atol=1e-6)
    np.testing.assert_allclose(x[:, 3], [3, 0, 0], atol=1e-6)
    # camera from the focus point
    np.testing.assert_allclose(f2w.reshape(3, 4)[:, 3], [0, 1, 4], atol=1e-6)


def test_loader_errors(lib, tmp_path):
    with pytest.raises(capi.PathError) as e:
        api.Scene.load_xml(str(tmp_path / "missing.xml"), 1.0)
    assert e.value.status == 7
    bad = tmp_path / "bad.xml"
    bad.write_text("<scenefile><object type='tree' name='root'><transblock>"
                   "<object type='primitive' name='sphere'/></transblock></object></scenefile>")
    with pytest.raises(capi.PathError) as e:
        api.Scene.load_xml(str(bad), 1.0)
    assert e.value.status == 2
    light = tmp_path / "light.xml"
    light.write_text("<scenefile><lightdata/></scenefile>")
    with pytest.raises(capi.PathError) as e:
        api.Scene.load_xml(str(light), 1.0)
    assert e.value.status == 2
    mtl = tmp_path / "m.mtl"
    mtl.write_text("newmtl x\nillum 4\nKd 1 1 1\n")
    (tmp_path / "m.obj").write_text("mtllib m.mtl\nv 0 0 0\nv 1 0 0\nv 0 1 0\nusemtl x\nf 1 2 3\n")
    xml = tmp_path / "m.xml"
    xml.write_text("<scenefile><object type='tree' name='root'><transblock>"
                   "<object type='primitive' name='mesh' filename='m.obj'/></transblock>"
                   "</object></scenefile>")
    with pytest.raises(capi.PathError) as e:
        api.Scene.load_xml(str(xml), 1.0)
    assert "illum" in str(e.value)


@pytest.mark.skipif(not REFERENCE_SCENES or not os.path.isdir(REFERENCE_SCENES),
                    reason="PATH_REFERENCE_SCENES does not name the reference's scenes folder")
def test_reference_scenes_load(lib):
    loaded = 0
    for name in sorted(os.listdir(REFERENCE_SCENES)):
        if not name.endswith(".xml"):
            continue
        try:
            sc, f2w = api.Scene.load_xml(os.path.join(REFERENCE_SCENES, name), 1.0)
        except capi.PathError as e:
            # only failures the reference itself reports are acceptable
            assert any(k in str(e) for k in ("illum", "light", "primitive", "cannot open")), (name, e)
            continue
        z = sc.sizes()
        assert z["triangles"] > 0, name
        loaded += 1
    assert loaded >= 5


FIXTURES = os.path.join(HERE, "golden", "reference_scenes.npz")
FIXTURE_SCENES = ["cornell-diffuse", "cornell-glossy-sphere", "cornell-mirror",
                  "cornell-glass-box"]


def _obj_faces(path):
    """Polygons of an OBJ file (negative indices resolved), in file order."""
    verts, faces = [], []
    with open(path) as f:
        for line in f:
            tok = line.split()
            if not tok:
                continue
            if tok[0] == "v":
                verts.append([float(x) for x in tok[1:4]])
            elif tok[0] == "f":
                idx = []
                for t in tok[1:]:
                    i = int(t.split("/")[0])
                    idx.append(i - 1 if i > 0 else len(verts) + i)
                faces.append(np.array([verts[i] for i in idx]))
    return faces


@pytest.mark.skipif(not REFERENCE_SCENES or not os.path.isdir(REFERENCE_SCENES),
                    reason="PATH_REFERENCE_SCENES does not name the reference's scenes folder")
@pytest.mark.parametrize("name", FIXTURE_SCENES)
def test_reference_scene_loads_as_the_fixture_and_covers_every_face(lib, name):
    # The loader's output for the reference's own scene is what the GPU
    # tests render (tests/golden/reference_scenes.npz); and every polygon of
    # the OBJ is cut into triangles of its own vertices covering its area
    # (tinyobjloader's triangulation, which the reference uses).
    g = np.load(FIXTURES)
    sc, f2w = api.Scene.load_xml(os.path.join(REFERENCE_SCENES, name + ".xml"), 1.0)
    ex = sc.export()
    for k in ("triangles", "normals", "tri_material"):
        assert np.array_equal(ex[k], g[f"{name}/{k}"]), k
    assert np.array_equal(ex["instance_xforms"][0], g[f"{name}/object_to_world"])
    assert np.array_equal(f2w, g[f"{name}/film_to_world"])
    n_mat = ex["n_materials"]
    assert bytes(ex["materials"])[:64 * n_mat] == g[f"{name}/materials"].tobytes()
    tris = ex["triangles"].reshape(-1, 3, 3).astype(np.float64)
    faces = _obj_faces(os.path.join(REFERENCE_SCENES, "models", name + ".obj"))
    assert sum(len(f) - 2 for f in faces) == len(tris)
    k = 0
    for face in faces:
        part = tris[k:k + len(face) - 2]
        k += len(face) - 2
        for t in part:
            for v in t:
                assert np.min(np.linalg.norm(face - v, axis=1)) < 1e-6
        area = 0.5 * np.linalg.norm(np.cross(part[:, 1] - part[:, 0], part[:, 2] - part[:, 0]),
                                    axis=1).sum()
        # the polygon's area: fan from its first vertex (convex in these files)
        fan = 0.5 * np.linalg.norm(np.cross(face[1:-1] - face[0], face[2:] - face[0]),
                                   axis=1).sum()
        assert abs(area - fan) <= 1e-5 * max(fan, 1e-6)
