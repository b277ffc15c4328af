"""Writes tests/golden/reference_scenes.npz: four of the reference's own
scenes (scenes/*.xml with their OBJ / MTL models) as loaded by this
library's scene-file loader (path_scene_load_xml, the restatement of
ScenefileLoader, src/scene/scenefile_compat/scenefile_loader.cpp:23-319).

Per scene: the object-space triangles, vertex normals, per-triangle
material, the mesh's object-to-world transform, the materials (raw
path_material records) and the camera's film_to_world for a square image.
The GPU tests render these scenes and compare them with the oracle; the
CPU tests reload the XML files (when a checkout of the reference is at
hand) and hold the loader to these arrays bit for bit.

Run from the repository root with PATH_REFERENCE_SCENES naming the
reference's scenes/ folder:
  PATH_REFERENCE_SCENES=<reference>/scenes python tests/golden/make_reference_scene_fixtures.py
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

OUT = os.path.join(HERE, "reference_scenes.npz")
SCENES = ["cornell-diffuse", "cornell-glossy-sphere", "cornell-mirror", "cornell-glass-box"]


def load(folder, name):
    from path_gb300 import api
    sc, f2w = api.Scene.load_xml(os.path.join(folder, name + ".xml"), 1.0)
    ex = sc.export()
    assert len(ex["mesh_ends"]) == 1 and len(ex["instance_mesh"]) == 1, name
    n_mat = ex["n_materials"]
    mats = np.frombuffer(bytes(ex["materials"])[:64 * n_mat], np.uint8).reshape(n_mat, 64)
    return {"triangles": ex["triangles"], "normals": ex["normals"],
            "tri_material": ex["tri_material"], "object_to_world": ex["instance_xforms"][0],
            "materials": mats.copy(), "film_to_world": f2w}


def main():
    folder = os.environ.get("PATH_REFERENCE_SCENES", "")
    if not os.path.isdir(folder):
        raise SystemExit("PATH_REFERENCE_SCENES must name the reference's scenes folder")
    arrays = {}
    for name in SCENES:
        for k, v in load(folder, name).items():
            arrays[f"{name}/{k}"] = v
    np.savez_compressed(OUT, **arrays)
    print(f"wrote {OUT}: {', '.join(SCENES)}")


if __name__ == "__main__":
    main()
