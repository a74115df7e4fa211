"""MRay scene-format reader (mray_gb300/scene_json.py): parsing, transforms,
materials, lights, camera, error paths; the scene renders through the
oracle.  CPU only."""
import math
import os

import numpy as np
import pytest

import oracle
from mray_gb300 import scene_json

HERE = os.path.join(os.path.dirname(__file__), "scenes")
SCENE = os.path.join(HERE, "open_box.json")


def test_strip_comments_keeps_strings():
    t = '{"a": "x // not a comment", /* block */ "b": 1 // tail\n}'
    assert scene_json.load_jsonc(t) == {"a": "x // not a comment", "b": 1}


def test_trailing_comma_rejected():
    with pytest.raises(scene_json.SceneError):
        scene_json.load_jsonc('{"a": [1, 2,]}')


def test_read_open_box():
    surfaces, cam, env = scene_json.read_scene(SCENE)
    kinds = [s.get("material", s["kind"]) for s in surfaces]
    assert kinds == ["lambert", "reflect", "refract", "unreal", "light"]
    assert surfaces[0]["texture"].shape == (64, 64, 4) and surfaces[0]["uv"].shape == (4, 2)
    assert surfaces[2]["ior"] == (1.0, 1.5) and surfaces[2]["cull"] is False
    assert surfaces[3]["idx"].shape == (8, 3)                    # nodeTriangle
    assert surfaces[4]["radiance"] == [12.0, 11.0, 9.0]
    # trs: translate * rotZ * rotY * rotX * scale
    m = surfaces[2]["m34"].reshape(3, 4)
    a = math.radians(25)
    np.testing.assert_allclose(m[:, :3] @ [1, 0, 0], [0.25 * math.cos(a), 0, -0.25 * math.sin(a)], atol=1e-6)
    np.testing.assert_allclose(m[:, 3], [0.3, 0.151, 0.55], atol=1e-6)
    assert env["texels"].shape == (1, 1, 4) and np.allclose(env["texels"][0, 0, :3], [0.35, 0.45, 0.6])
    assert cam["pos"] == (0.5, 0.6, -1.3)
    assert abs(cam["fov"][0] - math.radians(42.0)) < 1e-12 and abs(cam["fov"][1] - cam["fov"][0]) < 1e-12


def test_renders_with_oracle():
    surfaces, cam, env = scene_json.read_scene(SCENE)
    S = oracle.PtScene(surfaces, env=env)
    img = S.render(S.params(24, 24, 8, cam, seed=1))
    rgb = img[..., :3] / img[..., 3:]
    assert np.all(np.isfinite(rgb)) and rgb.mean() > 0.05


@pytest.mark.parametrize("bad,msg", [
    ('"Primitives": [{"id": 0, "type": "Sphere", "tag": "nodeSphere", "radius": 1, "center": [0,0,0]}]', "triangles"),
    ('"Primitives": [{"id": 0, "type": "Triangle", "tag": "assimp", "file": "x.obj", "innerIndex": 0}]', "tag"),
])
def test_unsupported_inputs(bad, msg):
    base = ('{"Cameras": [{"id":0,"type":"Pinhole","isFovX":true,"fov":40,"aspect":1,"planes":[0.1,10],'
            '"gaze":[0,0,0],"position":[0,0,-1],"up":[0,1,0]}], "Lights": [{"id":0,"type":"Null"}],'
            '"Mediums": [], "Transforms": [{"id":0,"type":"Identity"}], "Textures": [],'
            '"Materials": [{"id":0,"type":"Lambert","albedo":[0.5,0.5,0.5]}], %s,'
            '"Boundary": {"medium":0,"light":0,"transform":0},'
            '"Surfaces": [{"transform":0,"material":0,"primitive":0}], "LightSurfaces": [],'
            '"CameraSurfaces": [{"camera":0}]}')
    with pytest.raises(scene_json.SceneError, match=msg):
        scene_json.read_scene(base % bad)
