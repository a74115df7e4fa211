"""Seeded workload generators are deterministic and platform-independent:
digests recorded by tests/golden/make_golden.py must reproduce."""
import hashlib
import json
import os

import numpy as np

from mray_gb300 import scenes

DIG = os.path.join(os.path.dirname(__file__), "golden", "scene_digests.json")


def test_scene_digests(built_libs):
    d = json.load(open(DIG))
    pos, idx = scenes.icosphere(5, 1.0, 0.05, 4.0, 0)
    assert [hashlib.sha256(pos.tobytes()).hexdigest(), hashlib.sha256(idx.tobytes()).hexdigest()] == d["icosphere_l5"]
    assert hashlib.sha256(scenes.instance_field(64, 0).tobytes()).hexdigest() == d["instance_field_64"]
    assert hashlib.sha256(scenes.primary_rays(64, 48, 0).tobytes()).hexdigest() == d["primary_64x48"]


def test_icosphere_topology(built_libs):
    pos, idx = scenes.icosphere(4, 2.0, 0.0, 4.0, 0)
    assert idx.shape == (20 * 4 ** 4, 3)
    r = np.linalg.norm(pos, axis=1)
    assert np.allclose(r, 2.0, rtol=1e-6)
    # outward winding: normal . centroid > 0
    v = pos[idx]
    n = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
    assert (np.einsum("ij,ij->i", n, v.mean(1)) > 0).all()
    # watertight: every edge is shared by exactly two triangles (by position)
    key = lambda a, b: tuple(sorted((tuple(a), tuple(b))))
    edges = {}
    for t in v[:2000]:
        for a, b in ((0, 1), (1, 2), (2, 0)):
            edges[key(t[a], t[b])] = edges.get(key(t[a], t[b]), 0) + 1
    assert max(edges.values()) <= 2


def test_stress_scene_sizes(built_libs):
    pos, idx, m = scenes.bvh_stress_scene(level=8)
    assert idx.shape[0] == 1310720 and m.shape == (64, 12)
    R = m.reshape(64, 3, 4)[:, :, :3].astype(np.float64)
    assert np.allclose(np.einsum("nij,nkj->nik", R, R), np.eye(3), atol=1e-6)
    # the rotation family keeps MRay's inverse exact: m0*m6 == m2*m4
    assert np.abs(R[:, 0, 0] * R[:, 1, 2] - R[:, 0, 2] * R[:, 1, 0]).max() < 1e-6
