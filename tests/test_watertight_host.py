"""The opt-in watertight triangle test (Woop, Benthin and Wald, JCGT 2013) of
the oracle: no cracks between triangles that share an edge, and the same
answers as MRay's Moller-Trumbore test away from edges."""
import ctypes as C

import numpy as np

import oracle


def _grid_mesh(n, seed):
    """A jittered n x n grid of quads (two triangles each) in a rotated,
    shifted plane: every interior edge and vertex is shared."""
    rng = np.random.default_rng(seed)
    u, v = np.meshgrid(np.arange(n + 1, dtype=np.float64), np.arange(n + 1, dtype=np.float64))
    p = np.stack([u, v, np.zeros_like(u)], -1).reshape(-1, 3)
    p[:, :2] += rng.uniform(-0.3, 0.3, (p.shape[0], 2))
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    pos = (p / n - 0.5) @ q.T * 7.0 + rng.uniform(-3, 3, 3)
    idx = []
    for j in range(n):
        for i in range(n):
            a, b, c, d = j * (n + 1) + i, j * (n + 1) + i + 1, (j + 1) * (n + 1) + i, (j + 1) * (n + 1) + i + 1
            idx += [(a, b, d), (a, d, c)]
    return pos.astype(np.float32), np.array(idx, np.uint32), q[:, 2]


def _rays_at(targets, normal, rng, spread=0.8):
    """Rays from random points on the normal's side towards the targets."""
    n = targets.shape[0]
    off = rng.normal(size=(n, 3)) * spread + normal * 4.0
    org = targets + off
    d = targets - org
    d = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = org
    rays[:, 4:7] = d
    rays[:, 7] = 1e30
    return rays


def test_no_cracks_on_shared_edges_and_vertices():
    """Rays aimed at the shared vertices and edges of jittered grid meshes
    (front and back): with the watertight test none of them slips through."""
    rng = np.random.default_rng(7)
    misses = {}
    for wt in (False, True):
        total = 0
        for seed in range(4):
            pos, idx, nrm = _grid_mesh(24, seed)
            n = 25
            interior = [j * n + i for j in range(1, n - 1) for i in range(1, n - 1)]
            verts = pos[interior]
            edges = []
            for (a, b, c) in idx:
                for e0, e1 in ((a, b), (b, c), (c, a)):
                    w = rng.uniform(0.05, 0.95)
                    edges.append(pos[e0] * (1 - w) + pos[e1] * w)
            edges = np.array(edges, np.float32)
            # keep edge points away from the grid's outer border
            cen = pos.mean(0)
            keep = np.linalg.norm(edges - cen, axis=1) < 2.0
            targets = np.vstack([verts, edges[keep]]).astype(np.float32)
            for side in (1.0, -1.0):          # front and back faces
                S = oracle.Scene(watertight=wt)
                mid = S.add_mesh(pos, idx)
                S.add_instance(mid, np.eye(3, 4, dtype=np.float32), cull=False)
                S.build()
                rays = _rays_at(targets, nrm * side, rng)
                # every triangle tested (AcceleratorLinear): MRay's LBVH leaf
                # boxes are the triangles' exact AABBs, and a ray through a
                # shared vertex can graze all of them in the slab test
                _, hits, _, inst = S.cast_closest(rays, linear=True)
                total += int((inst == 0xFFFFFFFF).sum())
        misses[wt] = total
    print("rays through shared vertices and edges that miss: MT %d, watertight %d" % (misses[False], misses[True]))
    assert misses[True] == 0
    assert misses[False] > 0        # the cracks the option exists for


def test_same_hits_as_moller_trumbore_away_from_edges():
    L = oracle.lib()
    rng = np.random.default_rng(11)
    vp = C.c_void_p
    n = 4000
    agree = 0
    for _ in range(n):
        v = rng.uniform(-1, 1, (3, 3)).astype(np.float32)
        o = rng.uniform(-3, 3, 3).astype(np.float32)
        # a point well inside the triangle
        w = rng.dirichlet((4, 4, 4))
        p = (w @ v.astype(np.float64))
        d = (p - o) / np.linalg.norm(p - o)
        d = d.astype(np.float32)
        out = []
        for fn in (L.orc_intersect_triangle, L.orc_intersect_triangle_wt):
            b = np.zeros(3, np.float32); t = np.zeros(1, np.float32); bf = np.zeros(1, np.int32)
            h = fn(d.ctypes.data_as(vp), o.ctypes.data_as(vp), v[0].ctypes.data_as(vp), v[1].ctypes.data_as(vp),
                   v[2].ctypes.data_as(vp), 0, b.ctypes.data_as(vp), t.ctypes.data_as(vp), bf.ctypes.data_as(vp))
            out.append((h, b.copy(), float(t[0]), int(bf[0])))
        (h0, b0, t0, f0), (h1, b1, t1, f1) = out
        assert h0 == h1 == 1
        assert f0 == f1
        # both are float evaluations of the same t and barycentrics (MT divides
        # by a determinant that can be small; the edge functions do not)
        assert abs(t0 - t1) <= 1e-4 * t0
        assert np.abs(b0 - b1).max() <= 1e-3
        agree += 1
    assert agree == n
