"""GPU parity of the closest-hit / any-hit kernels against the CPU oracle,
through the C ABI.  Bar: bit-exact hit keys, barycentrics and t for every ray
except exact-t ties between different primitives (first-found wins in MRay,
Source/Tracer/AcceleratorLBVH.hpp:363-367); bit-exact visibility bits."""
import numpy as np
import pytest

import oracle
from mray_gb300 import Accelerator, MRGError, scenes
from parity_util import (MISS, build_pair, compare_closest, gpu_closest, gpu_visibility, tri_retest,
                         stress_workload)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _libs(cuda_lib, built_libs):
    return True


def small(level=3, ninst=8, seed=0, box=6.0):
    pos, idx = scenes.icosphere(level, 1.0, 0.05, 4.0, seed)
    m = scenes.instance_field(ninst, seed, box=box, jitter=0.3)
    return pos, idx, m


@pytest.mark.parametrize("level,ninst", [(0, 1), (1, 3), (3, 8), (4, 27), (5, 64)])
@pytest.mark.parametrize("cull", [True, False])
def test_closest_small_scenes(level, ninst, cull):
    pos, idx, m = small(level, ninst, seed=level)
    acc, S = build_pair(pos, idx, m, cull=cull)
    rays = scenes.primary_rays(97, 61, level, eye=(0, 0, -14), tan_half_fov=0.5)
    ora = S.cast_closest(rays)
    gpu = gpu_closest(acc, rays)
    n, hits, ties = compare_closest(ora, gpu, retest=tri_retest(S, rays, pos, idx, cull=cull))
    assert hits > 0


def _mesh_of(ntri, seed):
    """A random triangle soup of ntri triangles inside a unit cube."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(-1, 1, (ntri, 1, 3))
    pos = (c + rng.uniform(-0.35, 0.35, (ntri, 3, 3))).reshape(-1, 3).astype(np.float32)
    return pos, np.arange(3 * ntri, dtype=np.uint32).reshape(-1, 3)


def test_batched_blas_build_mixed_mesh_sizes():
    """All BLASes are built in one batch: meshes of 1, 2, 3, 7, 100 and 5,000
    triangles (leaf roots, tiny trees, one-triangle and three-triangle leaf
    sizes) side by side, each instanced, against the oracle's per-mesh
    builds; per-mesh prim keys and world boxes must survive the batching."""
    sizes = [1, 2, 3, 7, 100, 5000, 1, 40]
    acc = Accelerator(0)
    S = oracle.Scene()
    rng = np.random.default_rng(3)
    inst = 0
    for k, nt in enumerate(sizes):
        pos, idx = _mesh_of(nt, 10 + k)
        base = 0x10000000 + 0x10000 * k
        mid = acc.upload_mesh(pos, idx, prim_key_base=base)
        oid = S.add_mesh(pos, idx, prim_key_base=base)
        for j in range(2):
            m = np.zeros((3, 4), np.float32)
            m[:, :3] = np.eye(3) * rng.uniform(0.8, 1.5)
            m[:, 3] = rng.uniform(-5, 5, 3)
            m = m.reshape(12)
            acc.add_instance(mid, m, light_or_mat_key=inst, trans_key=(1 << 24) | inst, accel_key=(2 << 20) | inst)
            S.add_instance(oid, m, lm_key=inst, trans_key=(1 << 24) | inst, accel_key=(2 << 20) | inst)
            inst += 1
    acc.construct()
    S.build()
    st = acc.stats()
    assert st["accelerators"] == len(sizes) and st["instances"] == 2 * len(sizes)
    assert st["blasTriangles"] == sum(sizes)
    rays = scenes.primary_rays(160, 120, 4, eye=(0, 0, -16), tan_half_fov=0.45)
    ora = S.cast_closest(rays)
    gpu = gpu_closest(acc, rays)
    n, hits, ties = compare_closest(ora, gpu)
    assert hits > 1000
    keys = gpu[1][:, 0][gpu[1][:, 0] != MISS]
    assert len(np.unique(keys >> 16)) >= len(sizes) - 2   # nearly every mesh is hit somewhere


def _general_rotations(n=12, seed=5):
    rng = np.random.default_rng(seed)
    mats = []
    for i in range(n):
        q = rng.normal(size=4); q /= np.linalg.norm(q)
        w, x, y, z = q
        R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                      [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                      [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
        mats.append(np.hstack([R, rng.uniform(-3, 3, (3, 1))]).reshape(12))
    return np.array(mats, np.float32)


def test_corrected_inverse_mode_general_rotations():
    """General random rotations with the corrected inverse: bit-exact on every ray."""
    pos, idx = scenes.icosphere(3, 1.0, 0.05, 4.0, 0)
    mats = _general_rotations()
    rays = scenes.primary_rays(80, 80, 9, eye=(0, 0, -12), tan_half_fov=0.5)
    acc, S = build_pair(pos, idx, mats, corrected=True)
    compare_closest(S.cast_closest(rays), gpu_closest(acc, rays), retest=tri_retest(S, rays, pos, idx))


def test_reference_inverse_mode_general_rotations():
    """MRay's own inverse on general rotations misplaces the BLAS geometry
    relative to the instance's world AABB, so which hit MRay reports depends on
    the order its TLAS visits instances (its LBVH result differs from its own
    brute force on ~14% of these rays).  The GPU visits nearest-first; it must
    agree bit for bit on >= 99% of rays, and every ray where it differs must
    carry a genuine MRay hit: the reported triangle, intersected with the
    oracle's MT in that instance's (MRay-inverted) space, gives exactly the
    reported t and barycentrics."""
    pos, idx = scenes.icosphere(3, 1.0, 0.05, 4.0, 0)
    mats = _general_rotations()
    rays = scenes.primary_rays(80, 80, 9, eye=(0, 0, -12), tan_half_fov=0.5)
    acc, S = build_pair(pos, idx, mats, corrected=False)
    ora = S.cast_closest(rays)
    gr, gh, gm = gpu_closest(acc, rays)
    diff = np.nonzero(ora[0][:, 7].view(np.uint32) != gr[:, 7].view(np.uint32))[0]
    assert diff.size <= 0.01 * rays.shape[0]
    for k in diff:
        if gr[k, 7] >= 3e38:
            continue
        inst = int(gh[k, 2] & 0xFFFFFF)
        prim = int(gh[k, 0] - 0x10000000)
        inv = S.instance_inverse(inst)
        R = inv.reshape(3, 4)
        import ctypes as C
        L = oracle.lib()
        d = np.ascontiguousarray(rays[k, 4:7]); p = np.ascontiguousarray(rays[k, 0:3])
        ld = np.zeros(3, np.float32); lp = np.zeros(3, np.float32)
        L.orc_transform_ray(inv.ctypes.data_as(C.c_void_p), d.ctypes.data_as(C.c_void_p),
                            p.ctypes.data_as(C.c_void_p), ld.ctypes.data_as(C.c_void_p),
                            lp.ctypes.data_as(C.c_void_p))
        v = pos[idx[prim]]
        hit, bary, t, _ = oracle.intersect_triangle(ld, lp, v[0], v[1], v[2], True)
        assert hit and np.float32(t).view(np.uint32) == gr[k, 7].view(np.uint32)
        assert np.array_equal(bary[:2].view(np.uint32), gm[k].view(np.uint32))
    other = np.setdiff1d(np.arange(rays.shape[0]), diff)
    compare_closest(ora, (gr, gh, gm), listed=other)


def test_indirection_partial_lists_and_prefilled_hits():
    pos, idx, m = small(4, 27)
    acc, S = build_pair(pos, idx, m)
    rays = scenes.primary_rays(64, 64, 3, eye=(0, 0, -12), tan_half_fov=0.6)
    rng = np.random.default_rng(1)
    sel = rng.permutation(rays.shape[0])[:1237].astype(np.uint32)
    pre = np.full((rays.shape[0], 4), 0x5A5A5A5A, np.uint32)
    ora = S.cast_closest(rays, ray_idx=sel, hits=pre)
    gpu = gpu_closest(acc, rays, ray_idx=sel, pre_hits=pre)
    compare_closest(ora, gpu)      # all rays: unlisted ones must be untouched too
    assert (gpu[1][np.setdiff1d(np.arange(rays.shape[0]), sel)] == 0x5A5A5A5A).all()


def test_visibility_small():
    pos, idx, m = small(4, 27)
    acc, S = build_pair(pos, idx, m)
    rays = scenes.primary_rays(71, 53, 4, eye=(0, 0, -12), tan_half_fov=0.6)
    closest = S.cast_closest(rays)
    hitm = closest[3] != MISS
    seg = rays.copy()
    seg[hitm, 7] = closest[0][hitm, 7] * np.float32(1.0001)   # segments ending just after the hit
    seg[::3, 7] = closest[0][::3, 7] * np.float32(0.5)
    for rs in (rays, seg):
        assert np.array_equal(gpu_visibility(acc, rs), S.cast_visibility(rs))
    sel = np.arange(0, rays.shape[0], 7, dtype=np.uint32)
    pre = np.full((rays.shape[0] + 31) // 32, 0xFFFF0000, np.uint32)
    assert np.array_equal(gpu_visibility(acc, seg, ray_idx=sel, pre_bits=pre),
                          S.cast_visibility(seg, ray_idx=sel, bits=pre))


def test_edge_rays():
    """Axis-parallel directions (zero components), rays starting inside the
    geometry, empty [tMin, tMax), far tMin, degenerate triangles."""
    pos, idx, m = small(3, 8)
    pos = pos.copy()
    idx = np.vstack([idx, [[0, 0, 1]], [[2, 2, 2]]]).astype(np.uint32)   # degenerate tris
    acc, S = build_pair(pos, idx, m, cull=False)
    rng = np.random.default_rng(11)
    n = 4096
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = rng.uniform(-4, 4, (n, 3))
    d = rng.normal(size=(n, 3))
    d[: n // 4, 1:] = 0.0
    d[n // 4: n // 2, 0] = 0.0
    d[n // 2: n // 2 + 16] = [0.0, -0.0, 1.0]
    rays[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays[:, 3] = 0.0
    rays[:, 7] = 3.4e38
    rays[100:200, 3] = 50.0          # tMin beyond everything
    rays[200:300, 7] = 0.0           # empty interval
    rays[300:400, 3] = 1.0
    rays[300:400, 7] = 1.0           # [1, 1): empty for a half-open range
    compare_closest(S.cast_closest(rays), gpu_closest(acc, rays), retest=tri_retest(S, rays, pos, idx, cull=False))
    assert np.array_equal(gpu_visibility(acc, rays), S.cast_visibility(rays))


def test_scale_extremes():
    """Instances scaled by 1e-3 .. 1e3 in one scene (TLAS quantisation and box
    inflation across six orders of magnitude) and a mesh placed 1e5 away from
    its own origin (BLAS quantisation frames with large exponents)."""
    pos, idx = scenes.icosphere(3, 1.0, 0.05, 4.0, 5)
    far = (pos + np.float32(1.0e5)).astype(np.float32)
    acc = Accelerator(0)
    S = oracle.Scene()
    ids = []
    for k, p in enumerate((pos, far)):
        ids.append((acc.upload_mesh(p, idx, prim_key_base=0x10000000 + 0x100000 * k),
                    S.add_mesh(p, idx, prim_key_base=0x10000000 + 0x100000 * k)))
    mats = []
    for i, (sc, t) in enumerate(((1e-3, (0.0, 0.0, 0.0)), (1.0, (3.0, 0.0, 0.0)), (1e3, (0.0, 0.0, 3000.0)),
                                  (1e-2, (0.01, 0.005, 0.0)), (1.0, (-1.0e5 - 3.0, -1.0e5, -1.0e5)))):
        m = np.zeros((3, 4), np.float32)
        m[:, :3] = np.eye(3) * sc
        m[:, 3] = t
        mats.append((1 if i == 4 else 0, m.reshape(12)))
    for i, (mesh, m) in enumerate(mats):
        acc.add_instance(ids[mesh][0], m, light_or_mat_key=i, trans_key=(1 << 24) | i, accel_key=i)
        S.add_instance(ids[mesh][1], m, lm_key=i, trans_key=(1 << 24) | i, accel_key=i)
    acc.construct()
    S.build()
    rays = []
    for eye, fov in (((0, 0, -0.01), 0.3), ((0, 0, -10), 0.5), ((0, 0, -1.0e4), 0.4)):
        rays.append(scenes.primary_rays(80, 60, 3, eye=eye, tan_half_fov=fov))
    rays = np.ascontiguousarray(np.vstack(rays))
    n, hits, ties = compare_closest(S.cast_closest(rays), gpu_closest(acc, rays))
    assert hits > 1000
    assert np.array_equal(gpu_visibility(acc, rays), S.cast_visibility(rays))


def test_zero_rays_and_not_built_errors():
    import torch
    from mray_gb300 import Accelerator
    acc = Accelerator(0)
    dr = torch.zeros((4, 8), device="cuda")
    hits = torch.zeros((4, 4), dtype=torch.int32, device="cuda")
    meta = torch.zeros((4, 2), device="cuda")
    with pytest.raises(MRGError):
        acc.cast_rays(dr, hits, meta)
    pos, idx, m = small(1, 1)
    acc.upload_mesh(pos, idx)
    acc.add_instance(0, m[0])
    acc.construct()
    acc.cast_rays(dr, hits, meta, count=0)
    acc.sync_status()
    with pytest.raises(MRGError):
        acc.add_instance(5, m[0])


@pytest.mark.parametrize("cull", [True, False])
def test_local_cast_matches_oracle(cull):
    """mrg_cast_local (CastLocalRays): random instance per listed ray, an index
    list over part of the rays, prefilled hits that misses keep; bit-exact
    against the oracle.  An out-of-range instance id skips its ray and is
    reported by mrg_sync_status."""
    import torch
    pos, idx, m = small(3, 8, seed=2)
    acc, S = build_pair(pos, idx, m, cull=cull)
    rays = scenes.primary_rays(96, 64, 9, eye=(0, 0, -10), tan_half_fov=0.35)   # ~29% of rays hit
    n = rays.shape[0]
    rng = np.random.default_rng(4)
    sel = np.sort(rng.permutation(n)[: n * 3 // 4]).astype(np.uint32)
    # two thirds: the instance of the ray's closest hit (when it hits); the rest random
    own = S.cast_closest(rays)[3][sel]
    ids = rng.integers(0, m.shape[0], sel.shape[0]).astype(np.uint32)
    take = (own != MISS) & (rng.random(sel.shape[0]) < 2.0 / 3.0)
    ids[take] = own[take]
    pre = np.full((n, 4), 0x5A5A5A5A, np.uint32)
    ora = S.cast_local(rays, ids, ray_idx=sel, hits=pre)
    dr = torch.from_numpy(rays.copy()).cuda()
    dh = torch.from_numpy(pre.view(np.int32).copy()).cuda()
    dm = torch.zeros((n, 2), dtype=torch.float32, device="cuda")
    di = torch.from_numpy(ids.view(np.int32)).cuda()
    ds = torch.from_numpy(sel.view(np.int32)).cuda()
    acc.cast_local_rays(dr, dh, dm, di, ray_idx=ds)
    acc.sync_status()
    got = (dr.cpu().numpy(), dh.cpu().numpy().view(np.uint32), dm.cpu().numpy())
    assert np.array_equal(got[0].view(np.uint32), ora[0].view(np.uint32))
    assert np.array_equal(got[1], ora[1])
    hit = ora[1][:, 0] != 0x5A5A5A5A
    assert hit.sum() > 400
    assert np.array_equal(got[2][hit].view(np.uint32), ora[2][hit].view(np.uint32))
    bad = torch.full((n,), m.shape[0], dtype=torch.int32, device="cuda")
    acc.cast_local_rays(dr, dh, dm, bad)
    with pytest.raises(MRGError):
        acc.sync_status()


def test_host_buffer_entry_point_matches_device():
    pos, idx, m = small(4, 27)
    acc, S = build_pair(pos, idx, m)
    rays = scenes.primary_rays(128, 96, 6, eye=(0, 0, -12), tan_half_fov=0.6)
    hr = rays.copy()
    hh = np.zeros((rays.shape[0], 4), np.uint32)
    hm = np.zeros((rays.shape[0], 2), np.float32)
    acc.cast_rays_host(hr, hh, hm)
    ora = S.cast_closest(rays)
    compare_closest(ora, (hr, hh, hm))


@pytest.mark.parametrize("chunks", ["1", "7", "32"])
def test_host_buffer_pipeline_chunks(chunks, monkeypatch):
    """The host-buffer cast moves the rays through in chunks (copy-in, cast,
    copy-out overlapped); any split gives the device-buffer results, and rays
    that miss keep the caller's hit and meta values."""
    pos, idx, m = small(4, 31)
    acc, _ = build_pair(pos, idx, m)
    rays = scenes.primary_rays(400, 250, 8, eye=(0, 0, -12), tan_half_fov=0.7)
    pre = np.full((rays.shape[0], 4), 0xABCD, np.uint32)
    want = gpu_closest(acc, rays, pre_hits=pre.copy())
    monkeypatch.setenv("MRG_HOST_CHUNKS", chunks)
    hr, hh = rays.copy(), pre.copy()
    hm = np.zeros((rays.shape[0], 2), np.float32)
    acc.cast_rays_host(hr, hh, hm)
    assert np.array_equal(hr.view(np.uint32), want[0].view(np.uint32))
    assert np.array_equal(hh, want[1])
    assert np.array_equal(hm.view(np.uint32), want[2].view(np.uint32))
    assert np.any(hh[:, 0] == 0xABCD) and np.any(hh[:, 0] != 0xABCD)


def test_stress_scene_full_size_parity():
    """1.31M-triangle icosphere x 64 instances, 1920x1080 primary rays plus
    one diffuse bounce (~4M rays) and shadow rays: bit-exact against the
    oracle at the benchmark's full size."""
    pos, idx, m, prim = stress_workload()
    acc, S = build_pair(pos, idx, m)
    ora_p = S.cast_closest(prim)
    gpu_p = gpu_closest(acc, prim)
    n, hits, ties = compare_closest(ora_p, gpu_p, retest=tri_retest(S, prim, pos, idx))
    assert hits > 0.8 * n
    bounce, src = scenes.bounce_rays(prim, ora_p[3], ora_p[1][:, 0] - 0x10000000, ora_p[0][:, 7],
                                     pos, idx, m, seed=1)
    ora_b = S.cast_closest(bounce)
    gpu_b = gpu_closest(acc, bounce)
    compare_closest(ora_b, gpu_b, retest=tri_retest(S, bounce, pos, idx))
    shadow = scenes.shadow_rays(bounce, (0.0, 80.0, -60.0))
    assert np.array_equal(gpu_visibility(acc, shadow), S.cast_visibility(shadow))
    st = acc.stats()
    assert st["blasTriangles"] == 1310720 and st["instances"] == 64 and st["accelerators"] == 1


def test_watertight_mode_matches_oracle():
    """The opt-in watertight triangle test: the GPU (records holding the three
    vertices, the WT kernel instantiation) against the oracle's watertight
    restatement, bit for bit, on closest and any-hit casts; and the
    watertightness itself on rays aimed at shared vertices and edges."""
    from test_watertight_host import _grid_mesh, _rays_at
    pos, idx, m = small(4, 27, seed=2)
    acc = Accelerator(0, watertight=True)
    S = oracle.Scene(watertight=True)
    mid = acc.upload_mesh(pos, idx, prim_key_base=0x10000000)
    oid = S.add_mesh(pos, idx, prim_key_base=0x10000000)
    for i in range(m.shape[0]):
        acc.add_instance(mid, m[i], light_or_mat_key=i, trans_key=(1 << 24) | i, accel_key=(2 << 20) | i)
        S.add_instance(oid, m[i], lm_key=i, trans_key=(1 << 24) | i, accel_key=(2 << 20) | i)
    acc.construct()
    S.build()
    rays = scenes.primary_rays(128, 96, 6, eye=(0, 0, -14), tan_half_fov=0.5)
    n, hits, ties = compare_closest(S.cast_closest(rays), gpu_closest(acc, rays),
                                    retest=tri_retest(S, rays, pos, idx, watertight=True))
    assert hits > 1000
    assert np.array_equal(gpu_visibility(acc, rays), S.cast_visibility(rays))
    acc.close()
    # a jittered grid, rays through its shared vertices and edges: the GPU
    # hits exactly what the oracle's brute force hits (no cracks in either)
    rng = np.random.default_rng(3)
    gpos, gidx, nrm = _grid_mesh(24, 1)
    inner = [j * 25 + i for j in range(1, 24) for i in range(1, 24)]
    targets = gpos[inner]
    rays = _rays_at(targets, nrm, rng)
    acc = Accelerator(0, watertight=True)
    S = oracle.Scene(watertight=True)
    acc.add_instance(acc.upload_mesh(gpos, gidx), np.eye(3, 4, dtype=np.float32).reshape(12), cull=False)
    S.add_instance(S.add_mesh(gpos, gidx), np.eye(3, 4, dtype=np.float32), cull=False)
    acc.construct()
    S.build()
    gr, gh, gm = gpu_closest(acc, rays)
    assert (gr[:, 7] < 1e29).all()          # every ray through a shared vertex hits
    lin = S.cast_closest(rays, linear=True)
    assert np.array_equal(gr[:, 7].view(np.uint32), lin[0][:, 7].view(np.uint32))
    acc.close()
