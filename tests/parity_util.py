"""Shared helpers for the GPU parity tests: build the same scene in the CUDA
accelerator (through the C ABI) and in the CPU oracle, cast the same rays,
compare bit for bit (closest hits may differ only on exact-t ties)."""
import numpy as np

import oracle
from mray_gb300 import Accelerator, scenes

MISS = 0xFFFFFFFF
PRIM_BASE = 0x10000000


def inst_trans_key(i):
    return (1 << 24) | i


def build_pair(pos, idx, mats, cull=True, corrected=False):
    acc = Accelerator(0)
    S = oracle.Scene()
    mid = acc.upload_mesh(pos, idx, prim_key_base=PRIM_BASE)
    oid = S.add_mesh(pos, idx, prim_key_base=PRIM_BASE)
    for i in range(mats.shape[0]):
        kw = dict(cull=cull, corrected_inverse=corrected)
        acc.add_instance(mid, mats[i], light_or_mat_key=100 + i, trans_key=inst_trans_key(i),
                         accel_key=(2 << 20) | i, **kw)
        S.add_instance(oid, mats[i], lm_key=100 + i, trans_key=inst_trans_key(i),
                       accel_key=(2 << 20) | i, **kw)
    acc.construct()
    S.build()
    return acc, S


def gpu_closest(acc, rays, ray_idx=None, pre_hits=None):
    import torch
    dr = torch.from_numpy(np.ascontiguousarray(rays)).cuda()
    n = rays.shape[0]
    hits = torch.zeros((n, 4), dtype=torch.int32, device="cuda") if pre_hits is None else \
        torch.from_numpy(pre_hits.view(np.int32)).cuda()
    meta = torch.zeros((n, 2), dtype=torch.float32, device="cuda")
    ridx = None if ray_idx is None else torch.from_numpy(np.ascontiguousarray(ray_idx, np.uint32).view(np.int32)).cuda()
    acc.cast_rays(dr, hits, meta, ray_idx=ridx)
    acc.sync_status()
    return dr.cpu().numpy(), hits.cpu().numpy().view(np.uint32), meta.cpu().numpy()


def gpu_visibility(acc, rays, ray_idx=None, pre_bits=None):
    import torch
    n = rays.shape[0]
    words = (n + 31) // 32
    dr = torch.from_numpy(np.ascontiguousarray(rays)).cuda()
    bits = torch.zeros(words, dtype=torch.int32, device="cuda") if pre_bits is None else \
        torch.from_numpy(pre_bits.view(np.int32).copy()).cuda()
    ridx = None if ray_idx is None else torch.from_numpy(np.ascontiguousarray(ray_idx, np.uint32).view(np.int32)).cuda()
    acc.cast_visibility_rays(bits, dr, ray_idx=ridx)
    acc.sync_status()
    return bits.cpu().numpy().view(np.uint32)


def tri_retest(S, rays, pos, idx, prim_base=PRIM_BASE, cull=True, watertight=False,
               inst_of=lambda keys: int(keys[2] & 0xFFFFFF)):
    """A re-test for compare_closest: the GPU's reported triangle, intersected
    by the oracle's triangle test in the reported instance's space (the
    oracle's own inverse), must give exactly the reported t and barycentrics.
    Instance = low 24 bits of the transform key (build_pair's keys)."""
    import ctypes as C
    L = oracle.lib()
    vp = C.c_void_p
    fn = L.orc_intersect_triangle_wt if watertight else L.orc_intersect_triangle

    def check(k, keys, meta, tval):
        inst = inst_of(keys)
        prim = int(keys[0]) - prim_base
        if prim < 0 or prim >= idx.shape[0]:
            return False
        inv = np.ascontiguousarray(S.instance_inverse(inst), np.float32)
        d = np.ascontiguousarray(rays[k, 4:7], np.float32)
        p = np.ascontiguousarray(rays[k, 0:3], np.float32)
        ld = np.zeros(3, np.float32)
        lp = np.zeros(3, np.float32)
        L.orc_transform_ray(inv.ctypes.data_as(vp), d.ctypes.data_as(vp), p.ctypes.data_as(vp),
                            ld.ctypes.data_as(vp), lp.ctypes.data_as(vp))
        v = np.ascontiguousarray(pos[idx[prim]], np.float32)
        b = np.zeros(3, np.float32)
        t = np.zeros(1, np.float32)
        bf = np.zeros(1, np.int32)
        hit = fn(ld.ctypes.data_as(vp), lp.ctypes.data_as(vp), v[0].ctypes.data_as(vp), v[1].ctypes.data_as(vp),
                 v[2].ctypes.data_as(vp), 1 if cull else 0, b.ctypes.data_as(vp), t.ctypes.data_as(vp),
                 bf.ctypes.data_as(vp))
        return bool(hit) and t.view(np.uint32)[0] == np.float32(tval).view(np.uint32) and \
            np.array_equal(b[:2].view(np.uint32), np.asarray(meta, np.float32).view(np.uint32))
    return check


def compare_closest(ora, gpu, listed=None, retest=None):
    """ora = (rays, hits, meta, inst) from the oracle; gpu = (rays, hits, meta).
    Returns (n_compared, n_hits, n_ties).  Asserts bit equality except on
    exact-t ties between different primitives: the t must be the same, and
    every such ray is re-tested (retest(k, gpu keys, gpu meta, gpu t), e.g.
    tri_retest): the GPU's primitive must give exactly its reported t and
    barycentrics.  Without a re-test no difference is accepted."""
    orays, ohits, ometa, oinst = ora
    grays, ghits, gmeta = gpu
    n = orays.shape[0]
    sel = np.arange(n) if listed is None else np.asarray(listed)
    ot = orays[sel, 7].view(np.uint32)
    gt = grays[sel, 7].view(np.uint32)
    assert np.array_equal(ot, gt), "t mismatch on %d rays (first %s)" % (
        int((ot != gt).sum()), sel[np.nonzero(ot != gt)[0][:5]])
    same_keys = (ohits[sel] == ghits[sel]).all(axis=1)
    same_meta = (ometa[sel].view(np.uint32) == gmeta[sel].view(np.uint32)).all(axis=1)
    ok = same_keys & same_meta
    ties = int((~ok).sum())
    # a difference is only acceptable as a tie: same t, different primitive,
    # and the GPU's primitive really is hit at exactly that t
    if ties:
        bad = sel[~ok]
        assert (oinst[bad] != MISS).all()
        assert retest is not None, "%d key / barycentric differences and no re-test" % ties
        failed = [int(k) for k in bad if not retest(int(k), ghits[k], gmeta[k], grays[k, 7])]
        assert not failed, "GPU hits that do not re-test: %s" % failed[:5]
    hitn = int((oinst[sel] != MISS).sum())
    assert ties <= max(2, hitn // 10000), "%d non-tie-looking differences" % ties
    return len(sel), hitn, ties


def stress_workload(level=8, instances=64, width=1920, height=1080, seed=0):
    pos, idx, m = scenes.bvh_stress_scene(level=level, instances=instances, seed=seed)
    prim = scenes.primary_rays(width, height, seed)
    return pos, idx, m, prim
