"""The allocation-free host-buffer cast (mrg_cast_closest_host_noalloc).

Callers that cannot call cudaMalloc when they cast -- an application whose
own allocator owns every device allocation, or a real-time / plugin thread
that may not grow the device heap -- use this entry point: its device staging
and control words live in a static __device__ array inside the library.  Its
results must equal the allocating host-buffer entry point's (bit for bit, the
tolerance of every hit test here) on two calls in a row, since the array
keeps the previous call's contents.  The call must also leave the device's
free memory unchanged: its whole point is that nothing is allocated.

The file name sorts last so that a run which stops at the first failure has
already run every other test when this one runs; it also passes alone in a
fresh process (its fixtures build the library and the scene it needs).
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cast(fn, h, rays):
    r = rays.copy()
    hits = np.zeros((rays.shape[0], 4), np.uint32)
    meta = np.zeros((rays.shape[0], 2), np.float32)
    st = fn(h, r.ctypes.data_as(C.c_void_p), rays.shape[0], hits.ctypes.data_as(C.c_void_p),
            meta.ctypes.data_as(C.c_void_p))
    return st, r, hits, meta


def test_noalloc_cast_matches_allocating_entry_point(cuda_lib, built_libs):
    from mray_gb300 import Accelerator, scenes
    from mray_gb300 import _native as N
    pos, idx = scenes.icosphere(5, 1.0, 0.05, 4.0, 0)
    m = scenes.instance_field(27, 0, box=6.0, jitter=0.3)
    acc = Accelerator(0)
    mid = acc.upload_mesh(pos, idx, prim_key_base=0x10000000)
    for i in range(m.shape[0]):
        acc.add_instance(mid, m[i], light_or_mat_key=i, trans_key=(1 << 24) | i, accel_key=i)
    acc.construct()
    L = N.lib()
    h = acc._h
    import torch
    for seed, (w, hgt) in ((1, (512, 400)), (2, (300, 211))):      # two calls in a row
        rays = scenes.primary_rays(w, hgt, seed, eye=(0, 0, -10), tan_half_fov=0.45)
        assert rays.shape[0] <= N.MRG_NOALLOC_MAX_RAYS
        st0, r0, h0, m0 = _cast(L.mrg_cast_closest_host, h, rays)
        free0 = torch.cuda.mem_get_info(0)[0]
        st1, r1, h1, m1 = _cast(L.mrg_cast_closest_host_noalloc, h, rays)
        free1 = torch.cuda.mem_get_info(0)[0]
        assert st0 == N.MRG_OK and st1 == N.MRG_OK, L.mrg_last_error()
        # the allocating call ran the same kernel just before, so any lazy
        # driver set-up is done: the no-allocation call must not move free memory
        assert free1 == free0, (free0, free1)
        assert np.array_equal(r0.view(np.uint32), r1.view(np.uint32))
        assert np.array_equal(h0, h1)
        assert np.array_equal(m0.view(np.uint32), m1.view(np.uint32))
        assert (r1[:, 7] < 3e38).sum() > 1000
    big = np.zeros((N.MRG_NOALLOC_MAX_RAYS + 1, 8), np.float32)
    st, *_ = _cast(L.mrg_cast_closest_host_noalloc, h, big)
    assert st == N.MRG_ERR_LIMIT
    assert b"MRG_NOALLOC_MAX_RAYS" in L.mrg_last_error()
    acc.close()
