"""Host-side mirror of MRay's accelerator interface over the C ABI.

``Accelerator`` follows ``BaseAcceleratorI`` (Source/Tracer/AcceleratorC.h:375-430):
``construct`` (BaseAccelerator::Construct), ``cast_rays`` (CastRays),
``cast_visibility_rays`` (CastVisibilityRays), ``scene_aabb`` (SceneAABB).
Buffers are device tensors (torch is used only to own device memory and
streams); ``cast_rays_host`` takes numpy arrays and goes through the
host-buffer entry point.  Errors raise ``MRGError``, the analogue of MRay's
``MRayError`` crossing the TracerI boundary.
"""
import ctypes as C

import numpy as np

from . import _native as N

RAY_FLOATS = 8          # RayGMem: pos[3], tMin, dir[3], tMax
HIT_WORDS = 4           # HitKeyPack
META_FLOATS = 2         # MetaHit (triangle barycentrics)


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream_ptr(stream):
    if stream is None:
        return None
    return C.c_void_p(int(stream.cuda_stream) if hasattr(stream, "cuda_stream") else int(stream))


class Accelerator:
    """Two-level 8-wide BVH accelerator on one GPU."""

    def __init__(self, device=0, watertight=False):
        """watertight: the watertight triangle test (Woop, Benthin and Wald
        2013) instead of MRay's Moller-Trumbore test for every cast of this
        accelerator."""
        self._lib = N.lib()
        p = N.MrgParams(device=device,
                        triangle_test=N.MRG_TRI_WATERTIGHT if watertight else N.MRG_TRI_MOLLER_TRUMBORE)
        h = C.c_void_p()
        N.check(self._lib.mrg_create(C.byref(p), C.byref(h)))
        self._h = h
        self.device = device

    def close(self):
        if getattr(self, "_h", None):
            self._lib.mrg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- scene ----------------------------------------------------------------
    def upload_mesh(self, pos, idx, prim_key_base=0):
        pos = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 3)
        idx = np.ascontiguousarray(idx, dtype=np.uint32).reshape(-1, 3)
        out = C.c_uint32()
        N.check(self._lib.mrg_upload_mesh(self._h, pos.ctypes.data_as(C.c_void_p), pos.shape[0],
                                          idx.ctypes.data_as(C.c_void_p), idx.shape[0],
                                          prim_key_base, C.byref(out)))
        return out.value

    def add_instance(self, mesh_id, m34, cull=True, light_or_mat_key=0, trans_key=0,
                     accel_key=0, corrected_inverse=False):
        m = np.ascontiguousarray(m34, dtype=np.float32).reshape(12)
        out = C.c_uint32()
        flags = (N.MRG_INSTANCE_CULL_BACKFACE if cull else 0) | \
            (N.MRG_INSTANCE_CORRECTED_INVERSE if corrected_inverse else 0)
        N.check(self._lib.mrg_add_instance(self._h, mesh_id, m.ctypes.data_as(N.fp), flags,
                                           light_or_mat_key, trans_key, accel_key, C.byref(out)))
        return out.value

    def construct(self):
        N.check(self._lib.mrg_build(self._h))

    def scene_aabb(self):
        out = (C.c_float * 6)()
        N.check(self._lib.mrg_scene_aabb(self._h, out))
        return np.array(out[:], dtype=np.float32)

    def stats(self):
        s = N.MrgAccelStats()
        N.check(self._lib.mrg_get_stats(self._h, C.byref(s)))
        return {f: getattr(s, f) for f, _ in s._fields_}

    # -- casts ----------------------------------------------------------------
    def cast_rays(self, rays, hits, meta, ray_idx=None, count=None, stream=None):
        """Closest hit on device buffers (CastRays).  rays: float32 [N, 8]
        (updated tMax on hit), hits: int32/uint32 [N, 4], meta: float32 [N, 2]."""
        n = int(ray_idx.numel()) if ray_idx is not None else int(rays.shape[0])
        if count is not None:
            n = int(count)
        N.check(self._lib.mrg_cast_closest(self._h, _ptr(rays), _ptr(ray_idx), n, _ptr(hits),
                                           _ptr(meta), _stream_ptr(stream)))

    def cast_local_rays(self, rays, hits, meta, inst_ids, ray_idx=None, stream=None):
        """Local cast on device buffers (CastLocalRays): listed ray i against
        instance inst_ids[i] only.  inst_ids: int32/uint32 [n], n = the list
        length (ray_idx) or the ray count."""
        n = int(ray_idx.numel()) if ray_idx is not None else int(rays.shape[0])
        if int(inst_ids.numel()) != n:
            raise ValueError("cast_local_rays: one instance id per listed ray")
        N.check(self._lib.mrg_cast_local(self._h, _ptr(rays), _ptr(ray_idx), _ptr(inst_ids), n, _ptr(hits),
                                         _ptr(meta), _stream_ptr(stream)))

    def cast_visibility_rays(self, visible_bits, rays, ray_idx=None, count=None, stream=None):
        """Any hit (CastVisibilityRays) into a device bitspan of 32-bit words."""
        n = int(ray_idx.numel()) if ray_idx is not None else int(rays.shape[0])
        if count is not None:
            n = int(count)
        N.check(self._lib.mrg_cast_visibility(self._h, _ptr(visible_bits), _ptr(rays),
                                              _ptr(ray_idx), n, _stream_ptr(stream)))

    def cast_rays_host(self, rays, hits, meta):
        """Closest hit on host numpy buffers (copies in and out, synchronous)."""
        for a, dt in ((rays, np.float32), (hits, np.uint32), (meta, np.float32)):
            if a.dtype != dt or not a.flags.c_contiguous:
                raise TypeError("host buffers must be C-contiguous %s" % dt)
        N.check(self._lib.mrg_cast_closest_host(self._h, rays.ctypes.data_as(C.c_void_p),
                                                rays.shape[0], hits.ctypes.data_as(C.c_void_p),
                                                meta.ctypes.data_as(C.c_void_p)))

    def sync_status(self, stream=None):
        N.check(self._lib.mrg_sync_status(self._h, _stream_ptr(stream)))

    def traversal_counts(self, rays, stream=None):
        out = (C.c_uint64 * 8)()
        N.check(self._lib.mrg_cast_closest_stats(self._h, _ptr(rays), int(rays.shape[0]), out,
                                                 _stream_ptr(stream)))
        return {"rays": out[0], "node_visits": out[1], "tri_tests": out[2],
                "instance_entries": out[3], "tlas_node_visits": out[4], "dry_instance_entries": out[5]}
