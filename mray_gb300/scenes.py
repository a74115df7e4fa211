"""Seeded synthetic workloads (numpy front end of libmrg_scenes.so).

``bvh_stress_scene`` is the 1.31M-triangle displaced icosphere instanced 64
times with rigid transforms inside a 100^3 cube; ``primary_rays`` /
``bounce_rays`` build its 1920x1080 primary + one-diffuse-bounce ray set.
All generators use only IEEE basic operations, so the same seed gives the same
bits on every host.
"""
import ctypes as C

import numpy as np

from . import _native as N

FLT_MAX = np.float32(3.4028235e38)

# 1.31M-triangle stress scene
STRESS_LEVEL = 8              # 20 * 4^8 = 1,310,720 triangles
STRESS_RADIUS = 11.0
STRESS_NOISE_AMP = 0.05       # relative to the radius, 3-octave value noise
STRESS_NOISE_FREQ = 4.0
STRESS_INSTANCES = 64
STRESS_BOX = 100.0
STRESS_JITTER = 1.5
STRESS_EYE = (0.0, 0.0, -90.0)
STRESS_TARGET = (0.0, 0.0, 0.0)
STRESS_UP = (0.0, 1.0, 0.0)
STRESS_TAN_HALF_FOV = 0.5


def _vp(a):
    return a.ctypes.data_as(C.c_void_p)


def _d3(v):
    return (C.c_double * 3)(*[float(x) for x in v])


def icosphere(level, radius=1.0, noise_amp=0.0, noise_freq=4.0, seed=0):
    s = N.scenes_lib()
    nv, nt = C.c_uint32(), C.c_uint32()
    s.mrgs_icosphere_counts(level, C.byref(nv), C.byref(nt))
    pos = np.empty((nv.value, 3), np.float32)
    idx = np.empty((nt.value, 3), np.uint32)
    rc = s.mrgs_icosphere(level, radius, noise_amp, noise_freq, seed, _vp(pos), _vp(idx))
    if rc != 0:
        raise RuntimeError("icosphere generation failed (%d)" % rc)
    return pos, idx


def instance_field(count, seed=0, box=STRESS_BOX, jitter=STRESS_JITTER):
    m = np.empty((count, 12), np.float32)
    N.scenes_lib().mrgs_instance_field(count, seed, box, jitter, _vp(m))
    return m


def bvh_stress_scene(level=STRESS_LEVEL, instances=STRESS_INSTANCES, seed=0):
    """(pos, idx, transforms) of the displaced-icosphere instance field."""
    pos, idx = icosphere(level, STRESS_RADIUS, STRESS_NOISE_AMP, STRESS_NOISE_FREQ, seed)
    m = instance_field(instances, seed)
    return pos, idx, m


def primary_rays(width, height, seed=0, eye=STRESS_EYE, target=STRESS_TARGET, up=STRESS_UP,
                 tan_half_fov=STRESS_TAN_HALF_FOV):
    rays = np.empty((width * height, 8), np.float32)
    N.scenes_lib().mrgs_primary_rays(width, height, _d3(eye), _d3(target), _d3(up),
                                     tan_half_fov, seed, _vp(rays))
    return rays


def bounce_rays(primary, hit_inst, hit_prim, hit_t, pos, idx, m34, seed=0):
    """One cosine-weighted diffuse ray per primary hit.  Returns (rays, src)."""
    n = primary.shape[0]
    out = np.empty((n, 8), np.float32)
    src = np.empty(n, np.uint32)
    hi = np.ascontiguousarray(hit_inst, np.uint32)
    hp = np.ascontiguousarray(hit_prim, np.uint32)
    ht = np.ascontiguousarray(hit_t, np.float32)
    m = N.scenes_lib().mrgs_bounce_rays(n, _vp(primary), _vp(hi), _vp(hp), _vp(ht),
                                        _vp(np.ascontiguousarray(pos, np.float32)),
                                        _vp(np.ascontiguousarray(idx, np.uint32)),
                                        _vp(np.ascontiguousarray(m34, np.float32)),
                                        seed, _vp(out), _vp(src))
    return out[:m].copy(), src[:m].copy()


def shadow_rays(origins, light):
    out = np.empty_like(origins)
    N.scenes_lib().mrgs_shadow_rays(origins.shape[0], _vp(origins), _d3(light), _vp(out))
    return out
