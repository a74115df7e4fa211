"""Radiance cache over the C ABI (include/mray_gb300.h, "Radiance cache"):
hash-grid encoding + fully fused BF16 tensor-core MLP, trained online with
Adam.  Buffers are CUDA tensors; parameters transfer as numpy arrays."""
import ctypes as C

import numpy as np

from . import _native as N
from .accel import _stream_ptr

WEIGHTS = 5 * 64 * 64 + 16 * 64          # hidden W0..W4 [64][64], output W5 [16][64]


class RadianceCache:
    def __init__(self, owner=None, device=0, levels=16, log2_table_size=19, base_resolution=16,
                 max_resolution=2048, learning_rate=1e-2, beta1=0.9, beta2=0.99, epsilon=1e-15, seed=0,
                 max_batch=65536, aabb=(0, 0, 0, 1, 1, 1)):
        """owner: an Accelerator / PathTracer whose context hosts the cache
        (the path tracer's cache mode uses it), or None for a private one."""
        self._lib = N.lib()
        self._own = owner is None
        if owner is None:
            h = C.c_void_p()
            N.check(self._lib.mrg_create(C.byref(N.MrgParams(device=device)), C.byref(h)))
            self._h = h
        else:
            acc = getattr(owner, "acc", owner)
            self._h = acc._h
            self._owner = owner
        p = N.MrgCacheParams(levels=levels, log2_table_size=log2_table_size, base_resolution=base_resolution,
                             max_resolution=max_resolution, learning_rate=learning_rate, beta1=beta1, beta2=beta2,
                             epsilon=epsilon, seed=seed, max_batch=max_batch)
        p.aabb[:] = [float(x) for x in aabb]
        N.check(self._lib.mrg_cache_create(self._h, C.byref(p)))
        self.table_size = levels * (1 << log2_table_size) * 2
        self.levels, self.log2_table_size = levels, log2_table_size
        self.base_resolution, self.max_resolution, self.aabb = base_resolution, max_resolution, tuple(aabb)

    def close(self):
        if self._own and getattr(self, "_h", None):
            self._lib.mrg_destroy(self._h)
        self._h = None

    def query(self, inputs, out=None, stream=None):
        """inputs: (n, 16) float32 CUDA tensor; returns (n, 4)."""
        import torch
        n = inputs.shape[0]
        if out is None:
            out = torch.empty((n, 4), dtype=torch.float32, device=inputs.device)
        N.check(self._lib.mrg_cache_query(self._h, C.c_void_p(inputs.data_ptr()), n, C.c_void_p(out.data_ptr()),
                                          _stream_ptr(stream)))
        return out

    def train(self, inputs, targets, loss=True, stream=None):
        l = C.c_float(0.0)
        N.check(self._lib.mrg_cache_train(self._h, C.c_void_p(inputs.data_ptr()), C.c_void_p(targets.data_ptr()),
                                          inputs.shape[0], C.byref(l) if loss else None, _stream_ptr(stream)))
        return l.value if loss else None

    def gradients(self, inputs, targets):
        gw = np.zeros(WEIGHTS, np.float32)
        gt = np.zeros(self.table_size, np.float32)
        l = C.c_float(0.0)
        N.check(self._lib.mrg_cache_gradients(self._h, C.c_void_p(inputs.data_ptr()), C.c_void_p(targets.data_ptr()),
                                              inputs.shape[0], gw.ctypes.data_as(N.fp), gt.ctypes.data_as(N.fp),
                                              C.byref(l)))
        return l.value, gw, gt

    def get_params(self):
        w = np.zeros(WEIGHTS, np.float32)
        t = np.zeros(self.table_size, np.float32)
        N.check(self._lib.mrg_cache_get_params(self._h, w.ctypes.data_as(N.fp), t.ctypes.data_as(N.fp)))
        return w, t

    def set_params(self, weights=None, table=None):
        w = None if weights is None else np.ascontiguousarray(weights, np.float32)
        t = None if table is None else np.ascontiguousarray(table, np.float32)
        N.check(self._lib.mrg_cache_set_params(self._h, None if w is None else w.ctypes.data_as(N.fp),
                                               None if t is None else t.ctypes.data_as(N.fp)))
