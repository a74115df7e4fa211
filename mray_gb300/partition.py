"""Host-side mirror of MRay's RayPartitioner::MultiPartition
(Source/Tracer/RayPartitioner.h:105-133, RayPartitioner.cu:263-411) over the
C ABI.  Buffers are device tensors; the work runs on the GPU.
"""
import ctypes as C

import torch

from . import _native as N
from .accel import _stream_ptr


class RayPartitioner:
    """Stable (batch, data)-bit sort of (key, index) pairs plus the runs of
    equal batch bits, on one GPU."""

    def __init__(self, device=0, max_partitions=4096):
        self._lib = N.lib()
        h = C.c_void_p()
        N.check(self._lib.mrg_create(C.byref(N.MrgParams(device=device)), C.byref(h)))
        self._h = h
        self.device = device
        self.max_partitions = max_partitions

    def close(self):
        if getattr(self, "_h", None):
            self._lib.mrg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def multi_partition(self, keys, indices=None, key_data_bits=(0, 0), key_batch_bits=(0, 32),
                        only_sort_for_batches=False, stream=None):
        """keys / indices: uint32 (int32-typed) CUDA tensors of n elements.
        Returns (count, offsets[count + 1], partition_keys[count],
        sorted_indices, sorted_keys) -- MultiPartitionOutput's fields."""
        n = int(keys.numel())
        dev = keys.device
        sk = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
        si = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
        cnt = torch.zeros(1, dtype=torch.int32, device=dev)
        off = torch.zeros(self.max_partitions + 1, dtype=torch.int32, device=dev)
        bk = torch.zeros(max(self.max_partitions, 1), dtype=torch.int32, device=dev)
        db = (C.c_uint32 * 2)(*key_data_bits)
        bb = (C.c_uint32 * 2)(*key_batch_bits)
        N.check(self._lib.mrg_multi_partition(
            self._h, C.c_void_p(keys.data_ptr()) if n else None,
            None if indices is None else C.c_void_p(indices.data_ptr()), n, db, bb,
            1 if only_sort_for_batches else 0, C.c_void_p(sk.data_ptr()), C.c_void_p(si.data_ptr()),
            C.c_void_p(cnt.data_ptr()), C.c_void_p(off.data_ptr()), C.c_void_p(bk.data_ptr()),
            self.max_partitions, _stream_ptr(stream)))
        torch.cuda.synchronize(dev)
        c = int(cnt.item())
        k = min(c, self.max_partitions)
        return c, off[:k + 1] if c <= self.max_partitions else off[:k], bk[:k], si[:n], sk[:n]
