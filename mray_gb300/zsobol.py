"""MRay's ZSobol random-number group (RNGGroupZSobol, Source/Tracer/Random.h:454-523,
Random.cu:1147-1380) on the GPU: ``seeds`` gives the per-pixel seeds of a
width x height image and ``generate`` one sample's numbers for every pixel, for
an RNRequestList given as a list of request sizes (1..3 numbers each)."""
import ctypes as C

import numpy as np

from . import _native as N


def seeds(width, height, seed):
    """Per-pixel seeds (row-major uint32), as RNGGroupZSobol's constructor
    draws them from std::mt19937."""
    out = np.zeros(width * height, np.uint32)
    N.check(N.lib().mrg_zsobol_seeds(width, height, seed, out.ctypes.data_as(C.c_void_p)))
    return out


def encode_requests(requests):
    """RNRequestList: request r's size in bits 2r..2r+1."""
    enc = 0
    for r, d in enumerate(requests):
        if d not in (1, 2, 3):
            raise ValueError("request sizes are 1, 2 or 3")
        enc |= int(d) << (2 * r)
    return enc, len(requests)


def generate(width, height, d_seeds, initial_max_spp, sample_index, dim_start, requests, out=None, stream=None):
    """Numbers of sample ``sample_index`` of every pixel: a (total numbers,
    width * height) uint32 CUDA tensor (number k of pixel i at [k, i])."""
    import torch
    enc, count = encode_requests(requests)
    total = int(sum(requests))
    if out is None:
        out = torch.zeros((total, width * height), dtype=torch.int32, device=d_seeds.device)
    N.check(N.lib().mrg_zsobol_generate(width, height, C.c_void_p(d_seeds.data_ptr()), initial_max_spp,
                                        sample_index, dim_start, enc, count, C.c_void_p(out.data_ptr()),
                                        None if stream is None else C.c_void_p(stream.cuda_stream)))
    return out
