"""ZSobol on the GPU (mrg_zsobol_generate) against the oracle's restatement,
bit for bit: odd and even powers of four of samples, sample indices past the
initial count (rotation into doubled blocks), non-square images whose sides
are not powers of two, and request lists mixing 1D, 2D and 3D requests."""
import numpy as np
import pytest
import torch

import oracle
from mray_gb300 import zsobol

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("w,h,spp", [(64, 48, 4), (37, 21, 8), (1, 1, 1), (300, 7, 16)])
def test_zsobol_matches_oracle(w, h, spp):
    seeds = zsobol.seeds(w, h, 0xABCDEF0123)
    assert np.array_equal(seeds, oracle.zsobol_seeds(w, h, 0xABCDEF0123))
    d_seeds = torch.from_numpy(seeds.view(np.int32)).cuda()
    for req, dim0 in (([2, 1, 3, 2], 0), ([1], 7), ([3, 3, 2, 1, 1, 2], 11)):
        for s in (0, 1, spp - 1, spp, 3 * spp + 1, 13 * spp + 5):
            got = zsobol.generate(w, h, d_seeds, spp, s, dim0, req).cpu().numpy().view(np.uint32)
            ref = oracle.zsobol_generate(w, h, seeds, spp, s, dim0, req)
            assert np.array_equal(got, ref), (w, h, spp, req, dim0, s)


def test_zsobol_full_hd_frame():
    """One 1920x1080 sample, eight 2D requests, against the oracle."""
    w, h = 1920, 1080
    seeds = zsobol.seeds(w, h, 42)
    d_seeds = torch.from_numpy(seeds.view(np.int32)).cuda()
    got = zsobol.generate(w, h, d_seeds, 64, 37, 0, [2] * 8).cpu().numpy().view(np.uint32)
    ref = oracle.zsobol_generate(w, h, seeds, 64, 37, 0, [2] * 8)
    assert np.array_equal(got, ref)
