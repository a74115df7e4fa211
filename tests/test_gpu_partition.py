"""GPU MultiPartition (hand-written multi-split radix passes) against the
oracle's restatement: bit-exact sorted keys, sorted indices, partition
offsets and keys, including ties (stability), empty and single inputs,
non-multiple-of-tile sizes, 32-bit keys (four digit passes) and MRay's
maximum path count (2^21, Source/Core/TracerI.h:54)."""
import numpy as np
import pytest
import torch

import oracle
from mray_gb300.partition import RayPartitioner

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rp():
    r = RayPartitioner(0, max_partitions=1 << 16)
    yield r
    r.close()


def _t(a):
    return torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32)).cuda()


def _u(t):
    return t.cpu().numpy().view(np.uint32)


def _check(rp, keys, idx, data, batch, only=False):
    got = rp.multi_partition(_t(keys), None if idx is None else _t(idx), data, batch, only)
    want = oracle.multi_partition(keys, idx, data, batch, only)
    assert got[0] == want[0]
    assert np.array_equal(_u(got[1]), want[1])
    assert np.array_equal(_u(got[2]), want[2])
    assert np.array_equal(_u(got[3]), want[3])
    assert np.array_equal(_u(got[4]), want[4])
    return got


def test_reference_simulation(rp):
    """T_RayPartitioner.cu's layout: 16 batches in bits 28-31, 256 data values
    in bits 0-7; every partition non-empty and every ray in one."""
    rng = np.random.default_rng(333)
    n = 1 << 20
    keys = ((rng.integers(0, 16, n) << 28) | rng.integers(0, 256, n)).astype(np.uint32)
    got = _check(rp, keys, np.arange(n, dtype=np.uint32), (0, 8), (28, 32))
    assert got[0] == 16
    assert np.all(np.diff(_u(got[1]).astype(np.int64)) > 0)


@pytest.mark.parametrize("n", [0, 1, 2, 2047, 2048, 2049, 100003])
def test_sizes(rp, n):
    rng = np.random.default_rng(n)
    keys = rng.integers(0, 1 << 12, n).astype(np.uint32)
    idx = rng.permutation(n).astype(np.uint32)
    _check(rp, keys, idx, (0, 6), (6, 12))


def test_ties_are_stable(rp):
    keys = np.repeat(np.array([7, 3, 7, 1], np.uint32), 5000)
    _check(rp, keys, None, (0, 2), (2, 3))
    _check(rp, np.zeros(70000, np.uint32), None, (0, 1), (1, 2))       # one partition


def test_full_32_bit_keys_and_only_batches(rp):
    rng = np.random.default_rng(9)
    keys = rng.integers(0, 2 ** 32, 300000, dtype=np.uint64).astype(np.uint32)
    _check(rp, keys, None, (0, 20), (20, 32))                           # four passes
    _check(rp, keys, None, (0, 0), (24, 32), only=True)
    _check(rp, keys, None, (28, 32), (0, 4))                            # data above batch


def test_max_path_count(rp):
    rng = np.random.default_rng(21)
    n = 1 << 21
    keys = ((rng.integers(0, 40, n) << 24) | rng.integers(0, 1 << 24, n)).astype(np.uint32)
    _check(rp, keys, np.arange(n, dtype=np.uint32)[::-1].copy(), (0, 24), (24, 30))


def test_partition_cap(rp):
    """More runs than max_partitions: the count is exact, the stored runs
    are the first max_partitions."""
    small = RayPartitioner(0, max_partitions=8)
    keys = np.arange(100, dtype=np.uint32)
    c, off, pk, si, sk = small.multi_partition(_t(keys), None, (0, 0), (0, 8), True)
    assert c == 100 and np.array_equal(_u(pk), np.arange(8)) and np.array_equal(_u(off), np.arange(8))
    small.close()
