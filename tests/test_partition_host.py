"""MultiPartition restatement (oracle) on small inputs against a plain
Python stable sort; the bit-range arithmetic of the reference's own
simulation (Source/Tests/Tracer/T_RayPartitioner.cu:33-47).  CPU only."""
import numpy as np

import oracle


def _py(keys, idx, data, batch, only):
    def bits(v, r):
        return (v >> r[0]) & ((1 << (r[1] - r[0])) - 1)
    def comp(k):
        c = bits(k, batch)
        return c if only else (c << (data[1] - data[0])) | bits(k, data)
    pairs = sorted(zip(keys, idx), key=lambda p: comp(p[0]))     # sorted() is stable
    sk = [p[0] for p in pairs]
    starts = [j for j in range(len(sk)) if j == 0 or bits(sk[j], batch) != bits(sk[j - 1], batch)]
    return len(starts), starts + [len(sk)], [sk[j] for j in starts], [p[1] for p in pairs], sk


def test_restatement_matches_python_stable_sort():
    rng = np.random.default_rng(1)
    for data, batch, only in [((0, 8), (28, 32), False), ((0, 4), (4, 9), False), ((3, 7), (20, 24), True)]:
        keys = rng.integers(0, 2 ** 32, 700, dtype=np.uint64).astype(np.uint32)
        keys[::7] = keys[0]                                  # ties
        idx = rng.permutation(700).astype(np.uint32)
        got = oracle.multi_partition(keys, idx, data, batch, only)
        want = _py([int(x) for x in keys], [int(x) for x in idx], data, batch, only)
        assert got[0] == want[0]
        assert list(got[1]) == want[1] and list(got[2]) == want[2]
        assert list(got[3]) == want[3] and list(got[4]) == want[4]


def test_reference_simulation_layout():
    """16 batches (bits 28-31) x 256 data values (bits 0-7): every partition
    non-empty, their union is every ray."""
    rng = np.random.default_rng(333)
    n = 4096
    keys = ((rng.integers(0, 16, n) << 28) | rng.integers(0, 256, n)).astype(np.uint32)
    c, off, pk, si, sk = oracle.multi_partition(keys, None, (0, 8), (28, 32))
    assert c == 16 and np.all(np.diff(off) > 0) and off[-1] == n
    assert np.array_equal(np.sort(si), np.arange(n))
    assert np.array_equal(pk >> 28, np.arange(16))


def test_empty_and_single():
    c, off, pk, si, sk = oracle.multi_partition(np.zeros(0, np.uint32))
    assert c == 0 and list(off) == [0]
    c, off, pk, si, sk = oracle.multi_partition(np.array([5], np.uint32), None, (0, 2), (2, 4))
    assert c == 1 and list(off) == [0, 1] and list(pk) == [5]
