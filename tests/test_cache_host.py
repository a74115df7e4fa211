"""FP64 radiance-cache reference (oracle/nrc.py): its gradients against
central finite differences of its own loss.  CPU only."""
import numpy as np

from oracle import nrc


def _batch(n, seed):
    rng = np.random.default_rng(seed)
    x = np.zeros((n, 16), np.float32)
    x[:, 0:3] = rng.random((n, 3))
    x[:, 3] = rng.random(n)
    d = rng.standard_normal((n, 3))
    x[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    nn = rng.standard_normal((n, 3))
    x[:, 8:11] = nn / np.linalg.norm(nn, axis=1, keepdims=True)
    x[:, 12:15] = rng.random((n, 3))
    t = np.zeros((n, 4), np.float32)
    t[:, :3] = rng.random((n, 3)) * 2.0
    return x, t


def test_reference_gradients_match_finite_differences():
    ref = nrc.CacheRef(levels=4, log2_table=8, base=4, max_res=32)
    rng = np.random.default_rng(0)
    w = rng.uniform(-0.3, 0.3, nrc.WEIGHTS)
    tab = rng.uniform(-0.5, 0.5, 4 * 256 * 2)
    x, t = _batch(64, 1)
    loss, gw, gt = ref.gradients(x, t, w, tab)
    y0 = ref.query(x, w, tab)
    den = y0 * y0 + 0.01                      # the stop-gradient denominator, frozen

    def L(w_, t_):
        return ref.gradients(x, t, w_, t_, den=den)[0]
    h = 1e-6
    for i in rng.choice(len(w), 12, replace=False):
        wp, wm = w.copy(), w.copy()
        wp[i] += h
        wm[i] -= h
        fd = (L(wp, tab) - L(wm, tab)) / (2 * h)
        assert abs(fd - gw[i]) <= 1e-5 * max(1.0, abs(fd)), (i, fd, gw[i])
    live = np.nonzero(gt)[0]
    for i in rng.choice(live, 8, replace=False):
        tp, tm = tab.copy(), tab.copy()
        tp[i] += h
        tm[i] -= h
        fd = (L(w, tp) - L(w, tm)) / (2 * h)
        assert abs(fd - gt[i]) <= 1e-5 * max(1.0, abs(fd)), (i, fd, gt[i])


def test_bf16_rounding():
    a = np.array([1.0, 1.00390625, 1.001953125, 3.14159265, -2.5e-3], np.float64)
    r = nrc.round_bf16(a)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0               # ties to even
    assert nrc.round_bf16(np.array([1.01171875]))[0] == 1.015625
    assert abs(r[3] - 3.140625) < 1e-9 and r[4] < 0
