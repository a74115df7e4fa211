"""FP64 reference of the radiance cache (TEST INFRASTRUCTURE ONLY).

Project-written (MRay has no learned cache): the multiresolution hash-grid
encoding (Mueller et al. 2022), the MLP of 5 hidden 64-wide ReLU layers and a
16-wide output layer without biases, the relative L2 loss and its gradients,
in float64 numpy.  ``bf16=True`` rounds what the GPU holds in BF16 (inputs,
weights, activations, the per-sample gradient rows) so that GPU results can
be compared tightly; ``bf16=False`` is the plain FP64 model.
"""
import numpy as np

WIDTH, OUT, HIDDEN = 64, 16, 5
LAYERS = HIDDEN + 1                       # hidden layers + the output layer
WEIGHTS = HIDDEN * WIDTH * WIDTH + OUT * WIDTH
PRIMES = (1, 2654435761, 805459861)


def round_bf16(a):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def split_weights(w):
    w = np.asarray(w, np.float64)
    mats = [w[i * 4096:(i + 1) * 4096].reshape(64, 64) for i in range(HIDDEN)]
    mats.append(w[HIDDEN * 4096:HIDDEN * 4096 + 1024].reshape(16, 64))
    return mats


def join_weights(mats):
    return np.concatenate([m.ravel() for m in mats])


def sh16(d):
    x, y, z = d[:, 0], d[:, 1], d[:, 2]
    xx, yy, zz = x * x, y * y, z * z
    return np.stack([
        np.full_like(x, 0.28209479177387814), -0.48860251190291987 * y, 0.48860251190291987 * z,
        -0.48860251190291987 * x, 1.0925484305920792 * x * y, -1.0925484305920792 * y * z,
        0.94617469575755997 * zz - 0.31539156525251999, -1.0925484305920792 * x * z,
        0.54627421529603959 * (xx - yy), 0.59004358992664352 * y * (-3 * xx + yy),
        2.8906114426405538 * x * y * z, 0.45704579946446572 * y * (1 - 5 * zz),
        0.3731763325901154 * z * (5 * zz - 3), 0.45704579946446572 * x * (1 - 5 * zz),
        1.4453057213202769 * z * (xx - yy), 0.59004358992664352 * x * (-xx + 3 * yy)], 1)


class CacheRef:
    def __init__(self, levels=16, log2_table=19, base=16, max_res=2048, aabb=(0, 0, 0, 1, 1, 1)):
        self.levels, self.log2T = levels, log2_table
        self.T = 1 << log2_table
        lb = (np.log2(max_res) - np.log2(base)) / (levels - 1) if levels > 1 else 0.0
        self.scale = np.array([np.float32(2.0 ** (l * lb) * base - 1.0) for l in range(levels)], np.float32)
        self.res = np.array([int(np.ceil(np.float64(s))) + 2 for s in self.scale], np.uint64)
        self.dense = self.res ** 3 <= self.T
        a = np.asarray(aabb, np.float32)
        self.amin = a[:3]
        ext = a[3:] - a[:3]
        self.ainv = np.where(ext > 0, np.float32(1.0) / np.where(ext > 0, ext, 1), 0).astype(np.float32)

    def _corners(self, inputs):
        """Per level: (n, 8) table indices and (n, 8) trilinear weights."""
        p = np.asarray(inputs, np.float32)[:, 0:3]
        u = np.clip((p - self.amin) * self.ainv, 0.0, 1.0).astype(np.float32)
        out = []
        mask = np.uint64(self.T - 1)
        for l in range(self.levels):
            pos = (u * self.scale[l] + np.float32(0.5)).astype(np.float32)
            base = np.floor(pos)
            f = (pos - base).astype(np.float64)
            b = base.astype(np.uint64)
            idx = np.zeros((p.shape[0], 8), np.uint64)
            w = np.ones((p.shape[0], 8), np.float64)
            for c in range(8):
                o = np.array([c & 1, (c >> 1) & 1, (c >> 2) & 1], np.uint64)
                q = b + o
                if self.dense[l]:
                    r = self.res[l]
                    ix = (q[:, 0] + q[:, 1] * r + q[:, 2] * r * r) & mask
                else:
                    ix = (q[:, 0] ^ ((q[:, 1] * np.uint64(PRIMES[1])) & np.uint64(0xFFFFFFFF)) ^
                          ((q[:, 2] * np.uint64(PRIMES[2])) & np.uint64(0xFFFFFFFF))) & mask
                idx[:, c] = ix + np.uint64(l) * np.uint64(self.T)
                for k in range(3):
                    w[:, c] *= f[:, k] if o[k] else 1.0 - f[:, k]
            out.append((idx.astype(np.int64), w))
        return out

    def encode(self, inputs, table):
        """(n, 64) input features; table: levels * T * 2 features."""
        x = np.asarray(inputs, np.float64).reshape(-1, 16)
        tab = np.asarray(table, np.float64).reshape(-1, 2)
        n = x.shape[0]
        X = np.zeros((n, 64))
        for l, (idx, w) in enumerate(self._corners(inputs.reshape(-1, 16))):
            X[:, 2 * l] = np.sum(w * tab[idx, 0], 1)
            X[:, 2 * l + 1] = np.sum(w * tab[idx, 1], 1)
        X[:, 32:48] = sh16(x[:, 4:7])
        X[:, 48:51] = (x[:, 8:11] + 1.0) * 0.5
        X[:, 51:54] = x[:, 12:15]
        X[:, 54] = x[:, 3]
        X[:, 55] = 1.0
        return X

    def forward(self, X, weights, bf16=False):
        r = round_bf16 if bf16 else (lambda a: a)
        W = [r(m) for m in split_weights(weights)]
        acts = [r(X)]
        a = acts[0]
        for l in range(HIDDEN):
            a = r(np.maximum(a @ W[l].T, 0.0))
            acts.append(a)
        y = a @ W[HIDDEN].T
        return y, acts, W

    def query(self, inputs, weights, table, bf16=False):
        return self.forward(self.encode(inputs, table), weights, bf16)[0][:, :3]

    def gradients(self, inputs, targets, weights, table, bf16=False, den=None):
        """(loss, dWeights flat, dTable flat) of the mean relative L2 over RGB,
        sum (y - t)^2 / (sg(y)^2 + 0.01) / n: the denominator is a constant
        of the gradient (stop-gradient).  den (n, 3) fixes it explicitly."""
        r = round_bf16 if bf16 else (lambda a: a)
        inputs = np.asarray(inputs, np.float32).reshape(-1, 16)
        X = self.encode(inputs, table)
        y, acts, W = self.forward(X, weights, bf16)
        t = np.asarray(targets, np.float64).reshape(-1, 4)[:, :3]
        n = X.shape[0]
        yy = y[:, :3]
        den = yy * yy + 0.01 if den is None else den
        loss = float(np.sum((yy - t) ** 2 / den) / n)
        gy = np.zeros((n, 16))
        gy[:, :3] = 2.0 * (yy - t) / den / n
        # with bf16, the per-sample gradient rows enter both the weight
        # gradient and the next layer's data gradient rounded to bf16
        gW = [None] * LAYERS
        gW[HIDDEN] = r(gy).T @ acts[HIDDEN]
        g = r(gy) @ W[HIDDEN]
        for l in range(HIDDEN - 1, -1, -1):
            g = g * (acts[l + 1] > 0)
            gW[l] = r(g).T @ acts[l]
            g = r(g) @ W[l]
        gX = g
        gT = np.zeros(len(np.asarray(table).ravel()))
        for l, (idx, w) in enumerate(self._corners(inputs)):
            for f in range(2):
                np.add.at(gT, (idx * 2 + f).ravel(), (w * gX[:, 2 * l + f:2 * l + f + 1]).ravel())
        return loss, join_weights(gW), gT
