"""Test infrastructure (the oracle): a numpy restatement of the learned scan
order's scorer and features, to check the CUDA kernels against.

The scorer has no counterpart in the reference; this file states the same
mathematics as gpusharesat_gb300/csrc/order.cu in plain float64 numpy:

  z1 = W1 x + b1, h1 = relu(z1)          W1 [64][12]
  z2 = W2 h1 + b2, h2 = relu(z2)         W2 [64][64]
  z  = w3 . h2 + b3                      the logit
  loss = mean over rows of max(z,0) - z*y + log(1 + exp(-|z|))

with the flat weight layout W1, b1, W2, b2, w3, b3 (5057 floats).
Inference on the GPU rounds x, W1, h1 and W2 to BF16 (round to nearest
even) and accumulates in FP32; `infer_bf16` emulates that.
"""
import numpy as np

F, H = 12, 64
P = H * F + H + H * H + H + H + 1
O_W1, O_B1 = 0, H * F
O_W2 = O_B1 + H
O_B2 = O_W2 + H * H
O_W3 = O_B2 + H
O_B3 = O_W3 + H


def unpack(w):
    w = np.asarray(w, dtype=np.float64)
    return (w[O_W1:O_B1].reshape(H, F), w[O_B1:O_W2], w[O_W2:O_B2].reshape(H, H), w[O_B2:O_W3], w[O_W3:O_B3],
            w[O_B3])


def forward(w, x):
    W1, b1, W2, b2, w3, b3 = unpack(w)
    x = np.asarray(x, dtype=np.float64)
    z1 = x @ W1.T + b1
    h1 = np.maximum(z1, 0)
    z2 = h1 @ W2.T + b2
    h2 = np.maximum(z2, 0)
    return h2 @ w3 + b3, (x, h1, h2)


def loss_and_grad(w, x, y):
    """Mean logistic loss and its gradient (flat, float64)."""
    W1, b1, W2, b2, w3, b3 = unpack(w)
    y = np.asarray(y, dtype=np.float64)
    z, (x, h1, h2) = forward(w, x)
    B = x.shape[0]
    loss = np.mean(np.maximum(z, 0) - z * y + np.log1p(np.exp(-np.abs(z))))
    dz = (1.0 / (1.0 + np.exp(-z)) - y) / B
    d2 = np.outer(dz, w3) * (h2 > 0)
    d1 = (d2 @ W2) * (h1 > 0)
    g = np.zeros(P)
    g[O_W1:O_B1] = (d1.T @ x).ravel()
    g[O_B1:O_W2] = d1.sum(0)
    g[O_W2:O_B2] = (d2.T @ h1).ravel()
    g[O_B2:O_W3] = d2.sum(0)
    g[O_W3:O_B3] = dz @ h2
    g[O_B3] = dz.sum()
    return loss, g


def adam_step(w, g, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (t = step number from 1); returns new (w, m, v)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    c1, c2 = 1 - b1 ** t, 1 - b2 ** t
    return w - lr * (m / c1) / (np.sqrt(v / c2) + eps), m, v


def bf16(a):
    """Rounds float32 values to the nearest BF16 (ties to even), as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r.astype(np.uint32)).view(np.float32)


def infer_bf16(w, x):
    """Logits as the tensor-core inference computes them."""
    W1, b1, W2, b2, w3, b3 = unpack(np.asarray(w, dtype=np.float32))
    xb = bf16(np.asarray(x, dtype=np.float32)).astype(np.float64)
    z1 = xb @ bf16(W1).astype(np.float64).T + b1
    h1 = bf16(np.maximum(z1, 0).astype(np.float32)).astype(np.float64)
    z2 = h1 @ bf16(W2).astype(np.float64).T + b2
    h2 = np.maximum(z2, 0)
    return h2 @ w3 + b3


def features(length, lbd, age, hist_bytes, total, since_last):
    """The 12 features of one clause (order.cu clause_features).
    hist_bytes[k] = slot reports in pass now-1-k (k = 0..7), saturated at
    255; since_last = passes since the last report, -1 if never."""
    if lbd == 0:
        lbd = length
    b = [int(v) for v in hist_bytes]
    s1, s2 = b[0], b[0] + b[1]
    s4 = s2 + b[2] + b[3]
    s8 = s4 + b[4] + b[5] + b[6] + b[7]
    age = max(age, 0)
    f32 = np.float32
    x = np.zeros(F, dtype=np.float32)
    x[0] = f32(length) / f32(64)
    x[1] = f32(lbd) / f32(64)
    x[2] = f32(lbd) / f32(max(length, 1))
    x[3] = np.log2(f32(1) + f32(age)) / f32(16)
    x[4] = f32(min(s1, 8)) / f32(8)
    x[5] = f32(min(s2, 16)) / f32(16)
    x[6] = f32(min(s4, 32)) / f32(32)
    x[7] = f32(min(s8, 64)) / f32(64)
    x[8] = f32(sum(v != 0 for v in b)) / f32(8)
    x[9] = f32(1) if since_last < 0 else min(np.log2(f32(1) + f32(since_last)) / f32(16), f32(1))
    x[10] = np.log2(f32(1) + f32(total)) / f32(16)
    x[11] = min(f32(total) / f32(max(age, 1)), f32(1))
    return x


class History:
    """Per-clause report history as the order keeps it: after each ordered
    pass p, `record(p, counts)` with the slot reports of each clause id."""

    def __init__(self):
        self.birth, self.hist, self.total, self.last = {}, {}, {}, {}

    def born(self, ids, p):
        for i in ids:
            self.birth.setdefault(int(i), p)
            self.hist.setdefault(int(i), [0] * 8)
            self.total.setdefault(int(i), 0)
            self.last.setdefault(int(i), -1)

    def record(self, p, counts):
        """counts: {id: slot reports in pass p} (ids not given: 0)."""
        for i in self.hist:
            c = int(counts.get(i, 0))
            self.hist[i] = [min(c, 255)] + self.hist[i][:7]
            self.total[i] += c
            if c:
                self.last[i] = p

    def features(self, i, length, lbd, now):
        last = self.last[i]
        return features(length, lbd, now - self.birth[i], self.hist[i], self.total[i],
                        -1 if last < 0 else now - last)
