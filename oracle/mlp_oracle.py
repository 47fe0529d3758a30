"""CPU restatement of the learned cooling step's network (numpy, float64).

TEST INFRASTRUCTURE ONLY: the checker of the GPU forward and backward
kernels.  It follows the kernels' rounding points exactly -- the inputs,
W1, W2, the first hidden layer and dz2 are rounded to bfloat16 (round to
nearest even) where the kernels hand them to the tensor cores, w3 is
rounded to bfloat16 -- and computes everything else in float64, so the
only differences left are the kernels' FP32 accumulation order and
rounding.

Network: u = features (4) -> z1 = W1 u + b1 -> h1 = silu(z1)
                          -> z2 = W2 bf16(h1) + b2 -> h2 = silu(z2)
                          -> y = bf16(w3) . h2 + b3
Loss: mean over rows of (y - y*)^2, y* = (log10 T_new - log10 T) / 4.
Parameter vector: W1[64][4], b1[64], W2[64][64], b2[64], w3[64], b3.
"""
import numpy as np

H = 64
N_PARAMS = 4545


def bf16(x):
    """Round float64 values to bfloat16 (through float32, nearest even)."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return dict(W1=p[0:256].reshape(64, 4), b1=p[256:320], W2=p[320:4416].reshape(64, 64),
                b2=p[4416:4480], w3=p[4480:4544], b3=p[4544])


def pack(g):
    return np.concatenate([g["W1"].ravel(), g["b1"], g["W2"].ravel(), g["b2"], g["w3"],
                           [g["b3"]]])


def features(tuples, lo, hi):
    """u = 2 (log10 v - lo) / (hi - lo) - 1 per column, as float32 values."""
    lt = np.log10(np.asarray(tuples, dtype=np.float64))
    lo, hi = np.asarray(lo, dtype=np.float64), np.asarray(hi, dtype=np.float64)
    return ((lt - lo) * (2.0 / (hi - lo)) - 1.0).astype(np.float32).astype(np.float64)


def targets(tuples, t_new):
    t = np.asarray(tuples, dtype=np.float64)
    return ((np.log10(t_new) - np.log10(t[:, 1])) * 0.25).astype(np.float32).astype(np.float64)


def _sig(z):
    return 1.0 / (1.0 + np.exp(-z))


def forward(p, u, exact=False):
    """Network output; exact=True skips every bfloat16 rounding (the plain
    float64 network, used to pin the gradient formulas by finite
    differences)."""
    r = (lambda a: np.asarray(a, dtype=np.float64)) if exact else bf16
    q = unpack(p)
    xb = r(u)
    z1 = xb @ r(q["W1"]).T + q["b1"]
    h1b = r(z1 * _sig(z1))
    z2 = h1b @ r(q["W2"]).T + q["b2"]
    h2 = z2 * _sig(z2)
    y = h2 @ r(q["w3"]) + q["b3"]
    return y, dict(xb=xb, z1=z1, h1b=h1b, z2=z2, h2=h2)


def loss_grad(p, u, t, exact=False):
    """Mean squared error and its gradient (parameter layout)."""
    bf = (lambda a: np.asarray(a, dtype=np.float64)) if exact else bf16
    q = unpack(p)
    y, c = forward(p, u, exact)
    B = len(u)
    e = y - t
    dy = 2.0 * e / B
    s2 = _sig(c["z2"])
    dz2 = dy[:, None] * bf(q["w3"])[None, :] * (s2 * (1.0 + c["z2"] * (1.0 - s2)))
    dz2b = bf(dz2)
    dh1 = dz2b @ bf(q["W2"])
    s1 = _sig(c["z1"])
    dz1 = dh1 * (s1 * (1.0 + c["z1"] * (1.0 - s1)))
    g = dict(W1=dz1.T @ c["xb"], b1=dz1.sum(0), W2=dz2b.T @ c["h1b"], b2=dz2.sum(0),
             w3=c["h2"].T @ dy, b3=dy.sum())
    return float(np.mean(e * e)), pack(g)
