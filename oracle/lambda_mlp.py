"""FP64 restatement of the learned lambda proposal (test infrastructure only).

The proposal is not part of the reference: it is the network that the GPU
library trains and runs (include/pgsvt.h, "Learned lambda proposal";
pgure-svt_gb300/csrc/lambda.cu).  This module is its CPU checker: the
features of a window from its singular values, the forward pass, the
gradient of the training loss by hand-written backpropagation (itself checked
against central finite differences in tests/test_lambda_oracle.py) and one
AdamW step.  Weights enter at their bf16 values (round to nearest even), as
on the GPU; everything else is float64.  Nothing in the product imports it.
"""
import numpy as np
from scipy.special import erf

NF, H = 67, 128
NSAMPLES = 4096
OFF_MEAN, OFF_SCALE, OFF_W1 = 0, NF, 2 * NF
OFF_B1 = OFF_W1 + H * NF
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H * H
OFF_W4 = OFF_B3 + H
OFF_B4 = OFF_W4 + H
OFF_YMEAN = OFF_B4 + 1
OFF_YSCALE = OFF_YMEAN + 1
TOTAL = OFF_YSCALE + 1
NPARAM = OFF_YMEAN - OFF_W1
WEIGHT_RANGES = ((OFF_W1, OFF_B1), (OFF_W2, OFF_B2), (OFF_W3, OFF_B3), (OFF_W4, OFF_B4))


def bf16(x):
    """float32 -> nearest bf16 value (ties to even), returned as float64."""
    b = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def lowbias32(x):
    """The lowbias32 integer hash (C. Wellons), on uint32 values."""
    x = np.asarray(x, np.uint64) & 0xFFFFFFFF
    x ^= x >> 16
    x = (x * 0x7FEB352D) & 0xFFFFFFFF
    x ^= x >> 15
    x = (x * 0x846CA68B) & 0xFFFFFFFF
    x ^= x >> 16
    return x


def sample_indices(npatch):
    """Sorted-order indices of the kept patches the features use."""
    ns = min(npatch, NSAMPLES)
    i = np.arange(ns, dtype=np.uint64)
    h = lowbias32(i ^ np.uint64(0x5EED1234))
    return ((i * np.uint64(npatch) + ((h * np.uint64(npatch)) >> np.uint64(32))) //
            np.uint64(ns)).astype(np.int64)


def features(S, alpha, mu, sigma):
    """Features of one window: S is (npatch, nwin) singular values of its kept
    patches in the reference's sorted order; alpha/mu/sigma as the risk uses
    them."""
    S = np.asarray(S, np.float64)
    sv = S[sample_indices(S.shape[0])].ravel()
    x = np.full(sv.shape, -np.inf)
    pos = (sv > 0) & np.isfinite(sv)
    x[pos] = (np.log10(sv[pos]) + 4.0) * (64.0 / 6.0)
    b = np.clip(np.floor(np.where(np.isfinite(x), x, 0.0)), 0, 63).astype(np.int64)
    b[x >= 63.0] = 63
    hist = np.bincount(b, minlength=64).astype(np.float64) / sv.size
    f = np.empty(NF)
    f[:3] = np.arcsinh(np.array([alpha, mu, sigma]) * 1000.0) / 8.0
    f[3:] = hist
    return f


def _gelu(z):
    return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))


def _gelu_grad(z):
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)


def unpack(model, exact=False):
    """Model pieces; weights at their bf16 values unless `exact` (then every
    value is taken as given, in float64)."""
    if exact:
        f = np.asarray(model, np.float64)
        w = f
    else:
        m = np.asarray(model, np.float32)
        w = bf16(m)
        f = m.astype(np.float64)
    return dict(mean=f[OFF_MEAN:OFF_SCALE], scale=f[OFF_SCALE:OFF_W1],
                W1=w[OFF_W1:OFF_B1].reshape(H, NF), b1=f[OFF_B1:OFF_W2],
                W2=w[OFF_W2:OFF_B2].reshape(H, H), b2=f[OFF_B2:OFF_W3],
                W3=w[OFF_W3:OFF_B3].reshape(H, H), b3=f[OFF_B3:OFF_W4],
                W4=w[OFF_W4:OFF_B4], b4=f[OFF_B4], ymean=f[OFF_YMEAN], yscale=f[OFF_YSCALE])


def forward(model, feats, exact=False):
    """Network outputs o (before the y map) and the activations."""
    p = unpack(model, exact)
    x0 = (np.asarray(feats, np.float64) - p["mean"]) * p["scale"]
    z1 = x0 @ p["W1"].T + p["b1"]
    a1 = _gelu(z1)
    z2 = a1 @ p["W2"].T + p["b2"]
    a2 = _gelu(z2)
    z3 = a2 @ p["W3"].T + p["b3"]
    a3 = _gelu(z3)
    o = a3 @ p["W4"] + p["b4"]
    return o, (p, x0, z1, a1, z2, a2, z3, a3)


def predict(model, feats):
    """y = log10(lambda/upper) per feature row."""
    o, (p, *_) = forward(model, feats)
    return o * p["yscale"] + p["ymean"]


def loss_and_grad(model, feats, targets, exact=False):
    """L = mean((o - t)^2), t = (target - ymean)/yscale; gradient over the
    NPARAM trainable floats (bf16 weights treated as the parameters)."""
    o, (p, x0, z1, a1, z2, a2, z3, a3) = forward(model, feats, exact)
    t = (np.asarray(targets, np.float64) - p["ymean"]) / p["yscale"]
    n = o.shape[0]
    e = o - t
    L = float(np.mean(e * e))
    dO = 2.0 * e / n
    g = np.zeros(NPARAM)
    g[OFF_W4 - OFF_W1:OFF_B4 - OFF_W1] = dO @ a3
    g[OFF_B4 - OFF_W1] = dO.sum()
    dz3 = np.outer(dO, p["W4"]) * _gelu_grad(z3)
    g[OFF_W3 - OFF_W1:OFF_B3 - OFF_W1] = (dz3.T @ a2).ravel()
    g[OFF_B3 - OFF_W1:OFF_W4 - OFF_W1] = dz3.sum(0)
    dz2 = (dz3 @ p["W3"]) * _gelu_grad(z2)
    g[OFF_W2 - OFF_W1:OFF_B2 - OFF_W1] = (dz2.T @ a1).ravel()
    g[OFF_B2 - OFF_W1:OFF_W3 - OFF_W1] = dz2.sum(0)
    dz1 = (dz2 @ p["W2"]) * _gelu_grad(z1)
    g[0:OFF_B1 - OFF_W1] = (dz1.T @ x0).ravel()
    g[OFF_B1 - OFF_W1:OFF_W2 - OFF_W1] = dz1.sum(0)
    return L, g


def is_weight_mask():
    mask = np.zeros(NPARAM, bool)
    for a, b in WEIGHT_RANGES:
        mask[a - OFF_W1:b - OFF_W1] = True
    return mask


def adamw_step(model, m1, m2, grad, t, lr, wd, b1=0.9, b2=0.999, eps=1e-8):
    """One AdamW step (step count t >= 1, decay on weights only); returns the
    new (model, m1, m2)."""
    w = np.asarray(model, np.float64).copy()
    m1 = b1 * m1 + (1 - b1) * grad
    m2 = b2 * m2 + (1 - b2) * grad * grad
    p = w[OFF_W1:OFF_YMEAN]
    p = p - lr * wd * p * is_weight_mask()
    p = p - lr * (m1 / (1 - b1 ** t)) / (np.sqrt(m2 / (1 - b2 ** t)) + eps)
    w[OFF_W1:OFF_YMEAN] = p
    return w, m1, m2
