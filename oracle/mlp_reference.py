"""CPU reference of the learned doublet filter's network (numpy).

TEST INFRASTRUCTURE ONLY: the oracle of the GPU forward and backward
kernels of the network (traccc_gb300/csrc/seedgb_learned.cu,
seedgb_mlp.cuh).  The product never imports it.

The network has no counterpart in the reference; this file restates the
numerics the GPU kernels define, in exact arithmetic where the GPU
accumulates in fp32 (sums in float64, rounded once to fp32), so the GPU
results differ from it only by fp32 accumulation rounding:

forward  x  = bf16((f - mu) * isd)                      (fp32 product, then bf16)
         z1 = b1 + x W1b,  h1 = bf16(relu(z1))          (W1b = bf16(W1))
         z2 = b2 + h1 W2b, h2 = bf16(relu(z2))
         z3 = b3 + h2 w3b                               (the logit)
backward of L = mean(-(p y log s(z3) + (1 - y) log(1 - s(z3)))):
         g3  = (p y (s - 1) + (1 - y) s) / n            (fp32)
         db3 = sum g3,  dW3 = h2^T bf16(g3)
         dz2 = g3 w3b [z2 > 0],  db2 = sum dz2,  dW2 = h1^T bf16(dz2)
         dz1 = (bf16(dz2) W2b^T) [z1 > 0],  db1 = sum dz1,  dW1 = x^T bf16(dz1)
Parameter block (fp32): w1[8][32], b1[32], w2[32][32], b2[32], w3[32], b3.
"""
import numpy as np

IN, H = 8, 32
OFF_W1 = 0
OFF_B1 = OFF_W1 + IN * H
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H
N_PARAMS = OFF_B3 + 1


def bf16(x):
    """Round float32 values to bf16 (nearest even), as float32."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    nan = ((u & 0x7f800000) == 0x7f800000) & ((u & 0x007fffff) != 0)
    r = (u + 0x7fff + ((u >> 16) & 1)) & 0xffff0000
    r = np.where(nan, (u | 0x00400000) & 0xffff0000, r)
    return r.astype(np.uint32).view(np.float32).reshape(np.shape(x))


def unpack(p):
    p = np.asarray(p, np.float32)
    return (p[OFF_W1:OFF_B1].reshape(IN, H), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(H, H),
            p[OFF_B2:OFF_W3], p[OFF_W3:OFF_B3], p[OFF_B3])


def _f32(a):
    return np.asarray(a, np.float64).astype(np.float32)


def forward(params, norm, feat, exact=False):
    """Logits and the intermediate values (dict).  exact=True skips every
    rounding (float64 throughout), for finite-difference checks."""
    if exact:
        return _forward_exact(params, norm, feat)
    w1, b1, w2, b2, w3, b3 = unpack(params)
    norm = np.asarray(norm, np.float32)
    mu, isd = norm[:IN], norm[IN:]
    feat = np.asarray(feat, np.float32)
    x = bf16((feat - mu) * isd)
    w1b, w2b, w3b = bf16(w1), bf16(w2), bf16(w3)
    z1 = _f32(b1.astype(np.float64) + x.astype(np.float64) @ w1b.astype(np.float64))
    h1 = bf16(np.maximum(z1, 0))
    z2 = _f32(b2.astype(np.float64) + h1.astype(np.float64) @ w2b.astype(np.float64))
    h2 = bf16(np.maximum(z2, 0))
    z3 = _f32(np.float64(b3) + h2.astype(np.float64) @ w3b.astype(np.float64))
    return z3, dict(x=x, z1=z1, h1=h1, z2=z2, h2=h2, w2b=w2b, w3b=w3b)


def _forward_exact(params, norm, feat):
    p = np.asarray(params, np.float64)
    w1, b1 = p[OFF_W1:OFF_B1].reshape(IN, H), p[OFF_B1:OFF_W2]
    w2, b2 = p[OFF_W2:OFF_B2].reshape(H, H), p[OFF_B2:OFF_W3]
    w3, b3 = p[OFF_W3:OFF_B3], p[OFF_B3]
    norm = np.asarray(norm, np.float64)
    x = (np.asarray(feat, np.float64) - norm[:IN]) * norm[IN:]
    z1 = b1 + x @ w1
    h1 = np.maximum(z1, 0)
    z2 = b2 + h1 @ w2
    h2 = np.maximum(z2, 0)
    z3 = b3 + h2 @ w3
    return z3, dict(x=x, z1=z1, h1=h1, z2=z2, h2=h2, w2b=w2, w3b=w3)


def loss_and_grad(params, norm, feat, label, pos_weight, exact=False):
    """(loss, gradient block) of the mean weighted logistic loss.  exact=True:
    float64 throughout without any rounding (plain backpropagation)."""
    ident = lambda a: np.asarray(a, np.float64)
    rnd, f32 = (ident, ident) if exact else (bf16, _f32)
    ft = np.float64 if exact else np.float32
    z, c = forward(params, norm, feat, exact)
    y = np.asarray(label, ft)
    n = max(1, len(y))
    p = ft(pos_weight)
    z64 = z.astype(np.float64)
    s = 1.0 / (1.0 + np.exp(-z64))
    sp = lambda v: np.maximum(v, 0) + np.log1p(np.exp(-np.abs(v)))
    loss = float(np.sum(p * y * sp(-z64) + (1 - y) * sp(z64)) / n)
    g3 = f32((p * y * (s - 1) + (1 - y) * s) / n)
    dz2 = np.where(c["z2"] > 0, g3[:, None] * c["w3b"][None, :], 0).astype(ft)
    dz2b = rnd(dz2)
    dz1 = np.where(c["z1"] > 0, f32(dz2b.astype(np.float64) @ c["w2b"].T.astype(np.float64)),
                   0).astype(ft)
    dz1b = rnd(dz1)
    g = np.zeros(N_PARAMS, np.float64)
    g[OFF_W1:OFF_B1] = (c["x"].astype(np.float64).T @ dz1b.astype(np.float64)).reshape(-1)
    g[OFF_B1:OFF_W2] = dz1.astype(np.float64).sum(0)
    g[OFF_W2:OFF_B2] = (c["h1"].astype(np.float64).T @ dz2b.astype(np.float64)).reshape(-1)
    g[OFF_B2:OFF_W3] = dz2.astype(np.float64).sum(0)
    g[OFF_W3:OFF_B3] = c["h2"].astype(np.float64).T @ rnd(g3).astype(np.float64)
    g[OFF_B3] = g3.astype(np.float64).sum()
    return loss, g
