"""mlp_oracle.py -- CPU restatement of the learned-closure MLP (forward, loss,
backward, Adam step) used to check the GPU kernels' gradients and updates.

TEST INFRASTRUCTURE ONLY: only tests/, __graft_entry__.smoke() and bench.py's
CPU baseline may import it; the product never does.

The network has no counterpart in the reference.  Architecture and parameter
layout follow include/hyb_dvm.h (hyb_mlp_*): 8 -> 64 -> 64 -> 64 -> 4, tanh
hidden layers, linear output; FP32 layout W1[64][8] b1[64] W2[64][64] b2[64]
W3[64][64] b3[64] W4[4][64] b4[4]; loss = mean over samples and outputs of
the squared error of the normalised outputs.

quantize=True reproduces the GPU's number formats: every matrix-product
operand (normalised inputs, weights, hidden activations, output and hidden
gradients) is rounded to BF16 (round to nearest even) and the products are
accumulated exactly (float64 here, FP32 on the tensor cores); biases,
activations and bias gradients stay in FP32.  quantize=False is the plain
float64 network (for finite-difference checks of this restatement).
"""
import numpy as np

IN, H, OUT = 8, 64, 4
SHAPES = [("W1", (H, IN)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)),
          ("W3", (H, H)), ("b3", (H,)), ("W4", (OUT, H)), ("b4", (OUT,))]
NPARAM = sum(int(np.prod(s)) for _, s in SHAPES)   # 9156


def unpack(w):
    out, o = {}, 0
    for name, shp in SHAPES:
        n = int(np.prod(shp))
        out[name] = np.asarray(w[o:o + n], dtype=np.float64).reshape(shp)
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).ravel() for name, _ in SHAPES])


def bf16(a):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def forward(w, x, norm, quantize=True):
    """Returns the normalised outputs and the cache of the backward pass."""
    p = unpack(w)
    q = bf16 if quantize else (lambda a: np.asarray(a, dtype=np.float64))
    in_mu, in_sd = np.asarray(norm[0], np.float32), np.asarray(norm[1], np.float32)
    if quantize:
        xn = bf16((np.asarray(x, np.float32) - in_mu) * (np.float32(1.0) / in_sd))
    else:
        xn = (np.asarray(x, np.float64) - in_mu) / in_sd
    W = {k: q(p[k]) for k in ("W1", "W2", "W3", "W4")}
    z1 = xn @ W["W1"].T + p["b1"]
    h1 = q(np.tanh(z1))
    z2 = h1 @ W["W2"].T + p["b2"]
    h2 = q(np.tanh(z2))
    z3 = h2 @ W["W3"].T + p["b3"]
    h3 = q(np.tanh(z3))
    y = h3 @ W["W4"].T + p["b4"]
    return y, dict(xn=xn, h1=h1, h2=h2, h3=h3, W=W, q=q)


def loss_and_grad(w, x, y_true, norm, quantize=True):
    """Mean squared error of the normalised outputs and its gradient."""
    out_mu, out_sd = np.asarray(norm[2], np.float32), np.asarray(norm[3], np.float32)
    y, c = forward(w, x, norm, quantize)
    q, W = c["q"], c["W"]
    tn = (np.asarray(y_true, np.float32) - out_mu) / out_sd
    d = y - tn
    n = x.shape[0]
    loss = float(np.sum(d * d) / (n * OUT))
    dy = 2.0 * d / (n * OUT)
    g = {}
    dz4 = q(dy)
    g["W4"] = dz4.T @ c["h3"]
    g["b4"] = dy.sum(0)
    dz3 = (dz4 @ W["W4"]) * (1.0 - c["h3"] ** 2)
    g["b3"] = dz3.sum(0)
    dz3q = q(dz3)
    g["W3"] = dz3q.T @ c["h2"]
    dz2 = (dz3q @ W["W3"]) * (1.0 - c["h2"] ** 2)
    g["b2"] = dz2.sum(0)
    dz2q = q(dz2)
    g["W2"] = dz2q.T @ c["h1"]
    dz1 = (dz2q @ W["W2"]) * (1.0 - c["h1"] ** 2)
    g["b1"] = dz1.sum(0)
    g["W1"] = q(dz1).T @ c["xn"]
    return loss, pack(g)


def adam_step(w, m1, m2, g, t, lr):
    """One Adam step in FP32, as k_mlp_adam (csrc/hyb_mlp.cu) takes it:
    beta1 0.9, beta2 0.999, eps 1e-8, bias corrections 1 - beta^t of the
    step count t (1 for the first step).  Returns the new (w, m1, m2)."""
    f = np.float32
    w, m1, m2, g = (np.asarray(a, dtype=np.float32) for a in (w, m1, m2, g))
    c1 = f(1.0) - f(0.9) ** f(t)
    c2 = f(1.0) - f(0.999) ** f(t)
    a = f(0.9) * m1 + f(0.1) * g
    b = f(0.999) * m2 + f(0.001) * g * g
    w = w - f(lr) * (a / c1) / (np.sqrt(b / c2) + f(1e-8))
    return w.astype(np.float32), a, b


def glorot(seed):
    rng = np.random.default_rng(seed)
    d = {}
    for name, shp in SHAPES:
        if name.startswith("W"):
            a = np.sqrt(6.0 / (shp[0] + shp[1]))
            d[name] = rng.uniform(-a, a, size=shp)
        else:
            d[name] = np.zeros(shp)
    return pack(d).astype(np.float32).astype(np.float64)
