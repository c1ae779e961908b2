"""CPU reference of the collision-surrogate MLP -- TEST INFRASTRUCTURE ONLY.

Forward and backward of in -> 256 -> 256 -> 256 -> 256 -> 1 (SiLU, logit out,
BCE-with-logits loss) in FP64 numpy, with the BF16 rounding applied where the
device kernels round (inputs, weights and hidden activations as GEMM operands;
the pre-activations and accumulations stay wide).  The parameter vector uses
the device layout: W0[256][in], b0, W1, b1, W2, b2, W3, b3, w4[256], b4.
"""
import numpy as np

W = 256


def bf16(x):
    """Round to bfloat16 (round to nearest even) and return as float64."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p, d_in):
    o = 0
    out = {}

    def take(name, n, shape):
        nonlocal o
        out[name] = np.asarray(p[o:o + n], dtype=np.float64).reshape(shape)
        o += n
    take("W0", W * d_in, (W, d_in))
    take("b0", W, (W,))
    for l in (1, 2, 3):
        take("W%d" % l, W * W, (W, W))
        take("b%d" % l, W, (W,))
    take("w4", W, (W,))
    take("b4", 1, (1,))
    assert o == len(p)
    return out


def pack(g, d_in):
    parts = [g["W0"].ravel(), g["b0"]]
    for l in (1, 2, 3):
        parts += [g["W%d" % l].ravel(), g["b%d" % l]]
    parts += [g["w4"], g["b4"]]
    return np.concatenate(parts)


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, x, d_in):
    P = unpack(p, d_in)
    X = bf16(x)
    zs, hs = [], []
    z = X @ bf16(P["W0"]).T + P["b0"]
    zs.append(z)
    hs.append(bf16(silu(z)))
    for l in (1, 2, 3):
        z = hs[-1] @ bf16(P["W%d" % l]).T + P["b%d" % l]
        zs.append(z)
        hs.append(bf16(silu(z)))
    zout = hs[-1] @ bf16(P["w4"]) + P["b4"][0]
    return zout, (X, zs, hs, P)


def loss_and_grad(p, x, y, d_in):
    zout, (X, zs, hs, P) = forward(p, x, d_in)
    n = len(y)
    t = y.astype(np.float64)
    loss = np.mean(np.maximum(zout, 0) - zout * t + np.log1p(np.exp(-np.abs(zout))))
    dz = (1.0 / (1.0 + np.exp(-zout)) - t) / n
    g = {"w4": hs[3].T @ dz, "b4": np.array([dz.sum()])}
    dZ = bf16(np.outer(dz, bf16(P["w4"])) * dsilu(zs[3]))
    for l in (3, 2, 1):
        g["W%d" % l] = dZ.T @ hs[l - 1]
        g["b%d" % l] = dZ.sum(0)
        dZ = bf16((dZ @ bf16(P["W%d" % l])) * dsilu(zs[l - 1]))
    g["W0"] = dZ.T @ X
    g["b0"] = dZ.sum(0)
    return loss, pack(g, d_in), zout
