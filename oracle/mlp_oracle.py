"""CPU restatement of the warm-start network (TEST INFRASTRUCTURE ONLY: the
checker of the GPU forward/backward kernels in cufim-nvlink_gb300/csrc/
fim_mlp.cu; the product never imports it).

The network has no counterpart in the reference.  This file repeats the GPU's
arithmetic with NumPy: BF16 operands (round to nearest even) for the three
hidden-layer products with FP32 accumulation, BF16 storage of the hidden
activations and of the back-propagated deltas, FP32 everywhere else.  Only
the FP32 summation order differs from the tensor-core tiles, so results
agree to FP32 rounding (and to a BF16 step where such a rounding flips a
stored activation).

Parameter vector (as fim_mlp_get_params): W1 [64 x 128], W2 [128 x 128],
W3 [128 x 128] ([in][out], row-major), then b1, b2, b3 (128 each), w4 (128),
b4 (1).
"""
import numpy as np

IN, H = 64, 128
OW1, OW2, OW3 = 0, IN * H, IN * H + H * H
OB1 = OW3 + H * H
OB2, OB3, OW4, OB4 = OB1 + H, OB1 + 2 * H, OB1 + 3 * H, OB1 + 4 * H
NPARAMS = OB4 + 1


def bf16(x):
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    b = x.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


def bf16_from_bits(u16):
    """float32 values of raw bfloat16 bit patterns (uint16)."""
    return (np.asarray(u16, dtype=np.uint32) << 16).view(np.float32)


def unpack(p, dtype=np.float32):
    p = np.asarray(p, dtype=dtype)
    return dict(W1=p[OW1:OW2].reshape(IN, H), W2=p[OW2:OW3].reshape(H, H), W3=p[OW3:OB1].reshape(H, H),
                b1=p[OB1:OB2], b2=p[OB2:OB3], b3=p[OB3:OW4], w4=p[OW4:OB4], b4=p[OB4:OB4 + 1])


def forward(p, X, exact=False):
    """Hidden activations (BF16 values) and outputs of feature rows X (BF16
    values).  exact=True: the same network in FP64 without BF16 roundings
    (the reference for finite differences)."""
    r, ft = (lambda a: a, np.float64) if exact else (bf16, np.float32)
    q = unpack(p, ft)
    X = X.astype(ft)
    H1 = r(np.maximum(X @ r(q["W1"]) + q["b1"], 0))
    H2 = r(np.maximum(H1 @ r(q["W2"]) + q["b2"], 0))
    H3 = r(np.maximum(H2 @ r(q["W3"]) + q["b3"], 0))
    y = H3 @ q["w4"] + q["b4"][0]
    return H1, H2, H3, y.astype(ft)


def loss_and_gradients(p, X, t, exact=False):
    """Mean squared error of the outputs against t and its gradient vector."""
    r, ft = (lambda a: a, np.float64) if exact else (bf16, np.float32)
    q = unpack(p, ft)
    n = X.shape[0]
    X = X.astype(ft)
    H1, H2, H3, y = forward(p, X, exact)
    e = y - t.astype(ft)
    loss = float(np.sum(e * e) / n)
    dy = (2.0 * e / n).astype(ft)
    g = np.zeros(NPARAMS, dtype=ft)
    g[OW4:OB4] = H3.T @ dy
    g[OB4] = dy.sum()
    dZ3 = r(np.where(H3 > 0, dy[:, None] * q["w4"][None, :], 0).astype(ft))
    g[OW3:OB1] = (H2.T @ dZ3).ravel()
    g[OB3:OW4] = dZ3.sum(axis=0)
    dZ2 = r(np.where(H2 > 0, dZ3 @ r(q["W3"]).T, 0).astype(ft))
    g[OW2:OW3] = (H1.T @ dZ2).ravel()
    g[OB2:OB3] = dZ2.sum(axis=0)
    dZ1 = r(np.where(H1 > 0, dZ2 @ r(q["W2"]).T, 0).astype(ft))
    g[OW1:OW2] = (X.T @ dZ1).ravel()
    g[OB1:OB2] = dZ1.sum(axis=0)
    return loss, g


BLOCKS = {"W1": (OW1, OW2), "W2": (OW2, OW3), "W3": (OW3, OB1), "b1": (OB1, OB2), "b2": (OB2, OB3),
          "b3": (OB3, OW4), "w4": (OW4, OB4), "b4": (OB4, OB4 + 1)}
