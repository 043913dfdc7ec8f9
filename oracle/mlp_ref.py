"""TEST INFRASTRUCTURE ONLY: CPU reference of the learned forcing model.

Restates, in numpy, the per-Lagrangian-point MLP 96 -> 128 -> 128 -> 3 with
tanh-form GELU that the GPU trains and evaluates with BF16 tensor-core
kernels (FP32 accumulation): forward, mean-squared-error loss, backward and
one Adam step.  Where the GPU rounds to BF16 (GEMM inputs: features, weights
of layers 1-2, hidden activations, back-propagated pre-activation
gradients) this reference applies the same round-to-nearest-even, so the
remaining differences come from the FP32 summation order only.

Only tests/ may import this module.
"""
from __future__ import annotations

import numpy as np

N_IN, N_H, N_OUT = 96, 128, 3
GELU_C = np.float32(0.7978845608028654)  # sqrt(2/pi)
GELU_A = np.float32(0.044715)


def bf16(a: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (round to nearest even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    rounding = ((u >> 16) & 1) + 0x7FFF
    r = ((u + rounding) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def gelu(z: np.ndarray) -> np.ndarray:
    z = z.astype(np.float64)
    return 0.5 * z * (1.0 + np.tanh(float(GELU_C) * (z + float(GELU_A) * z ** 3)))


def gelu_grad(z: np.ndarray) -> np.ndarray:
    z = z.astype(np.float64)
    c, a = float(GELU_C), float(GELU_A)
    t = np.tanh(c * (z + a * z ** 3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * c * (1.0 + 3.0 * a * z * z)


# parameter vector layout shared with the GPU (FP32): W1[128][96], b1[128],
# W2[128][128], b2[128], W3[3][128], b3[3]
def split(params: np.ndarray):
    p = np.asarray(params, np.float32)
    o = 0
    out = []
    for shape in ((N_H, N_IN), (N_H,), (N_H, N_H), (N_H,), (N_OUT, N_H), (N_OUT,)):
        n = int(np.prod(shape))
        out.append(p[o:o + n].reshape(shape))
        o += n
    assert o == p.size
    return out


def n_params() -> int:
    return N_H * N_IN + N_H + N_H * N_H + N_H + N_OUT * N_H + N_OUT


def init_params(seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    w1 = rng.standard_normal((N_H, N_IN)) * np.sqrt(2.0 / N_IN)
    w2 = rng.standard_normal((N_H, N_H)) * np.sqrt(2.0 / N_H)
    w3 = rng.standard_normal((N_OUT, N_H)) * np.sqrt(1.0 / N_H) * 0.1
    parts = [w1, np.zeros(N_H), w2, np.zeros(N_H), w3, np.zeros(N_OUT)]
    return np.concatenate([np.ravel(x) for x in parts]).astype(np.float32)


def _ident(a):
    return np.asarray(a, np.float64)


def forward(params: np.ndarray, x: np.ndarray, exact: bool = False) -> dict:
    """exact=True skips every BF16 rounding (float64 throughout), for the
    finite-difference check of the backward formulas."""
    bf16 = _ident if exact else globals()["bf16"]
    w1, b1, w2, b2, w3, b3 = split(params)
    xb = bf16(x)
    z1 = xb.astype(np.float64) @ bf16(w1).T.astype(np.float64) + b1
    h1 = bf16(gelu(z1).astype(np.float32))
    z2 = h1.astype(np.float64) @ bf16(w2).T.astype(np.float64) + b2
    h2 = bf16(gelu(z2).astype(np.float32))
    y = h2.astype(np.float64) @ w3.T.astype(np.float64) + b3
    return {"x": xb, "z1": z1, "h1": h1, "z2": z2, "h2": h2, "y": y}


def f16(a: np.ndarray) -> np.ndarray:
    """Round float32 values to IEEE half precision (round to nearest even), returned as float32."""
    return np.asarray(a, np.float32).astype(np.float16).astype(np.float32)


def forward_f16(params: np.ndarray, x: np.ndarray) -> np.ndarray:
    """The rounding points of the tensor-core inference kernel: BF16 features
    and W1; pre-activations rounded to F16 before the F16 bias is added; the
    epilogue stores f16(2 gelu(x)) and layers 2 and 3 use f16(W2 / 2) and
    W3 / 2 split into an F16 value and its F16 remainder.  The GELU itself is
    evaluated exactly here (the kernel evaluates it in packed half precision)."""
    w1, b1, w2, b2, w3, b3 = split(params)
    z1 = bf16(x).astype(np.float64) @ bf16(w1).T.astype(np.float64)
    g1 = f16(2.0 * gelu(f16(f16(z1) + f16(b1))))
    z2 = g1.astype(np.float64) @ f16(0.5 * w2).T.astype(np.float64)
    g2 = f16(2.0 * gelu(f16(f16(z2) + f16(b2))))
    hi = f16(0.5 * w3)
    lo = f16(0.5 * w3 - hi)
    return g2.astype(np.float64) @ (hi.astype(np.float64) + lo).T + b3


def loss_and_grads(params: np.ndarray, x: np.ndarray, t: np.ndarray, exact: bool = False):
    """MSE loss mean over the batch of the squared error summed over outputs."""
    bf16 = _ident if exact else globals()["bf16"]
    w1, b1, w2, b2, w3, b3 = split(params)
    f = forward(params, x, exact)
    nb = x.shape[0]
    diff = f["y"] - t
    loss = float(np.sum(diff * diff) / nb)
    dy = 2.0 * diff / nb
    gw3 = dy.T @ f["h2"].astype(np.float64)
    gb3 = dy.sum(0)
    dh2 = dy @ w3.astype(np.float64)
    dz2 = bf16((dh2 * gelu_grad(f["z2"])).astype(np.float32)).astype(np.float64)
    gw2 = dz2.T @ f["h1"].astype(np.float64)
    gb2 = dz2.sum(0)
    dh1 = dz2 @ bf16(w2).astype(np.float64)
    dz1 = bf16((dh1 * gelu_grad(f["z1"])).astype(np.float32)).astype(np.float64)
    gw1 = dz1.T @ f["x"].astype(np.float64)
    gb1 = dz1.sum(0)
    g = np.concatenate([np.ravel(a) for a in (gw1, gb1, gw2, gb2, gw3, gb3)])
    return loss, g


def adam_step(params, grad, m, v, step, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad * grad
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return params - lr * mh / (np.sqrt(vh) + eps), m, v
