"""The CPU reference of the learned-forcing network (oracle/mlp_ref.py):
backward formulas against finite differences, BF16 rounding against torch."""
import numpy as np
import torch

from oracle import mlp_ref


def test_bf16_rounding_matches_torch():
    rng = np.random.default_rng(0)
    a = (rng.standard_normal(10000) * np.exp(rng.uniform(-20, 20, 10000))).astype(np.float32)
    a[:4] = [0.0, -0.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8]  # ties to even
    ref = torch.from_numpy(a).to(torch.bfloat16).to(torch.float32).numpy()
    assert np.array_equal(mlp_ref.bf16(a), ref)


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(1)
    p = mlp_ref.init_params(3).astype(np.float64)
    p[mlp_ref.n_params() - 3:] = rng.standard_normal(3) * 0.1
    x = rng.standard_normal((7, mlp_ref.N_IN))
    t = rng.standard_normal((7, mlp_ref.N_OUT)) * 0.1
    _, g = mlp_ref.loss_and_grads(p, x, t, exact=True)
    # float64 finite differences on a sample of parameters from every block
    idx = np.concatenate([rng.choice(np.arange(a, b), min(6, b - a), replace=False) for a, b in
                          ((0, 12288), (12288, 12416), (12416, 28800), (28800, 28928), (28928, 29312),
                           (29312, 29315))])
    for q in idx:
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[q] += h
        pm[q] -= h
        # split() casts to float32: evaluate the loss in float64 directly
        lp = _loss64(pp, x, t)
        lm = _loss64(pm, x, t)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[q]) <= 1e-5 * max(1.0, abs(g[q])), (q, fd, g[q])


def _loss64(p, x, t):
    o = 0
    parts = []
    for shape in ((128, 96), (128,), (128, 128), (128,), (3, 128), (3,)):
        n = int(np.prod(shape))
        parts.append(p[o:o + n].reshape(shape))
        o += n
    w1, b1, w2, b2, w3, b3 = parts
    h1 = mlp_ref.gelu(x @ w1.T + b1)
    h2 = mlp_ref.gelu(h1 @ w2.T + b2)
    y = h2 @ w3.T + b3
    return float(np.sum((y - t) ** 2) / x.shape[0])


def test_adam_first_step_is_signed_lr():
    g = np.array([1e-3, -2.0, 5.0], np.float64)
    p, m, v = mlp_ref.adam_step(np.zeros(3), g, np.zeros(3), np.zeros(3), 1, lr=1e-3)
    assert np.allclose(p, -1e-3 * np.sign(g), rtol=1e-4)


def test_f16_forward_is_closer_to_exact_than_bf16():
    """The F16 rounding model of the tensor-core inference kernel: within a
    few 1e-3 of the unrounded network, and closer to it than the BF16 model
    (the features and W1 are BF16 in both)."""
    rng = np.random.default_rng(5)
    p = mlp_ref.init_params(5)
    p[12288:12416] = rng.standard_normal(128) * 0.1
    p[28928:29312] *= 10.0
    x = rng.standard_normal((500, 96)).astype(np.float32)
    exact = mlp_ref.forward(p, x, exact=True)["y"]
    e16 = np.linalg.norm(mlp_ref.forward_f16(p, x) - exact) / np.linalg.norm(exact)
    eb = np.linalg.norm(mlp_ref.forward(p, x)["y"] - exact) / np.linalg.norm(exact)
    assert e16 < 5e-3
    assert e16 < eb
