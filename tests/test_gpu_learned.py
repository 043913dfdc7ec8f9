"""Learned forcing (IBM_MODE_MIXED_LEARNED): the library's BF16 tensor-core
training kernels against the CPU reference (oracle/mlp_ref.py), and what the
trained network gains over the forcing loop without it."""
import numpy as np
import pytest

from _util import field_errors, small_case
from interparts_mpich_gb300 import IBM_MODE_MIXED, IBM_MODE_MIXED_LEARNED, IBMSolver
from oracle import mlp_ref
from oracle.oracle import OracleSolver

pytestmark = pytest.mark.gpu

# GPU vs reference: the reference rounds to BF16 where the GPU does; what is
# left is FP32 summation order inside the tensor-core tiles and tanhf, which
# can move a value across a BF16 rounding boundary now and then.
GRAD_REL_TOL = 5e-3
OUT_REL_TOL = 2e-3
# the tensor-core inference kernel keeps its hidden activations in F16, the
# training kernels and the mma.sync inference kernel in BF16: the two differ
# by the BF16 rounding of the activations (3-4e-3 relative on these batches)
F16_VS_BF16_TOL = 6e-3


def _blocks():
    o = 0
    for name, shape in (("W1", (128, 96)), ("b1", (128,)), ("W2", (128, 128)), ("b2", (128,)),
                        ("W3", (3, 128)), ("b3", (3,))):
        n = int(np.prod(shape))
        yield name, slice(o, o + n)
        o += n


def _batch(nb, seed):
    rng = np.random.default_rng(seed)
    p = mlp_ref.init_params(seed)
    p[12288:12416] = rng.standard_normal(128) * 0.1   # b1
    p[28800:28928] = rng.standard_normal(128) * 0.1   # b2
    p[28928:29312] *= 10.0                             # W3 of order 1
    x = rng.standard_normal((nb, 96)).astype(np.float32)
    t = rng.standard_normal((nb, 3)).astype(np.float32)
    return p.astype(np.float32), x, t


@pytest.mark.parametrize("nb", [64, 200, 1000])
def test_mlp_gradient_matches_cpu_reference(gpu_lib, nb):
    case = small_case(n=16, nsp=0)
    g = IBMSolver(case, mode=IBM_MODE_MIXED_LEARNED)
    p, x, t = _batch(nb, seed=nb)
    loss, grad, y = g.mlp_gradient(p, x, t)
    f = mlp_ref.forward(p, x)
    ref_loss, ref_grad = mlp_ref.loss_and_grads(p, x, t)
    assert np.linalg.norm(y - f["y"]) <= OUT_REL_TOL * np.linalg.norm(f["y"])
    assert abs(loss - ref_loss) <= OUT_REL_TOL * ref_loss
    for name, sl in _blocks():
        a, b = grad[sl].astype(np.float64), ref_grad[sl]
        err = np.linalg.norm(a - b) / np.linalg.norm(b)
        assert err <= GRAD_REL_TOL, (name, err)


@pytest.mark.parametrize("nb", [16, 1000, 20011])
def test_mlp_inference_matches_cpu_reference(gpu_lib, nb):
    """The fused inference kernel (register-resident hidden layer) against
    the CPU reference and against the training forward."""
    case = small_case(n=16, nsp=0)
    g = IBMSolver(case, mode=IBM_MODE_MIXED_LEARNED)
    p, x, t = _batch(nb, seed=nb + 1)
    y = g.mlp_infer(p, x)
    ref = mlp_ref.forward(p, x)["y"]
    assert np.linalg.norm(y - ref) <= OUT_REL_TOL * np.linalg.norm(ref)
    _, _, y_train = g.mlp_gradient(p, x, t)
    assert np.linalg.norm(y - y_train) <= OUT_REL_TOL * np.linalg.norm(ref)


@pytest.mark.parametrize("nb", [16, 128, 1000, 20011])
def test_mlp_inference_tcgen05_matches_cpu_reference(gpu_lib, nb):
    """The tcgen05 inference kernel (TMEM accumulators, F16 hidden
    activations) against the CPU reference with its rounding points, the
    mma.sync inference kernel, and the unrounded network: no less accurate
    than the BF16 path."""
    case = small_case(n=16, nsp=0)
    g = IBMSolver(case, mode=IBM_MODE_MIXED_LEARNED)
    p, x, _ = _batch(nb, seed=nb + 7)
    y = g.mlp_infer_tc(p, x)
    ref = mlp_ref.forward_f16(p, x)
    assert np.linalg.norm(y - ref) <= OUT_REL_TOL * np.linalg.norm(ref)
    assert np.linalg.norm(y - g.mlp_infer(p, x)) <= F16_VS_BF16_TOL * np.linalg.norm(ref)
    exact = mlp_ref.forward(p, x, exact=True)["y"]
    bf = mlp_ref.forward(p, x)["y"]
    assert np.linalg.norm(y - exact) <= np.linalg.norm(bf - exact)


def test_mlp_adam_steps_match_cpu_reference(gpu_lib):
    case = small_case(n=16, nsp=0)
    g = IBMSolver(case, mode=IBM_MODE_MIXED_LEARNED)
    p, x, t = _batch(256, seed=7)
    lr = 1e-3
    out, losses = g.mlp_fit(p, x, t, nsteps=3, lr=lr)
    q = p.astype(np.float64)
    m = np.zeros_like(q)
    v = np.zeros_like(q)
    ref_losses = []
    for s in range(1, 4):
        ls, gr = mlp_ref.loss_and_grads(q.astype(np.float32), x, t)
        ref_losses.append(ls)
        q, m, v = mlp_ref.adam_step(q, gr, m, v, s, lr=lr)
    assert np.allclose(losses, ref_losses, rtol=OUT_REL_TOL)
    # each Adam step moves a weight by about lr: compare the displacements
    d_gpu = out.astype(np.float64) - p
    d_ref = q - p
    assert np.linalg.norm(d_gpu - d_ref) <= 2e-2 * np.linalg.norm(d_ref)


def test_mlp_training_reduces_loss(gpu_lib):
    """A learnable target (a fixed random network of the same shape): the
    GPU training loop drives the loss down by orders of magnitude."""
    case = small_case(n=16, nsp=0)
    g = IBMSolver(case, mode=IBM_MODE_MIXED_LEARNED)
    rng = np.random.default_rng(3)
    x = rng.standard_normal((2048, 96)).astype(np.float32)
    teacher = mlp_ref.init_params(11)
    t = mlp_ref.forward(teacher, x)["y"].astype(np.float32)
    t /= t.std()
    _, losses = g.mlp_fit(mlp_ref.init_params(12), x, t, nsteps=400, lr=2e-3)
    assert losses[-1] < 0.05 * losses[0], (losses[0], losses[-1])


def _flow_case():
    return small_case(n=48, nsp=10, radius_cells=5.0, seed=11, visc=1.0 / 1000.0)


@pytest.fixture(scope="module")
def trained(gpu_lib):
    """Harvest from the plain Nl=3 passes of 8 steps, train on the GPU."""
    case = _flow_case()
    s = IBMSolver(case, mode=IBM_MODE_MIXED_LEARNED)
    s.setup()
    dt = 0.5 * s.chkdt()
    s.harvest(capacity=400000, stride=1, passes=3)
    s.run(dt, 8)
    s.harvest(0)
    st = s.learned_stats()
    loss = s.train_forcing_model(nsteps=6000, batch=4096, lr=1e-3, seed=1)
    s.learned_calibration(0)  # the tests below call loops one at a time: no interleaved plain loops
    return s, dt, loss, st


def test_standardisation_matches_numpy(trained):
    """The device's two-pass FP64 column statistics of the harvested set
    against numpy's on the same samples (read back through the C ABI)."""
    s = trained[0]
    f, t = s.harvest_read()
    assert f.shape[0] > 10000
    _, norm = s.get_forcing_model()
    mu, sd = f.astype(np.float64).mean(0), f.astype(np.float64).std(0)
    tmu, tsd = t.astype(np.float64).mean(0), t.astype(np.float64).std(0)
    scale = np.maximum(sd, 1e-30)
    assert np.all(np.abs(norm[:96] - mu) <= 1e-5 * scale + 1e-6 * np.abs(mu))
    isd = np.where(sd > 1e-30, 1.0 / scale, 0.0)
    assert np.allclose(norm[96:192], isd, rtol=1e-5, atol=0)
    assert np.allclose(norm[192:195], tmu, rtol=1e-5, atol=1e-6 * tsd.max())
    assert np.allclose(norm[195:198], tsd, rtol=1e-5)


def _loop_residual(s, dt, nl):
    s.rk(1, dt)
    s.forcing_loop(dt, nl)
    return s.slip_residual()[1]


def test_learned_forcing_gain(trained):
    """Same state, same substep: the network after one plain sweep against
    the plain loop with one sweep (the method without it) and with Nl=3."""
    s, dt, loss, st = trained
    assert st["harvested"] > 10000 and st["plain_rms_ref"] > 0
    assert loss < 0.2, loss
    s.learned_config(enable=False)
    res_plain3 = _loop_residual(s, dt, 3)
    res_one = _loop_residual(s, dt, 1)
    s.learned_config(enable=True, fallback_ratio=1e9)
    res_learned = _loop_residual(s, dt, 3)
    stats = s.learned_stats()
    assert stats["fallbacks"] == 0
    print(f"rms no-slip residual: one sweep {res_one:.3e}, plain Nl=3 {res_plain3:.3e}, "
          f"one sweep + network {res_learned:.3e}")
    assert res_learned < 0.5 * res_one
    # the fallback criterion: within 1.5x of the plain loop's residual
    assert res_learned <= 1.5 * res_plain3


def test_learned_fallback_runs_plain_passes(trained):
    s, dt, _, _ = trained
    s.learned_config(enable=True, fallback_ratio=1e9)
    res_learned = _loop_residual(s, dt, 3)
    before = s.learned_stats()["fallbacks"]
    s.learned_config(enable=True, fallback_ratio=1e-12)  # every loop fails the test
    res_fb = _loop_residual(s, dt, 3)
    assert s.learned_stats()["fallbacks"] == before + 1
    assert res_fb < res_learned
    s.learned_config(enable=True, fallback_ratio=1.5)


def test_learned_model_roundtrip(trained):
    s, dt, _, _ = trained
    p, n = s.get_forcing_model()
    assert p.shape == (29315,) and n.shape == (198,) and np.all(np.isfinite(p))
    case = _flow_case()
    t = IBMSolver(case, mode=IBM_MODE_MIXED_LEARNED)
    t.set_forcing_model(p, n)
    q, m = t.get_forcing_model()
    assert np.array_equal(p, q) and np.array_equal(n, m)


def _steps(s, dt, nl, nsteps):
    for _ in range(nsteps):
        for r in (1, 2, 3):
            s.rk(r, dt)
            s.forcing_loop(dt, nl)
            s.project(r, dt)
            s.intgr_nwtn_eulr(r, dt)


def test_learned_20_steps_within_oracle_nl_spread(trained):
    """A fresh run with the trained model against the FP64 oracle after 20
    steps.  This is not the 1e-4 velocity target (the bench-size test
    test_gpu_fullsize.py holds that target, marked as missed): the learned
    correction approximates the plain Nl = 3 correction, and its flow departs
    from the Nl = 3 oracle by less than the plain method itself moves
    between Nl = 3 and Nl = 6 on this case."""
    s, dt, _, _ = trained
    p, n = s.get_forcing_model()
    case = _flow_case()
    m = IBMSolver(case, mode=IBM_MODE_MIXED_LEARNED)
    m.setup()
    m.set_forcing_model(p, n)
    m.learned_config(enable=True, fallback_ratio=1.5)
    m.run(dt, 20)
    o3 = OracleSolver(case)
    o3.setup()
    _steps(o3, dt, 3, 20)
    o6 = OracleSolver(case)
    o6.setup()
    _steps(o6, dt, 6, 20)
    f3 = o3.get_fields()
    e_learned = max(field_errors(m.get_fields(), f3, names=("u", "v", "w")).values())
    e_nl = max(field_errors(o6.get_fields(), f3, names=("u", "v", "w")).values())
    st = m.learned_stats()
    gs = m.learned_gate_state()
    print(f"velocity rel L2 after 20 steps vs oracle Nl=3: learned {e_learned:.3e}, oracle Nl=6 {e_nl:.3e}; "
          f"learned loops {int(st['learned_loops'])}, plain calibration loops {int(gs['plain_loops'])}, "
          f"fallbacks {int(st['fallbacks'])}")
    assert e_learned < e_nl
    assert st["learned_loops"] + gs["plain_loops"] == 60


def test_fallback_gate_fires_on_degraded_network(trained):
    """Mid-run on the 48^3 flow: the live gate compares the learned
    residual with 1.5 x the plain passes' reduction of the same loop's
    first-pass slip.  With the trained network its residual sits near the
    plain method's (ratio about 1.0-1.4 from substep to substep), so the gate
    lets at least three loops in four through; with every weight and bias of
    the network halved every loop falls back."""
    s, dt, _, _ = trained
    p, n = s.get_forcing_model()
    case = _flow_case()
    m = IBMSolver(case, mode=IBM_MODE_MIXED_LEARNED)
    m.setup()
    m.set_forcing_model(p, n)
    m.learned_config(enable=True, fallback_ratio=1.5)
    m.run(dt, 4)
    good = m.learned_stats()
    g_good = m.learned_gate_state()
    m.set_forcing_model(0.5 * p, n)
    m.learned_config(enable=True, fallback_ratio=1.5)
    m.run(dt, 2)
    bad = m.learned_stats()
    g_bad = m.learned_gate_state()
    print(f"good network: residual {good['last_rms']:.3e} vs reference {good['plain_rms_ref']:.3e} "
          f"(plain factor {g_good['plain_factor']:.3f}), fallbacks {int(good['fallbacks'])}; degraded: residual "
          f"{bad['last_rms']:.3e} vs reference {bad['plain_rms_ref']:.3e}, fallbacks "
          f"{int(bad['fallbacks'] - good['fallbacks'])} of {int(bad['learned_loops'] - good['learned_loops'])}")
    assert good["learned_loops"] > 0 and 4 * good["fallbacks"] <= good["learned_loops"]
    n_bad = bad["learned_loops"] - good["learned_loops"]
    assert n_bad > 0 and bad["fallbacks"] - good["fallbacks"] == n_bad
    assert bad["last_rms"] > 1.5 * bad["plain_rms_ref"]


def _point_force_error(s, dt):
    """Same state, same substep: the learned loop's point forces against the
    plain Nl = 3 loop's, rms of the difference of F*dt per component."""
    s.learned_config(enable=False)
    s.rk(1, dt)
    s.forcing_loop(dt, 3)
    f3 = s.get_particles()
    s.learned_config(enable=True, fallback_ratio=1e9)
    s.rk(1, dt)
    s.forcing_loop(dt, 3)
    fl = s.get_particles()
    s.learned_config(enable=True, fallback_ratio=1.5)
    return [float(np.sqrt(np.mean(((getattr(fl, n) - getattr(f3, n)) * dt) ** 2))) for n in ("fxl", "fyl", "fzl")]


def test_learned_error_budget_noise_ablation(trained):
    """What the learned form's 20-step deviation is made of.  sigma = the
    network's per-point error of F*dt on the same state; the mixed form with
    the exact Nl = 3 forcing plus independent point noise of that rms (and
    of a tenth of it) runs 20 steps against the oracle, beside the learned
    form.  A deviation that scales with the noise shows a linear response
    (no chaotic growth over 20 steps); the printed numbers compare the
    network's error with uncorrelated noise of the same size."""
    s, dt, _, _ = trained
    sigma = _point_force_error(s, dt)
    case = _flow_case()
    o = OracleSolver(case)
    o.setup()
    _steps(o, dt, 3, 20)
    fo = o.get_fields()
    errs = {}
    for scale in (1.0, 0.1):
        m = IBMSolver(case, mode=IBM_MODE_MIXED)
        m.setup()
        m.forcing_perturbation([scale * x for x in sigma], seed=7)
        m.run(dt, 20)
        errs[scale] = max(field_errors(m.get_fields(), fo, names=("u", "v", "w")).values())
        m.close()
    p, n = s.get_forcing_model()
    lm = IBMSolver(case, mode=IBM_MODE_MIXED_LEARNED)
    lm.setup()
    lm.set_forcing_model(p, n)
    lm.learned_config(enable=True, fallback_ratio=1.5)
    lm.run(dt, 20)
    e_learned = max(field_errors(lm.get_fields(), fo, names=("u", "v", "w")).values())
    print(f"network per-point error of F*dt (u, v, w): {sigma[0]:.3e} {sigma[1]:.3e} {sigma[2]:.3e}; "
          f"20-step velocity rel L2 vs oracle: exact Nl=3 + noise sigma {errs[1.0]:.3e}, + noise sigma/10 "
          f"{errs[0.1]:.3e}, learned {e_learned:.3e}")
    assert all(x > 0 for x in sigma)
    assert errs[1.0] > errs[0.1] > 1e-6
    # linear response: a tenth of the noise gives about a tenth of the deviation
    assert 3.0 < errs[1.0] / errs[0.1] < 30.0
