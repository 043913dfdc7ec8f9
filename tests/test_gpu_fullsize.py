"""Parity at the benchmarked configuration: the 256^3 channel with 1000
spheres of D = 16 dx (perturbed Poiseuille flow at Re_b = 5600, Nl = 3,
dt = 0.5 dtmax at t = 0, frozen), the case bench.py times.

One oracle run (the FP64 CPU restatement of the reference, OpenMP on all host
cores, about 5 s per step) gives the states after 10 and 20 RK3 steps; every
GPU form is checked against them:
  * plain FP64 (the drop-in), 10 steps: u, v, w, p, particle positions and
    velocities within 1e-10 relative L2, identical contact lists, the same
    chkdiv maximum to 1e-12;
  * mixed FP32/FP64: the per-field error table after 10 and 20 steps, the
    velocity within 1e-4 after 20;
  * learned forcing, trained with the bench's recipe (2M samples harvested
    from the plain Nl = 3 passes of six steps, 6000 Adam steps of batch 8192,
    lr 1e-3): the
    20-step error table next to the method without the network (one plain
    sweep per substep) and the 1e-4 target.
The tables are printed (pytest -s shows them)."""
import os

import numpy as np
import pytest

from _util import PLAIN_TOL_10STEP, field_errors, particle_errors
from interparts_mpich_gb300 import IBM_MODE_MIXED, IBM_MODE_MIXED_LEARNED, IBMSolver
from interparts_mpich_gb300.cases import channel_case
from oracle.oracle import OracleSolver, load

pytestmark = pytest.mark.gpu

MIXED_VEL_TOL_20 = 1e-4
LEARNED_VEL_TARGET_20 = 1e-4


def _snapshot(s):
    f = s.get_fields()
    ps = s.get_particles(lagrangian=False)
    _, mx, ijk = s.chkdiv()
    return {"fields": {n: f[n].copy() for n in "uvwp"}, "parts": ps, "divmax": mx, "ijk": ijk}


def _table(s, ref) -> dict:
    e = field_errors(s.get_fields(), ref["fields"])
    e.update(particle_errors(s.get_particles(lagrangian=False), ref["parts"]))
    return e


def _fmt(e: dict) -> str:
    return ", ".join(f"{k} {v:.3e}" for k, v in e.items())


@pytest.fixture(scope="module")
def oracle_run(gpu_lib):
    case = channel_case(256, 1000, seed=1234)
    lib, _ = load()
    lib.orc_set_threads(os.cpu_count() or 1)
    o = OracleSolver(case)
    o.setup()
    dt = 0.5 * o.chkdt()
    o.run(dt, 10)
    s10 = _snapshot(o)
    o.run(dt, 10)
    s20 = _snapshot(o)
    o.close()
    return case, dt, s10, s20


def test_plain_10_steps_fullsize(oracle_run):
    case, dt, s10, _ = oracle_run
    g = IBMSolver(case)
    g.setup()
    g.run(dt, 10)
    e = field_errors(g.get_fields(), s10["fields"])
    pe = particle_errors(g.get_particles(lagrangian=False), s10["parts"])
    print(f"\nplain FP64, 256^3, 1000 spheres, 10 steps vs oracle: {_fmt(e)}, {_fmt(pe)}")
    assert max(e.values()) <= PLAIN_TOL_10STEP, e
    assert max(pe.values()) <= PLAIN_TOL_10STEP, pe
    assert g.get_particles(lagrangian=False).contact_lists() == s10["parts"].contact_lists()
    _, mx, _ = g.chkdiv()
    print(f"chkdiv max: GPU {mx:.6e}, oracle {s10['divmax']:.6e}")
    assert abs(mx - s10["divmax"]) <= 1e-12
    g.close()


def test_mixed_20_steps_fullsize(oracle_run):
    case, dt, s10, s20 = oracle_run
    m = IBMSolver(case, mode=IBM_MODE_MIXED)
    m.setup()
    m.run(dt, 10)
    e10 = _table(m, s10)
    m.run(dt, 10)
    e20 = _table(m, s20)
    print(f"\nmixed FP32/FP64 vs oracle, 10 steps: {_fmt(e10)}\nmixed FP32/FP64 vs oracle, 20 steps: {_fmt(e20)}")
    assert max(e20[n] for n in "uvw") <= MIXED_VEL_TOL_20, e20
    assert max(e20["pos"], e20["vel"]) <= MIXED_VEL_TOL_20, e20
    assert m.get_particles(lagrangian=False).contact_lists() == s20["parts"].contact_lists()
    m.close()


def _substeps(s, dt, nl, nsteps):
    for _ in range(nsteps):
        for r in (1, 2, 3):
            s.rk(r, dt)
            s.forcing_loop(dt, nl)
            s.project(r, dt)
            s.intgr_nwtn_eulr(r, dt)


HARVEST_CAPACITY = 2_000_000
HARVEST_STEPS = 6


@pytest.fixture(scope="module")
def bench_model(oracle_run):
    """The bench's recipe: harvest every stride-th point of the plain Nl = 3
    passes of the first six steps from the initial state (2M samples), then
    train on the GPU."""
    case, dt, _, _ = oracle_run
    s = IBMSolver(case, mode=IBM_MODE_MIXED_LEARNED)
    s.setup()
    stride = -(-HARVEST_STEPS * 3 * case.np * case.nl // HARVEST_CAPACITY)
    s.harvest(capacity=HARVEST_CAPACITY, stride=stride, passes=3)
    s.run(dt, HARVEST_STEPS)
    s.harvest(0)
    loss = s.train_forcing_model(6000, batch=8192, lr=1e-3, seed=1)
    p, n = s.get_forcing_model()
    st = s.learned_stats()
    s.close()
    return p, n, loss, st


def test_learned_20_steps_fullsize(oracle_run, bench_model):
    """20 learned steps from the initial state against the oracle, beside the
    same run with one plain sweep per substep (the method without the
    network): the network must bring the flow closer to the Nl = 3 oracle
    than one sweep does, with its loops within the fallback bound."""
    case, dt, _, s20 = oracle_run
    p, n, loss, hv = bench_model
    m = IBMSolver(case, mode=IBM_MODE_MIXED_LEARNED)
    m.setup()
    m.set_forcing_model(p, n)
    m.learned_config(enable=True, fallback_ratio=1.5)
    m.run(dt, 20)
    el = _table(m, s20)
    st = m.learned_stats()
    gs = m.learned_gate_state()
    m.close()
    one = IBMSolver(case, mode=IBM_MODE_MIXED)
    one.setup()
    _substeps(one, dt, 1, 20)
    e1 = _table(one, s20)
    one.close()
    print(f"\nlearned (harvest {int(hv['harvested'])} samples, loss {loss:.4f}) vs oracle, 20 steps: {_fmt(el)}"
          f"\n  learned loops {int(st['learned_loops'])}, plain calibration loops {int(gs['plain_loops'])}, "
          f"fallbacks {int(st['fallbacks'])}, last residual {st['last_rms']:.3e} vs reference "
          f"{st['plain_rms_ref']:.3e} (plain factor {gs['plain_factor']:.3f})"
          f"\none plain sweep per substep vs oracle, 20 steps: {_fmt(e1)}")
    assert max(el[n] for n in "uvw") < max(e1[n] for n in "uvw")
    assert st["learned_loops"] + gs["plain_loops"] == 60


def test_learned_error_budget_fullsize(oracle_run, bench_model):
    """The bench network's per-point error of F*dt against the plain Nl = 3
    loop on the same state (the first substep), and the mixed form with the
    exact Nl = 3 forcing plus independent point noise of that rms, 20 steps
    against the oracle: the deviation a network with uncorrelated errors of
    that size would cause."""
    case, dt, _, s20 = oracle_run
    p, n, _, _ = bench_model
    s = IBMSolver(case, mode=IBM_MODE_MIXED_LEARNED)
    s.setup()
    s.set_forcing_model(p, n)
    s.learned_config(enable=True, fallback_ratio=1e9)
    s.learned_calibration(0)
    s.rk(1, dt)
    s.forcing_loop(dt, 3)  # the first loop with the network on measures the plain passes
    f3 = s.get_particles()
    s.rk(1, dt)
    s.forcing_loop(dt, 3)  # the same substep with the network
    fl = s.get_particles()
    assert s.learned_stats()["learned_loops"] == 1
    s.close()
    sigma = [float(np.sqrt(np.mean(((getattr(fl, k) - getattr(f3, k)) * dt) ** 2))) for k in ("fxl", "fyl", "fzl")]
    scale = [float(np.sqrt(np.mean((getattr(f3, k) * dt) ** 2))) for k in ("fxl", "fyl", "fzl")]
    m = IBMSolver(case, mode=IBM_MODE_MIXED)
    m.setup()
    m.forcing_perturbation(sigma, seed=7)
    m.run(dt, 20)
    e = _table(m, s20)
    m.close()
    print(f"\nnetwork per-point error of F*dt (u, v, w): {sigma[0]:.3e} {sigma[1]:.3e} {sigma[2]:.3e} "
          f"(rms F*dt {scale[0]:.3e} {scale[1]:.3e} {scale[2]:.3e})"
          f"\nexact Nl = 3 + point noise of that rms vs oracle, 20 steps: {_fmt(e)}")
    assert all(x > 0 for x in sigma)
    assert all(np.isfinite(v) for v in e.values())


@pytest.mark.xfail(strict=False, reason="the per-point network does not reproduce the Nl = 3 correction to the "
                                        "accuracy the 1e-4 velocity target needs (measured error printed)")
def test_learned_meets_velocity_target_fullsize(oracle_run, bench_model):
    case, dt, _, s20 = oracle_run
    p, n, _, _ = bench_model
    m = IBMSolver(case, mode=IBM_MODE_MIXED_LEARNED)
    m.setup()
    m.set_forcing_model(p, n)
    m.learned_config(enable=True, fallback_ratio=1.5)
    m.run(dt, 20)
    e = max(field_errors(m.get_fields(), s20["fields"], names=("u", "v", "w")).values())
    m.close()
    print(f"\nlearned velocity rel L2 after 20 steps: {e:.3e} (target {LEARNED_VEL_TARGET_20:.0e})")
    assert e <= LEARNED_VEL_TARGET_20, e


def test_mixed_100_steps_vs_plain_gpu(gpu_lib):
    """The mixed form on the same channel against the plain FP64 GPU path
    after 20 and 100 steps: the plain path stands in for the FP64 oracle
    beyond the 20 steps the oracle run covers (it matches the oracle to
    1e-10 over 10 steps above).  The per-field table is printed."""
    case = channel_case(256, 1000, seed=1234)
    g = IBMSolver(case)
    g.setup()
    dt = 0.5 * g.chkdt()
    m = IBMSolver(case, mode=IBM_MODE_MIXED)
    m.setup()
    out = {}
    done = 0
    for upto in (20, 100):
        g.run(dt, upto - done)
        m.run(dt, upto - done)
        done = upto
        ref = {"fields": g.get_fields(), "parts": g.get_particles(lagrangian=False)}
        out[upto] = _table(m, ref)
        print(f"\nmixed vs plain FP64 GPU, {upto} steps: {_fmt(out[upto])}")
    g.close()
    m.close()
    assert max(out[20][n] for n in "uvw") <= MIXED_VEL_TOL_20
    assert all(np.isfinite(v) for v in out[100].values())
