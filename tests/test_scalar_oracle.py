"""Pins of the oracle's scalar transport (scalad, scal.f90:11-58, in the RK3
substeps of rk3.f90:13-329, boundscal bound.f90:109-171) by known answers:

* a linear conduction profile between Dirichlet walls is steady;
* a Fourier mode at rest decays at the semi-discrete rate of the 3-point
  Laplacian, kappa*(2/dx*sin(pi*dx/lx))**2, to the RK3 truncation error;
* with Neumann walls and a divergence-free flow the scalar is conserved;
* buoyancy (momzbuoy, mom.f90:233-259) of a uniform scalar is a uniform
  force that the projection balances: the velocity stays at rest.
"""
import math

import numpy as np

from interparts_mpich_gb300 import IBM_BC_FREESLIP
from interparts_mpich_gb300._abi import IBM_BC_C_DIRICHLET, IBM_BC_C_NEUMANN
from interparts_mpich_gb300.cases import Case
from oracle.oracle import OracleSolver


def _rest(n=16, **kw):
    case = Case(name="scal", itot=n, jtot=n, ktot=n, np=0, visc=1e-2, flow="pur", perturb=0.0, **kw)
    s = OracleSolver(case)
    s.setup()
    return s, case


def _zc(case):
    return (np.arange(case.ktot + 2) - 0.5) / case.ktot


def test_linear_conduction_profile_is_steady():
    s, case = _rest()
    z = _zc(case)
    c0 = np.asfortranarray(np.broadcast_to((1.0 - z)[None, None, :], case.shape).copy())
    s.set_scalar(c0, pran=0.7, bc_c_top_val=0.0, bc_c_bot_val=1.0)
    for _ in range(5):
        s.rk3_step(1e-3)
    c, _ = s.get_scalar()
    assert np.abs(c[1:-1, 1:-1, 1:-1] - c0[1:-1, 1:-1, 1:-1]).max() < 1e-13


def test_fourier_mode_decay_rate():
    n = 16
    s, case = _rest(n)
    x = (np.arange(n + 2) - 0.5) / n
    c0 = np.asfortranarray(np.broadcast_to(np.cos(2 * math.pi * x)[:, None, None], case.shape).copy())
    pran = 0.5
    s.set_scalar(c0, pran=pran, bc_c_top_type=IBM_BC_C_NEUMANN, bc_c_bot_type=IBM_BC_C_NEUMANN)
    kappa = case.visc / pran
    lam = kappa * (2 * n * math.sin(math.pi / n)) ** 2
    dt, nsteps = 2e-3, 20
    for _ in range(nsteps):
        s.rk3_step(dt)
    c, _ = s.get_scalar()
    ratio = c[1:-1, 1:-1, 1:-1] / c0[1:-1, 1:-1, 1:-1]
    expected = math.exp(-lam * dt * nsteps)
    assert np.abs(ratio - expected).max() < 1e-6 * expected, (ratio.mean(), expected)


def test_scalar_conserved_with_neumann_walls():
    case = Case(name="scal", itot=16, jtot=16, ktot=16, np=0, visc=1e-2, flow="poi", perturb=0.05, seed=4)
    s = OracleSolver(case)
    s.setup()
    rng = np.random.default_rng(1)
    c0 = np.asfortranarray(rng.uniform(0, 1, case.shape))
    s.set_scalar(c0, pran=1.0, bc_c_top_type=IBM_BC_C_NEUMANN, bc_c_bot_type=IBM_BC_C_NEUMANN)
    c1, _ = s.get_scalar()
    total0 = c1[1:-1, 1:-1, 1:-1].sum()
    dt = 0.5 * s.chkdt()
    for _ in range(5):
        s.rk3_step(dt)
    c, _ = s.get_scalar()
    assert abs(c[1:-1, 1:-1, 1:-1].sum() - total0) < 1e-10 * total0


def test_uniform_buoyancy_is_balanced_by_pressure():
    s, case = _rest(bc_top=IBM_BC_FREESLIP, bc_bot=IBM_BC_FREESLIP)
    c0 = np.full(case.shape, 0.3, order="F")
    s.set_scalar(c0, pran=1.0, beta=2.0, bc_c_top_type=IBM_BC_C_NEUMANN, bc_c_bot_type=IBM_BC_C_NEUMANN)
    for _ in range(3):
        s.rk3_step(1e-3)
    f = s.get_fields()
    for name in ("u", "v", "w"):
        assert np.abs(f[name][1:-1, 1:-1, 1:-1]).max() < 1e-12, name
    c, _ = s.get_scalar()
    assert np.abs(c[1:-1, 1:-1, 1:-1] - 0.3).max() < 1e-14
