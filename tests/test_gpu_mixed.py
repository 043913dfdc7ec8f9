"""The mixed-precision form (IBM_MODE_MIXED) against the FP64 oracle.

FP32 velocity state, stencil, IBM interpolation/spreading and FFTs;
double-float Thomas sweep and pressure accumulation; one FP32 projection
solve (default) or the solve plus a defect-correction solve driven by the
double-float divergence residual; FP64 sphere integral totals and
Newton-Euler.  Target: velocity relative L2 <= 1e-4 after 20 RK3 steps."""
import numpy as np
import pytest

from _util import field_errors, particle_errors, rel_l2, small_case
from interparts_mpich_gb300 import IBM_MODE_MIXED, IBMSolver
from oracle.oracle import OracleSolver

pytestmark = pytest.mark.gpu

MIXED_VEL_TOL_20 = 1e-4


@pytest.mark.parametrize("solves", [1, 2])
def test_mixed_20_steps(gpu_lib, solves):
    case = small_case(n=48, nsp=10, radius_cells=5.0, seed=11, visc=1.0 / 1000.0)
    m = IBMSolver(case, mode=IBM_MODE_MIXED)
    m.set_projection_solves(solves)
    o = OracleSolver(case)
    m.setup()
    o.setup()
    dt = 0.5 * o.chkdt()
    m.run(dt, 20)
    o.run(dt, 20)
    e = field_errors(m.get_fields(), o.get_fields(), names=("u", "v", "w"))
    assert max(e.values()) <= MIXED_VEL_TOL_20, e
    pe = particle_errors(m.get_particles(), o.get_particles())
    assert max(pe.values()) <= 1e-4, pe
    tot, mx, _ = m.chkdiv()
    # the velocity state is FP32: the divergence is bounded by its rounding,
    # relative to the velocity-gradient scale |u|/dx
    umax = max(np.abs(m.get_fields()[n]).max() for n in "uvw")
    assert mx / (umax * case.dxi) < 1e-6, mx


@pytest.mark.parametrize("solves", [1, 2])
def test_mixed_projection_divergence(gpu_lib, solves):
    """One FP32 solve, or the solve plus one defect-correction solve driven
    by the double-float divergence residual: the divergence ends at the
    rounding level of the FP32 velocity state."""
    case = small_case(n=64, nsp=0)
    g = IBMSolver(case, mode=IBM_MODE_MIXED)
    g.set_projection_solves(solves)
    f = case.initial_fields()
    rng = np.random.default_rng(5)
    for n in ("u", "v", "w"):
        f[n][1:-1, 1:-1, 1:-1] += rng.standard_normal(f[n][1:-1, 1:-1, 1:-1].shape) * 0.1
    g.set_fields(f["u"], f["v"], f["w"], f["p"])
    g.set_particles(case.initial_particles(False))
    g.init_particles()
    dt = 0.5 * g.chkdt()
    g.rk(1, dt)
    g.project(1, dt)
    tot, mx, _ = g.chkdiv()
    umax = max(np.abs(g.get_fields()[n]).max() for n in "uvw")
    print(f"projection solves {solves}: max|div| / (|u|max/dx) = {mx / (umax * case.dxi):.2e}")
    assert mx / (umax * case.dxi) < 1e-6, (tot, mx)


def test_mixed_collisions_same_contacts(gpu_lib):
    """Contact detection stays FP64: the contact lists of a colliding case
    match the oracle's over a few steps."""
    from test_gpu_parity import collision_case

    case = collision_case(9)
    m = IBMSolver(case, mode=IBM_MODE_MIXED)
    o = OracleSolver(case)
    m.setup()
    o.setup()
    for _ in range(6):
        m.rk3_step(2e-3)
        o.rk3_step(2e-3)
    assert m.get_particles().contact_lists() == o.get_particles().contact_lists()

