"""The triply periodic settling sphere: the plain FP64 path with periodic z
(IBM_BC_PERIODIC) against the FP64 oracle's periodic-z variant.

64^3 unit cube, one sphere of D = 16 dx at the centre, density ratio 1.5,
Galileo 150, fluid at rest.  The reference cannot express this case (its z
boundaries are walls); the oracle restates the same algorithm with periodic
ghost planes, a cyclic Poisson solve in z and wrapped IBM stencils, sphere
integrals and position.  Parity: <= 1e-10 relative L2 after 10 steps, and
after the configuration's 200 steps (the reference's adaptive dt = 0.75
dtmax cadence; the wake is steady at Ga = 150, so round-off does not grow:
measured 2e-14), during which the sphere falls through the periodic
boundary three times."""
import numpy as np
import pytest

from _util import PLAIN_TOL_10STEP, field_errors, particle_errors
from interparts_mpich_gb300 import IBM_MODE_MIXED, IBMSolver
from interparts_mpich_gb300._abi import IBM_BC_FREESLIP, IBM_BC_PERIODIC
from interparts_mpich_gb300.cases import settling_case
from oracle.oracle import OracleSolver

pytestmark = pytest.mark.gpu


def test_periodic_settling_10_steps(gpu_lib):
    case = settling_case(64)
    g = IBMSolver(case)
    o = OracleSolver(case)
    vg = g.setup()
    vo = o.setup()
    assert abs(vg - vo) <= 1e-12 * abs(vo)
    dt = 0.5 * o.chkdt()
    g.run(dt, 10)
    o.run(dt, 10)
    e = field_errors(g.get_fields(), o.get_fields())
    pe = particle_errors(g.get_particles(lagrangian=False), o.get_particles(lagrangian=False))
    print("\nperiodic settling sphere 64^3, 10 steps vs oracle: " +
          ", ".join(f"{k} {v:.3e}" for k, v in {**e, **pe}.items()))
    assert max(e.values()) <= PLAIN_TOL_10STEP, e
    assert max(pe.values()) <= PLAIN_TOL_10STEP, pe
    _, mg, _ = g.chkdiv()
    _, mo, _ = o.chkdiv()
    assert abs(mg - mo) <= 1e-12 and mg < 1e-12
    g.close()
    o.close()


def test_periodic_settling_200_steps_crosses_boundary(gpu_lib):
    case = settling_case(64)
    g = IBMSolver(case)
    o = OracleSolver(case)
    g.setup()
    o.setup()
    dt_g = dt_o = 0.5 * o.chkdt()
    t_g = t_o = 0.0
    zs = []
    for _ in range(10):  # 200 steps, dt = 0.75 dtmax every 5 steps
        dt_g, t_g = g.run_adaptive(20, 5, dt_g, t_g)
        dt_o, t_o = o.run_adaptive(20, 5, dt_o, t_o)
        zs.append(float(g.get_particles(lagrangian=False).z[0]))
    assert abs(dt_g - dt_o) <= 1e-10 * dt_o and abs(t_g - t_o) <= 1e-10 * t_o
    e = field_errors(g.get_fields(), o.get_fields())
    pg, po = g.get_particles(lagrangian=False), o.get_particles(lagrangian=False)
    pe = particle_errors(pg, po)
    print(f"\nperiodic settling sphere 64^3, 200 steps (t = {t_g:.3f}) vs oracle: " +
          ", ".join(f"{k} {v:.3e}" for k, v in {**e, **pe}.items()) + f"; w {pg.w[0]:.4f}; z every 20 steps "
          + " ".join(f"{z:.3f}" for z in zs))
    assert max(e.values()) <= PLAIN_TOL_10STEP, e
    assert max(pe.values()) <= PLAIN_TOL_10STEP, pe
    # it settles (w < 0) and has wrapped through z = 0 to the top of the cube
    assert pg.w[0] < 0
    assert any(b > a + 0.5 for a, b in zip(zs, zs[1:])), zs
    g.close()
    o.close()


def test_periodic_z_restrictions(gpu_lib):
    case = settling_case(64)
    with pytest.raises(Exception):
        IBMSolver(case, mode=IBM_MODE_MIXED)  # plain FP64 form only
    one_sided = settling_case(64)
    one_sided.bc_bot = IBM_BC_FREESLIP
    with pytest.raises(Exception):
        IBMSolver(one_sided)
    g = IBMSolver(case)
    g.setup()
    with pytest.raises(Exception):
        g.post1d()
    with pytest.raises(Exception):
        g.set_scalar(pran=1.0)
    assert case.bc_top == IBM_BC_PERIODIC
    g.close()
