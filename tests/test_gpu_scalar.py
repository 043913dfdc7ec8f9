"""Scalar transport and buoyancy on the GPU (ibm_set_scalar; scalad and the
dcdt update in every RK substep, boundscal after the projection, momzbuoy in
the w predictor) against the oracle, with particles."""
import numpy as np
import pytest

from _util import PLAIN_TOL_10STEP, field_errors, particle_errors, rel_l2, small_case
from interparts_mpich_gb300 import IBM_MODE_MIXED, IBM_MODE_PLAIN_FP64, IBMSolver
from interparts_mpich_gb300._abi import IBM_BC_C_DIRICHLET, IBM_BC_C_NEUMANN
from oracle.oracle import OracleSolver

pytestmark = pytest.mark.gpu

# mixed form: FP32 velocities advect the FP64 scalar
MIXED_SCALAR_TOL = 1e-5


def _scalar(case):
    rng = np.random.default_rng(8)
    z = (np.arange(case.ktot + 2) - 0.5) / case.ktot
    c = np.broadcast_to((1.0 - z)[None, None, :], case.shape).copy()
    c += 0.05 * rng.standard_normal(case.shape)
    return np.asfortranarray(c)


@pytest.mark.parametrize("top", [IBM_BC_C_DIRICHLET, IBM_BC_C_NEUMANN])
def test_scalar_transport_matches_oracle_plain(gpu_lib, top):
    case = small_case(n=32, nsp=6, radius_cells=4.0, seed=21)
    g = IBMSolver(case, mode=IBM_MODE_PLAIN_FP64)
    o = OracleSolver(case)
    c0 = _scalar(case)
    for s in (g, o):
        s.setup()
        s.set_scalar(c0, pran=0.71, beta=0.5, bc_c_top_val=0.0, bc_c_bot_val=1.0, bc_c_top_type=top)
    dt = 0.5 * o.chkdt()
    g.run(dt, 10)
    o.run(dt, 10)
    cg, rg = g.get_scalar()
    co, ro = o.get_scalar()
    assert rel_l2(cg[1:-1, 1:-1, 1:-1], co[1:-1, 1:-1, 1:-1]) <= PLAIN_TOL_10STEP
    assert rel_l2(rg[1:-1, 1:-1, 1:-1], ro[1:-1, 1:-1, 1:-1]) <= PLAIN_TOL_10STEP
    # ghost planes of boundscal
    assert np.allclose(cg[:, :, 0], co[:, :, 0], rtol=0, atol=1e-10)
    assert np.allclose(cg[:, :, -1], co[:, :, -1], rtol=0, atol=1e-10)
    err = field_errors(g.get_fields(), o.get_fields())
    assert max(err.values()) <= PLAIN_TOL_10STEP, err
    perr = particle_errors(g.get_particles(), o.get_particles())
    assert perr["pos"] <= PLAIN_TOL_10STEP, perr
    # the buoyancy moved the flow: compare with a run without scalar
    h = IBMSolver(case, mode=IBM_MODE_PLAIN_FP64)
    h.setup()
    h.run(dt, 10)
    assert rel_l2(h.get_fields()["w"][1:-1, 1:-1, 1:-1], g.get_fields()["w"][1:-1, 1:-1, 1:-1]) > 1e-6


def test_scalar_transport_mixed(gpu_lib):
    case = small_case(n=32, nsp=6, radius_cells=4.0, seed=21)
    g = IBMSolver(case, mode=IBM_MODE_MIXED)
    o = OracleSolver(case)
    c0 = _scalar(case)
    for s in (g, o):
        s.setup()
        s.set_scalar(c0, pran=0.71, beta=0.5, bc_c_top_val=0.0, bc_c_bot_val=1.0)
    dt = 0.5 * o.chkdt()
    g.run(dt, 10)
    o.run(dt, 10)
    cg, _ = g.get_scalar()
    co, _ = o.get_scalar()
    err = rel_l2(cg[1:-1, 1:-1, 1:-1], co[1:-1, 1:-1, 1:-1])
    print(f"mixed form scalar rel L2 after 10 steps: {err:.2e}")
    assert err <= MIXED_SCALAR_TOL
