"""The FP32 predictor of the mixed forms (rk1..rk3 fused with mom.f90) in
its four kernels: planes staged in shared memory by 16-byte loads (the
default), by 4-byte loads, by tensor-memory-accelerator copies (the same
arithmetic in all three), and one cell per thread (terms grouped
differently).  The forced predictor dudt, dvdt, dwdt of the first RK stage
must agree bit for bit among the first three and to FP32 rounding with the
fourth, and stay within FP32 rounding through the later stages (whose input
carries the IBM loop's atomic flush order), on grids whose rows are a
multiple of the 64-cell tile, narrower than it (the staged rows wrap the
periodic domain more than once) and not a multiple of it."""
import numpy as np
import pytest

from _util import small_case
from interparts_mpich_gb300 import IBM_MODE_MIXED, IBMSolver
from interparts_mpich_gb300._abi import (IBM_PREDICTOR_AUTO, IBM_PREDICTOR_CELLS, IBM_PREDICTOR_PAIRS,
                                        IBM_PREDICTOR_TMA)

pytestmark = pytest.mark.gpu


def _stages(case, kind, dt):
    s = IBMSolver(case, mode=IBM_MODE_MIXED)
    s.setup()
    s.set_predictor_kernel(kind)
    out = []
    for r in (1, 2, 3):
        s.rk(r, dt)
        out.append(s.get_intermediate())
        s.forcing_loop(dt, 3)
        s.project(r, dt)
        s.intgr_nwtn_eulr(r, dt)
    s.close()
    return out


@pytest.mark.parametrize("n,nsp", [(64, 4), (48, 3), (96, 6)])
def test_predictor_kernels_agree(gpu_lib, n, nsp):
    case = small_case(n=n, nsp=nsp, radius_cells=5.0, seed=5, visc=1.0 / 1000.0)
    probe = IBMSolver(case, mode=IBM_MODE_MIXED)
    probe.setup()
    dt = 0.5 * probe.chkdt()
    probe.close()
    quad = _stages(case, IBM_PREDICTOR_AUTO, dt)
    pairs = _stages(case, IBM_PREDICTOR_PAIRS, dt)
    tma = _stages(case, IBM_PREDICTOR_TMA, dt)
    cells = _stages(case, IBM_PREDICTOR_CELLS, dt)
    for st in range(3):
        for name in ("dudt", "dvdt", "dwdt"):
            q, p, t, c = (r[st][name][1:-1, 1:-1, 1:-1] for r in (quad, pairs, tma, cells))
            if st == 0:
                assert np.array_equal(q, p), (n, st, name, float(np.abs(q - p).max()))
                assert np.array_equal(q, t), (n, st, name, float(np.abs(q - t).max()))
            for other, tol in ((p, 1e-6), (t, 1e-6), (c, 1e-5)):
                rel = float(np.linalg.norm(q - other) / np.linalg.norm(other))
                assert rel <= tol, (n, st, name, rel)


def test_predictor_kernel_rejects_unknown(gpu_lib):
    s = IBMSolver(small_case(n=32, nsp=1, radius_cells=4.0, seed=1), mode=IBM_MODE_MIXED)
    s.setup()
    with pytest.raises(Exception):
        s.set_predictor_kernel(7)
    s.close()
