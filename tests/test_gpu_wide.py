"""The wide channel of the learned-forcing runs (512 x 512 x 256 on a
(2, 2, 1) box, 8000 spheres of D = 16 dx, 25.6 % volume fraction): the plain
FP64 path against the oracle over 2 RK3 steps at full size (the oracle takes
about a minute per step here), and the mixed form's deviation from the plain
GPU path after 10 steps."""
import os

import pytest

from _util import PLAIN_TOL_10STEP, field_errors, particle_errors
from interparts_mpich_gb300 import IBM_MODE_MIXED, IBMSolver
from interparts_mpich_gb300.cases import wide_channel_case
from oracle.oracle import OracleSolver, load

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def wide():
    return wide_channel_case(512, 256, 8000, seed=1234)


def test_plain_2_steps_wide(gpu_lib, wide):
    case = wide
    lib, _ = load()
    lib.orc_set_threads(os.cpu_count() or 1)
    o = OracleSolver(case)
    o.setup()
    dt = 0.5 * o.chkdt()
    o.run(dt, 2)
    fo, po = o.get_fields(), o.get_particles(lagrangian=False)
    o.close()
    g = IBMSolver(case)
    g.setup()
    g.run(dt, 2)
    e = field_errors(g.get_fields(), fo)
    pg = g.get_particles(lagrangian=False)
    pe = particle_errors(pg, po)
    print(f"\nplain FP64, wide channel 512x512x256, 8000 spheres, 2 steps vs oracle: "
          + ", ".join(f"{k} {v:.3e}" for k, v in {**e, **pe}.items()))
    assert max(e.values()) <= PLAIN_TOL_10STEP, e
    assert max(pe.values()) <= PLAIN_TOL_10STEP, pe
    assert pg.contact_lists() == po.contact_lists()
    g.close()


def test_mixed_10_steps_wide_vs_plain_gpu(gpu_lib, wide):
    case = wide
    g = IBMSolver(case)
    g.setup()
    dt = 0.5 * g.chkdt()
    m = IBMSolver(case, mode=IBM_MODE_MIXED)
    m.setup()
    g.run(dt, 10)
    m.run(dt, 10)
    e = field_errors(m.get_fields(), g.get_fields())
    e.update(particle_errors(m.get_particles(lagrangian=False), g.get_particles(lagrangian=False)))
    print("\nmixed vs plain FP64 GPU, wide channel, 10 steps: " + ", ".join(f"{k} {v:.3e}" for k, v in e.items()))
    assert max(e[n] for n in "uvw") <= 1e-4, e
    g.close()
    m.close()
