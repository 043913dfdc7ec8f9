"""CUDA graphs of the RK stages: runs with the stages captured and replayed
give the same state as runs with every launch issued directly (to the
rounding the IBM spreading's atomic flush order leaves: the same run is not
bit-reproducible either), the same launch count, the same contact lists, and
the learned form the same calibration schedule."""
import numpy as np
import pytest

from _util import field_errors, small_case
from interparts_mpich_gb300 import IBM_MODE_MIXED, IBM_MODE_MIXED_LEARNED, IBM_MODE_PLAIN_FP64, IBMSolver

pytestmark = pytest.mark.gpu


def _case():
    return small_case(n=48, nsp=8, radius_cells=5.0, seed=21, visc=1.0 / 1000.0)


def _run(case, mode, graphs, nsteps, model=None):
    s = IBMSolver(case, mode=mode)
    s.setup()
    s.set_step_graphs(graphs)
    if model is not None:
        s.set_forcing_model(*model)
        # no fallbacks: a device decision near the threshold could differ between two runs at
        # rounding level; the calibration schedule (host-side) still runs both forcing kinds
        s.learned_config(enable=True, fallback_ratio=1e9)
    dt = 0.5 * s.chkdt()
    l0 = s.launch_count()
    s.run(dt, nsteps)  # a stage runs directly once, is captured the second time, replayed after
    launches = s.launch_count() - l0  # (reading the state back launches conversion kernels)
    out = {"fields": s.get_fields(), "particles": s.get_particles(), "launches": launches}
    if model is not None:
        out["learned"] = s.learned_stats()
        out["gate"] = s.learned_gate_state()
    s.close()
    return out


@pytest.mark.parametrize("mode,tol", [(IBM_MODE_PLAIN_FP64, 1e-12), (IBM_MODE_MIXED, 1e-5)])
def test_stage_graphs_match_direct_launches(gpu_lib, mode, tol):
    case = _case()
    direct = _run(case, mode, False, 6)
    graphed = _run(case, mode, True, 6)
    assert graphed["launches"] == direct["launches"] > 0
    errs = field_errors(graphed["fields"], direct["fields"], ("u", "v", "w", "p"))
    assert max(errs.values()) <= tol, errs
    pd, pg = direct["particles"], graphed["particles"]
    for name in ("x", "y", "z", "u", "v", "w"):
        a, b = getattr(pg, name), getattr(pd, name)
        assert np.linalg.norm(a - b) <= tol * max(np.linalg.norm(b), 1e-300), name
    assert pg.contact_lists() == pd.contact_lists()


def test_stage_graphs_learned_form(gpu_lib):
    case = _case()
    src = IBMSolver(case, mode=IBM_MODE_MIXED_LEARNED)
    src.setup()
    dt = 0.5 * src.chkdt()
    src.harvest(capacity=200000, stride=1, passes=3)
    src.run(dt, 3)
    src.harvest(0)
    src.train_forcing_model(nsteps=1500, batch=4096, lr=1e-3, seed=2, reinit=True)
    model = src.get_forcing_model()
    src.close()
    # 12 steps: learned and calibration loops at every stage (both graphs per stage)
    direct = _run(case, IBM_MODE_MIXED_LEARNED, False, 12, model)
    graphed = _run(case, IBM_MODE_MIXED_LEARNED, True, 12, model)
    assert graphed["launches"] == direct["launches"] > 0
    assert graphed["learned"]["learned_loops"] == direct["learned"]["learned_loops"]
    assert graphed["learned"]["fallbacks"] == direct["learned"]["fallbacks"] == 0
    assert graphed["gate"]["plain_loops"] == direct["gate"]["plain_loops"]
    assert direct["learned"]["learned_loops"] > 0 and direct["gate"]["plain_loops"] > 0
    errs = field_errors(graphed["fields"], direct["fields"], ("u", "v", "w"))
    assert max(errs.values()) <= 1e-4, errs


def test_prepared_stage_graphs_match_direct_launches(gpu_lib):
    """Stage graphs captured without launching (ibm_prepare_step_graphs)
    after one direct step, then replayed from the first later step."""
    case = _case()
    direct = _run(case, IBM_MODE_MIXED, False, 6)
    s = IBMSolver(case, mode=IBM_MODE_MIXED)
    s.setup()
    dt = 0.5 * s.chkdt()
    l0 = s.launch_count()
    s.run(dt, 1)
    l1 = s.launch_count()
    s.prepare_step_graphs(dt)
    assert s.launch_count() == l1  # capturing launches nothing
    s.run(dt, 5)
    assert s.launch_count() - l0 == direct["launches"]
    errs = field_errors(s.get_fields(), direct["fields"], ("u", "v", "w", "p"))
    assert max(errs.values()) <= 1e-5, errs
    assert s.get_particles().contact_lists() == direct["particles"].contact_lists()
    s.close()
