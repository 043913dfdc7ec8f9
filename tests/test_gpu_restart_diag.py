"""Restart through the reference's file formats on the device state, and the
updtintermediatevel / wall-shear diagnostics against the oracle.

Restart: ibm_get_fields / ibm_get_particles -> fld / allpartdata
(loadd.f90) -> read back -> ibm_set_fields / ibm_set_particles of a fresh
context (the warm start of main.f90:155-201: no sphere integrals, neighbour
flags from the centres) -> continue.  The continued run equals the
uninterrupted one up to the order of the spreading's atomic adds, which
differs between any two runs: within 1e-12 relative L2 (plain FP64) or 1e-5
(mixed, FP32 state), printed beside the difference of two uninterrupted
runs.  The oracle's restart is bit-identical (tests/test_checkpoint.py)."""
import numpy as np
import pytest

from _util import rel_l2, small_case
from interparts_mpich_gb300 import IBM_MODE_MIXED, IBM_MODE_PLAIN_FP64, IBMSolver
from interparts_mpich_gb300.cases import Case
from interparts_mpich_gb300.checkpoint import load_restart, save_restart
from oracle.oracle import OracleSolver

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [IBM_MODE_PLAIN_FP64, IBM_MODE_MIXED])
def test_restart_roundtrip_gpu(gpu_lib, tmp_path, mode):
    tol = 1e-12 if mode == IBM_MODE_PLAIN_FP64 else 1e-5
    c = Case(name="rs", itot=32, jtot=32, ktot=32, radius=4.0 / 32, np=4, visc=1.0 / 500.0, seed=5)
    a = IBMSolver(c, mode=mode)
    a.setup()
    dt = 0.5 * a.chkdt()
    a.run(dt, 4)
    a2 = IBMSolver(c, mode=mode)
    a2.setup()
    a2.run(dt, 4)
    b = IBMSolver(c, mode=mode)
    b.setup()
    b.run(dt, 2)
    assert all(q == 0 for q in b.get_particles(lagrangian=False).qmax)
    save_restart(b, tmp_path, 2, 2 * dt, dt)
    r = IBMSolver(c, mode=mode)
    _, istep, _ = load_restart(r, tmp_path, 2)
    assert istep == 2
    r.run(dt, 2)
    fa, fr, f2 = a.get_fields(), r.get_fields(), a2.get_fields()
    pa, pr, p2 = a.get_particles(), r.get_particles(), a2.get_particles()
    d_rs = {n: rel_l2(fr[n][1:-1, 1:-1, 1:-1], fa[n][1:-1, 1:-1, 1:-1]) for n in "uvwp"}
    d_rr = {n: rel_l2(f2[n][1:-1, 1:-1, 1:-1], fa[n][1:-1, 1:-1, 1:-1]) for n in "uvwp"}
    for n in ("x", "y", "z", "u", "v", "w", "intu", "xfp", "ul"):
        d_rs["p." + n] = rel_l2(getattr(pr, n), getattr(pa, n))
        d_rr["p." + n] = rel_l2(getattr(p2, n), getattr(pa, n))
    print(f"\nmode {mode}: restarted vs uninterrupted, max rel L2 {max(d_rs.values()):.2e}; "
          f"two uninterrupted runs {max(d_rr.values()):.2e}")
    assert max(d_rs.values()) <= tol, d_rs
    assert pa.contact_lists() == pr.contact_lists()
    for s in (a, a2, b, r):
        s.close()


def test_diagnostics_match_oracle(gpu_lib):
    """wallshearnew / wallshearold of rk3 (rk3.f90:88-103, 208-217,
    318-325) after a full step, and the total IBM force of the last forcing
    pass (updtintermediatevel's particle sums, forcing.f90:393-513)."""
    case = small_case(n=32, nsp=6, seed=3)
    g = IBMSolver(case)
    o = OracleSolver(case)
    g.setup()
    o.setup()
    dt = 0.5 * o.chkdt()
    for _ in range(3):
        g.rk3_step(dt)
        o.rk3_step(dt)
        dg, do = g.diagnostics(), o.diagnostics()
        for k in ("wallshearnew", "wallshearold"):
            assert abs(dg[k] - do[k]) <= 1e-10 * abs(do[k]), (k, dg[k], do[k])
        assert rel_l2(np.array(dg["forcetot"]), np.array(do["forcetot"])) <= 1e-10, (dg, do)
        assert abs(do["wallshearnew"]) > 0 and np.abs(do["forcetot"]).max() > 0
    g.close()
    o.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_fields_through_page_locked_buffers(gpu_lib, mode):
    """Page-locked host arrays are read and written by the layout-conversion
    kernels directly (mapped into the device's address space); pageable arrays
    go through the staging buffer.  Both give the same fields, both ways."""
    torch = pytest.importorskip("torch")
    from interparts_mpich_gb300 import IBMSolver
    from interparts_mpich_gb300.cases import Case
    case = Case(name="pin", itot=32, jtot=32, ktot=32, radius=4.0 / 32, np=2, visc=1.0 / 500.0, seed=3)
    s = IBMSolver(case, mode=mode)
    s.setup()
    dt = 0.5 * s.chkdt()
    s.run(dt, 2)
    pageable = s.get_fields()
    pin = {k: torch.empty(case.shape[::-1], dtype=torch.float64, pin_memory=True).numpy().T
           for k in ("u", "v", "w", "p", "durk", "dvrk", "dwrk")}
    s.get_fields(out=pin)
    for k in pin:
        assert np.array_equal(pin[k], pageable[k]), k
    # upload from the page-locked copies, download again (pageable)
    s.set_fields(pin["u"], pin["v"], pin["w"], pin["p"], pin["durk"], pin["dvrk"], pin["dwrk"])
    again = s.get_fields()
    for k in pin:
        assert np.array_equal(again[k], pageable[k]), k
    s.close()
