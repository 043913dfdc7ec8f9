"""Parity of the plain FP64 CUDA path against the CPU oracle (restatement of
the reference, single rank), through the C ABI.

Sizes are chosen so the oracle finishes in seconds; the full 256^3 / 1000
sphere channel is covered by test_gpu_fullsize.py.
"""
import numpy as np
import pytest

from _util import (PLAIN_TOL_10STEP, PLAIN_TOL_CALL, field_errors, interior, particle_errors, rel_l2,
                   small_case)
from interparts_mpich_gb300 import IBMSolver
from interparts_mpich_gb300.cases import Case, channel_case
from oracle.oracle import OracleSolver

pytestmark = pytest.mark.gpu


def pair(case, gpu_lib):
    g = IBMSolver(case)
    o = OracleSolver(case)
    vg = g.setup()
    vo = o.setup()
    return g, o, vg, vo


def test_init_particles(gpu_lib):
    case = small_case()
    g, o, vg, vo = pair(case, gpu_lib)
    assert abs(vg - vo) <= 1e-12 * abs(vo)
    pg, po = g.get_particles(), o.get_particles()
    assert np.array_equal(pg.nb, po.nb)
    for n in ("intu", "intv", "intw", "intomx", "intomy", "intomz"):
        assert rel_l2(getattr(pg, n), getattr(po, n)) < 1e-12 or np.max(np.abs(getattr(pg, n) - getattr(po, n))) < 1e-16
    assert np.array_equal(pg.xfp, po.xfp) and np.array_equal(pg.zfp, po.zfp)


def test_substep_phases(gpu_lib):
    """Each reference subroutine block separately, one substep of every RK stage."""
    case = small_case()
    g, o, _, _ = pair(case, gpu_lib)
    dt = 0.5 * o.chkdt()
    assert abs(g.chkdt() - o.chkdt()) <= 1e-14 * o.chkdt()
    for rkiter in (1, 2, 3):
        g.rk(rkiter, dt); o.rk(rkiter, dt)
        ig, io = g.get_intermediate(), o.get_intermediate()
        for n in ("dudt", "dvdt", "dwdt"):
            assert rel_l2(interior(ig[n]), interior(io[n])) < PLAIN_TOL_CALL, (rkiter, "predict", n)
        g.forcing_loop(dt); o.forcing_loop(dt)
        ig, io = g.get_intermediate(), o.get_intermediate()
        for n in ("dudt", "dvdt"):
            assert rel_l2(interior(ig[n]), interior(io[n])) < PLAIN_TOL_CALL, (rkiter, "ibm", n)
        # w(kmax) is overwritten by the wall condition afterwards; compare below it
        assert rel_l2(ig["dwdt"][1:-1, 1:-1, 1:-2], io["dwdt"][1:-1, 1:-1, 1:-2]) < PLAIN_TOL_CALL
        pg, po = g.get_particles(), o.get_particles()
        assert rel_l2(pg.fxl, po.fxl) < PLAIN_TOL_CALL
        assert rel_l2(pg.fzltot, po.fzltot) < PLAIN_TOL_CALL
        g.project(rkiter, dt); o.project(rkiter, dt)
        fg, fo = g.get_fields(), o.get_fields()
        e = field_errors(fg, fo)
        assert max(e.values()) < PLAIN_TOL_CALL, (rkiter, "project", e)
        # ghost layers as bounduvw/boundp leave them
        for n in ("u", "v", "p"):
            assert rel_l2(fg[n][:, :, [0, -1]], fo[n][:, :, [0, -1]]) < PLAIN_TOL_CALL
        g.intgr_nwtn_eulr(rkiter, dt); o.intgr_nwtn_eulr(rkiter, dt)
        pg, po = g.get_particles(), o.get_particles()
        e = particle_errors(pg, po)
        assert max(e.values()) < PLAIN_TOL_CALL, (rkiter, "newton_euler", e)
        assert np.array_equal(pg.nb, po.nb)
        assert pg.contact_lists() == po.contact_lists()
        assert rel_l2(pg.rkp, po.rkp) < 1e-11


def test_ten_steps_channel(gpu_lib):
    """10 RK3 steps of a channel with spheres: rel L2 <= 1e-10, same chkdiv max,
    identical contact lists."""
    case = small_case(n=48, nsp=10, radius_cells=5.0, seed=11, visc=1.0 / 1000.0)
    g, o, _, _ = pair(case, gpu_lib)
    dt = 0.5 * o.chkdt()
    g.run(dt, 10)
    o.run(dt, 10)
    fg, fo = g.get_fields(), o.get_fields()
    e = field_errors(fg, fo)
    assert max(e.values()) <= PLAIN_TOL_10STEP, e
    pg, po = g.get_particles(), o.get_particles()
    pe = particle_errors(pg, po)
    assert max(pe.values()) <= PLAIN_TOL_10STEP, pe
    assert pg.contact_lists() == po.contact_lists()
    _, mg, _ = g.chkdiv()
    _, mo, _ = o.chkdiv()
    assert abs(mg - mo) <= 1e-12


def collision_case(nb_copies=9):
    """Spheres placed to collide with each other, across the periodic edges and
    with both walls, with approach velocities."""
    n = 48
    R = 5.0 / n
    c = np.array([
        [0.30, 0.50, 0.50], [0.30 + 2 * R * 1.004, 0.50, 0.50],         # almost touching (lubrication)
        [0.05, 0.22, 0.40], [0.05 - 2 * R * 1.01 + 1.0, 0.22, 0.40],    # across x = 0
        [0.60, 0.99, 0.60], [0.60, 0.99 + 2 * R * 1.01 - 1.0, 0.60],    # across y = 0
        [0.75, 0.75, R * 1.02],                                         # bottom wall
        [0.20, 0.80, 1.0 - R * 1.05],                                   # top wall
    ])
    vel = np.array([
        [0.3, 0, 0], [-0.3, 0, 0],
        [-0.4, 0.1, 0], [0.4, -0.1, 0],
        [0, 0.3, 0], [0, -0.3, 0],
        [0, 0, -0.5], [0, 0, 0.5],
    ])
    return Case(name="collide", itot=n, jtot=n, ktot=n, radius=R, np=len(c), visc=1.0 / 300.0,
                ratiorho=2.0, flow="pur", perturb=0.0, centres=c, velocities=vel, nb_copies=nb_copies)


@pytest.mark.parametrize("nb_copies", [9, 1])
def test_collisions_contact_lists(gpu_lib, nb_copies):
    case = collision_case(nb_copies)
    g, o, _, _ = pair(case, gpu_lib)
    dt = 2e-3
    seen = 0
    for step in range(12):
        g.rk3_step(dt)
        o.rk3_step(dt)
        pg, po = g.get_particles(), o.get_particles()
        assert pg.contact_lists() == po.contact_lists(), step
        seen += sum(len(c) for c in po.contact_lists())
        e = particle_errors(pg, po)
        assert max(e.values()) < 1e-10, (step, e)
        assert rel_l2(pg.colfz, po.colfz) < 1e-9 or np.max(np.abs(pg.colfz - po.colfz)) < 1e-12
    assert seen > 0, "the case never produced a contact"


def test_projection_divergence_free(gpu_lib):
    """After the projection the velocity is divergence free to round-off
    (chkdiv, chkdiv.f90:7-61)."""
    case = small_case(n=64, nsp=0)
    g = IBMSolver(case)
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
    assert mx < 1e-10 and abs(tot) < 1e-9, (tot, mx)


def test_settling_sphere(gpu_lib):
    """The single settling sphere (free-slip walls) for a few steps."""
    from interparts_mpich_gb300.cases import settling_case
    case = settling_case(32, periodic=False)
    g, o, vg, vo = pair(case, gpu_lib)
    dt = 1e-3
    g.run(dt, 5)
    o.run(dt, 5)
    pg, po = g.get_particles(), o.get_particles()
    assert abs(pg.w[0] - po.w[0]) <= 1e-10 * max(abs(po.w[0]), 1e-30)
    assert pg.w[0] < 0  # it falls
    e = field_errors(g.get_fields(), o.get_fields())
    assert max(e.values()) < 1e-10, e


def test_adaptive_time_step_control_matches_oracle(gpu_lib):
    """main.f90:425-441 on the device: every ioutchk steps chkdt sets
    dt = 0.75 dtmax; same dt sequence and fields as the oracle's loop."""
    case = small_case(n=32, nsp=4, seed=21)
    g = IBMSolver(case)
    o = OracleSolver(case)
    g.setup()
    o.setup()
    dt0 = 0.5 * o.chkdt()
    dg, tg = g.run_adaptive(6, 2, dt0)
    do, to = o.run_adaptive(6, 2, dt0)
    assert abs(dg - do) <= 1e-12 * do and abs(tg - to) <= 1e-12 * to
    assert dg != dt0
    e = field_errors(g.get_fields(), o.get_fields())
    assert max(e.values()) <= PLAIN_TOL_10STEP, e
