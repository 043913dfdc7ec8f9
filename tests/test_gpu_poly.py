"""Polydisperse spheres (ibm_params.radii): the plain FP64 path against the
oracle's generalised restatement, and the mixed form against the oracle.

The reference has one radius and one point count (param.f90:48,
init.f90:129), so this is a variant it cannot express.  Each sphere has its
own force-point count and shell, Lagrangian volume, volume and moment of
inertia; pairs touch at the sum of the radii, with the spring/dashpot of the
pair's effective mass and the lubrication of the equivalent radius
2 Rp Rq / (Rp + Rq).  Parity: contact lists identical and particles to 1e-10
over 12 steps of a collision case (unequal pairs across the periodic edges,
at both walls, nearly touching for lubrication), fields and particles to
1e-10 after 10 steps of a perturbed channel with six spheres of 6..12 dx,
the mixed form within 1e-4 there, and equal radii reproducing the
monodisperse run."""
import numpy as np
import pytest

from _util import PLAIN_TOL_10STEP, field_errors, particle_errors, rel_l2
from interparts_mpich_gb300 import IBM_MODE_MIXED, IBMSolver
from interparts_mpich_gb300.cases import Case
from oracle.oracle import OracleSolver

pytestmark = pytest.mark.gpu


def poly_collision_case():
    n = 48
    r = np.array([5.0, 3.5, 6.0, 4.0, 3.0, 5.5, 6.0, 4.5]) / n
    c = np.array([
        [0.30, 0.50, 0.50], [0.30 + (r[0] + r[1]) * 1.004, 0.50, 0.50],     # almost touching (lubrication)
        [0.05, 0.22, 0.40], [0.05 - (r[2] + r[3]) * 1.01 + 1.0, 0.22, 0.40],  # across x = 0
        [0.60, 0.99, 0.60], [0.60, 0.99 + (r[4] + r[5]) * 1.01 - 1.0, 0.60],  # across y = 0
        [0.75, 0.75, r[6] * 1.02],                                           # bottom wall
        [0.20, 0.80, 1.0 - r[7] * 1.05],                                     # top wall
    ])
    vel = np.array([[0.3, 0, 0], [-0.3, 0, 0], [-0.4, 0.1, 0], [0.4, -0.1, 0], [0, 0.3, 0], [0, -0.3, 0],
                    [0, 0, -0.5], [0, 0, 0.5]])
    return Case(name="pcollide", itot=n, jtot=n, ktot=n, radius=float(r.max()), np=len(c), visc=1.0 / 300.0,
                ratiorho=2.0, flow="pur", perturb=0.0, centres=c, velocities=vel, radii=r)


def poly_channel_case(radii=None):
    rng = np.random.default_rng(3)
    r = rng.uniform(3.0, 6.0, 6) / 48 if radii is None else radii
    return Case(name="pchannel", itot=48, jtot=48, ktot=48, radius=5.0 / 48, np=6, visc=1.0 / 800.0, seed=7,
                gap=0.02, ratiorho=1.5, flow="poi", perturb=0.05, radii=r)


def test_poly_collisions_contact_lists(gpu_lib):
    case = poly_collision_case()
    g, o = IBMSolver(case), OracleSolver(case)
    vg, vo = g.setup(), o.setup()
    assert abs(vg - vo) <= 1e-12 * abs(vo)
    pg0, po0 = g.get_particles(), o.get_particles()
    for n in ("intu", "intv", "intw"):
        assert np.max(np.abs(getattr(pg0, n) - getattr(po0, n))) <= 1e-12 * max(1.0, np.max(np.abs(getattr(po0, n))))
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
    g.close()
    o.close()


def test_poly_channel_10_steps(gpu_lib):
    case = poly_channel_case()
    g, o = IBMSolver(case), OracleSolver(case)
    g.setup()
    o.setup()
    dt = 0.5 * o.chkdt()
    g.run(dt, 10)
    o.run(dt, 10)
    fo, po = o.get_fields(), o.get_particles(lagrangian=False)
    e = field_errors(g.get_fields(), fo)
    pe = particle_errors(g.get_particles(lagrangian=False), po)
    print("\npolydisperse channel 48^3, 6 spheres of 6..12 dx, 10 steps vs oracle: "
          + ", ".join(f"{k} {v:.3e}" for k, v in {**e, **pe}.items()))
    assert max(e.values()) <= PLAIN_TOL_10STEP, e
    assert max(pe.values()) <= PLAIN_TOL_10STEP, pe
    m = IBMSolver(case, mode=IBM_MODE_MIXED)
    m.setup()
    m.run(dt, 10)
    em = field_errors(m.get_fields(), fo, names=("u", "v", "w"))
    pm = particle_errors(m.get_particles(lagrangian=False), po)
    print("mixed form: " + ", ".join(f"{k} {v:.3e}" for k, v in {**em, **pm}.items()))
    assert max(em.values()) <= 1e-4 and max(pm.values()) <= 1e-4, (em, pm)
    for s in (g, o, m):
        s.close()


def test_equal_radii_reproduce_monodisperse(gpu_lib):
    r = 5.0 / 48
    runs = []
    centres = poly_channel_case(radii=np.full(6, r)).sphere_centres()
    for radii in (None, np.full(6, r)):
        case = poly_channel_case(radii=np.full(6, r))
        case.radii = radii
        case.radius = r
        case.centres = centres
        g = IBMSolver(case)
        g.setup()
        dt = 0.5 * g.chkdt() if not runs else runs[0][2]
        g.run(dt, 5)
        runs.append((g.get_fields(), g.get_particles(lagrangian=False), dt))
        g.close()
    (fa, pa, _), (fb, pb, _) = runs
    e = field_errors(fb, fa)
    assert max(e.values()) <= 1e-12, e
    assert max(particle_errors(pb, pa).values()) <= 1e-12
    assert pa.contact_lists() == pb.contact_lists()


def test_poly_state_round_trip(gpu_lib):
    """Each sphere keeps its own point count when the state goes out through
    ibm_get_particles with the Lagrangian arrays and back in through
    ibm_set_particles (the arrays' capacity is the largest sphere's count)."""
    case = poly_channel_case()
    a, b = IBMSolver(case), IBMSolver(case)
    a.setup()
    b.setup()
    dt = 0.5 * a.chkdt()
    a.run(dt, 2)
    b.run(dt, 2)
    f, ps = b.get_fields(), b.get_particles(lagrangian=True)
    b.set_fields(f["u"], f["v"], f["w"], f["p"], f["durk"], f["dvrk"], f["dwrk"])
    b.set_particles(ps)
    a.run(dt, 2)
    b.run(dt, 2)
    e = field_errors(b.get_fields(), a.get_fields())
    assert max(e.values()) <= 1e-12, e
    assert max(particle_errors(b.get_particles(lagrangian=False), a.get_particles(lagrangian=False)).values()) <= 1e-12
    a.close()
    b.close()
