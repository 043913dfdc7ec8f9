"""Pins of the oracle's phase indicator and plane statistics (post1d) by
known answers (the reference ships no output for them):

* the solid volume of the phase indicator against the sphere volume, the
  check the reference keeps in phase_indicator.f90:533-548;
* periodic-shift invariance of the fractions (a sphere moved by whole cells
  across the periodic boundary, exact on dyadic coordinates);
* the rigid-body velocity of the occupied cells, and the zero velocity of
  the self-neighbour copies (anb(1:8) carry positions only,
  phase_indicator.f90:68-78, 83-87);
* single-phase profiles of fields with known plane means and rms;
* the conductive Nusselt number 1 of a linear scalar profile.
"""
import math

import numpy as np
import pytest

from interparts_mpich_gb300.cases import Case
from oracle.oracle import OracleSolver


def _solver(n=32, centres=None, radius_cells=4.0, vel=None, om=None, flow="pur"):
    nsp = 0 if centres is None else len(centres)
    case = Case(name="stats", itot=n, jtot=n, ktot=n, radius=radius_cells / n, np=nsp, visc=1e-3,
                flow=flow, perturb=0.0, centres=None if centres is None else np.asarray(centres, float))
    s = OracleSolver(case)
    ps = case.initial_particles(lagrangian=False)
    if vel is not None:
        ps.u[:], ps.v[:], ps.w[:] = np.asarray(vel, float).T
    if om is not None:
        ps.omx[:], ps.omy[:], ps.omz[:] = np.asarray(om, float).T
    s.setup(particles=ps)
    return s, case


def test_solid_volume_matches_spheres():
    s, case = _solver(n=48, centres=[[0.3, 0.4, 0.5], [0.7, 0.6, 0.3], [0.02, 0.5, 0.6]], radius_cells=5.0)
    ph = s.phase_indicator(1)
    dv = 1.0 / 48 ** 3
    volp = case.np * 4.0 / 3.0 * math.pi * case.radius ** 3
    for n in ("gamu", "gamv", "gamw", "gamp"):
        vol = (1.0 - ph[n][1:-1, 1:-1, 1:-1]).sum() * dv
        assert abs(vol - volp) < 0.03 * volp, (n, vol, volp)
        # fractions in [0, 1], fluid far away
        assert ph[n].min() >= 0.0 and ph[n].max() <= 1.0


def test_fractions_invariant_under_periodic_shift():
    """The same sphere moved by (+20, -14) cells so that its box crosses the
    x and y boundaries: the fractions are the rolled ones, bit for bit
    (dyadic coordinates keep every difference and square exact)."""
    n = 32
    x0, y0, z0 = 0.5 + 1 / 64, 0.5 + 3 / 64, 0.5 + 1 / 128
    a, _ = _solver(n, centres=[[x0, y0, z0]])
    b, _ = _solver(n, centres=[[x0 + 20 / n - 1.0, y0 - 14 / n, z0]])
    pa, pb = a.phase_indicator(1), b.phase_indicator(1)
    for name in ("gamu", "gamv", "gamw", "gamp"):
        ra = np.roll(pa[name][1:-1, 1:-1, 1:-1], (20, -14), axis=(0, 1))
        assert np.array_equal(ra, pb[name][1:-1, 1:-1, 1:-1]), name
        assert (pb[name][1:-1, 1:-1, 1:-1] < 1).sum() > 100


def test_rigid_body_velocity_and_copies():
    n = 32
    dx = 1.0 / n
    # sphere centred near x = 0: part of it is covered through the copy nb=5 -> 1
    s, case = _solver(n, centres=[[2 * dx, 0.5, 0.5]], vel=[[0.3, -0.2, 0.1]], om=[[0.5, 1.5, -2.0]])
    ph = s.phase_indicator(1)
    u0, v0, w0 = 0.3, -0.2, 0.1
    omx, omy, omz = 0.5, 1.5, -2.0
    x, y, z = 2 * dx, 0.5, 0.5
    solid = ph["gamu"] < 1.0
    i, j, k = np.nonzero(solid[1:-1, 1:-1, 1:-1])
    i, j, k = i + 1, j + 1, k + 1
    own = i < n // 2          # cells of the particle itself
    ref = u0 + omy * ((k - 0.5) * dx - z) - omz * ((j - 0.5) * dx - y)
    up = ph["upart"][i, j, k]
    assert np.allclose(up[own], ref[own], rtol=0, atol=1e-14)
    assert own.sum() > 0 and (~own).sum() > 0
    assert np.all(up[~own] == 0.0)   # cells won by the shifted copy
    # pressure cells, itype 0: angular velocity
    ph0 = s.phase_indicator(0)
    sp = ph0["gamp"][1:-1, 1:-1, 1:-1] < 1.0
    ii, jj, kk = np.nonzero(sp)
    own0 = ii + 1 < n // 2
    assert np.all(ph0["upart"][1:-1, 1:-1, 1:-1][sp][own0] == omx)
    assert np.all(ph0["wpart"][1:-1, 1:-1, 1:-1][sp][own0] == omz)
    assert np.all(ph0["gamu"] == 1.0)  # itype 0 leaves the velocity cells fluid


def test_single_phase_profiles():
    n = 24
    s, case = _solver(n)
    shp = case.shape
    k = np.arange(shp[2], dtype=float)
    a = 0.1 + 0.01 * k
    b = 0.05 + 0.002 * k
    sign = np.fromfunction(lambda i, j, kk: (-1.0) ** (i + j), shp)
    u = np.asfortranarray(a[None, None, :] + b[None, None, :] * sign)
    v = np.asfortranarray(2 * a[None, None, :] - b[None, None, :] * sign)
    w = np.zeros(shp, order="F")
    p = np.asfortranarray(np.broadcast_to(3 * a[None, None, :], shp).copy())
    s.set_fields(u, v, w, p)
    prof, _ = s.post1d()
    ks = slice(1, n + 1)
    assert np.allclose(prof["um"][ks], a[ks], rtol=1e-12)
    assert np.allclose(prof["vm"][ks], 2 * a[ks], rtol=1e-12)
    assert np.allclose(prof["u2"][ks], b[ks], rtol=1e-9)
    assert np.allclose(prof["v2"][ks], b[ks], rtol=1e-9)
    assert np.allclose(prof["pm"][ks], 3 * a[ks], rtol=1e-12)
    # ghost planes of the means (output.f90:194-199, 460-465)
    assert prof["um"][0] == -prof["um"][1] and prof["vm"][n + 1] == -prof["vm"][n]


@pytest.mark.parametrize("cb,ct", [(1.0, 0.0), (0.5, -0.25)])
def test_conduction_nusselt_is_one(cb, ct):
    n = 16
    s, case = _solver(n)
    shp = case.shape
    z = (np.arange(shp[2]) - 0.5) / n
    c = np.asfortranarray(np.broadcast_to((cb + (ct - cb) * z)[None, None, :], shp).copy())
    s.set_scalar(c, pran=0.7, bc_c_top_val=ct, bc_c_bot_val=cb)
    _, sc = s.post1d()
    assert abs(sc["nu"] - 1.0) < 1e-12, sc["nu"]
