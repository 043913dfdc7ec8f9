"""Host-side logic: case generation, ghost conditions, the particle state
round trip through the oracle's C ABI, error codes."""
import numpy as np
import pytest

from interparts_mpich_gb300 import IBMError
from interparts_mpich_gb300.cases import (Case, bounduvw, channel_case, derived_nl, fibonacci_sphere,
                                          settling_case)
from oracle.oracle import OracleSolver


def test_channel_placement_gaps():
    c = channel_case(64, 12, seed=9)
    x = c.sphere_centres()
    R, D = c.radius, 2 * c.radius
    assert x.shape == (12, 3)
    assert np.all(x[:, 2] >= R + 0.1 * D - 1e-12) and np.all(x[:, 2] <= 1 - R - 0.1 * D + 1e-12)
    for i in range(len(x)):
        d = np.abs(x - x[i])
        d[:, 0] = np.minimum(d[:, 0], 1 - d[:, 0])
        d[:, 1] = np.minimum(d[:, 1], 1 - d[:, 1])
        r = np.sqrt((d ** 2).sum(1))
        r[i] = np.inf
        assert r.min() >= 1.1 * D - 1e-12


def test_channel_config_matches_benchmark():
    c = channel_case()
    assert (c.itot, c.jtot, c.ktot, c.np) == (256, 256, 256, 1000)
    assert c.nl == 746
    assert c.visc == pytest.approx(1 / 5600)
    vol_frac = c.np * 4 / 3 * np.pi * c.radius ** 3
    assert vol_frac == pytest.approx(0.128, abs=0.001)


def test_settling_config():
    c = settling_case(64)
    assert c.visc == pytest.approx(1.846e-3, rel=1e-3)
    assert c.nl == 746 and c.np == 1


def test_fibonacci_table():
    th, ph = fibonacci_sphere(746)
    assert th.shape == (746,) and np.all((th >= 0) & (th <= np.pi)) and np.all((ph >= 0) & (ph < 2 * np.pi))
    pts = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], 1)
    assert np.linalg.norm(pts.mean(0)) < 1e-2


def test_bounduvw_ghosts():
    c = Case(name="g", itot=8, jtot=8, ktot=8)
    f = c.initial_fields()
    u, v, w = f["u"], f["v"], f["w"]
    assert np.allclose(u[:, :, -1], -u[:, :, -2]) and np.allclose(v[:, :, 0], -v[:, :, 1])
    assert np.all(w[:, :, 0] == 0) and np.all(w[:, :, -2] == 0)
    assert np.array_equal(u[0], u[-2]) and np.array_equal(v[:, -1], v[:, 1])


def test_particle_state_roundtrip():
    c = Case(name="rt", itot=16, jtot=16, ktot=16, radius=3.0 / 16, np=2, seed=4)
    o = OracleSolver(c)
    o.setup()
    ps = o.get_particles()
    ps.u[:] = [0.1, -0.2]
    ps.intomz[:] = [3.0, 4.0]
    o.set_particles(ps)
    back = o.get_particles()
    for n in ("x", "u", "intomz", "xfp", "ul", "nb", "mslv", "qmax"):
        assert np.array_equal(getattr(back, n), getattr(ps, n)), n


def test_oracle_error_codes():
    c = Case(name="e", itot=16, jtot=16, ktot=16)
    o = OracleSolver(c)
    with pytest.raises(IBMError):
        o.rk(4, 1e-3)


def test_bench_kernel_model_covers_probe_classes():
    """Every kernel class the library times inside a step has an algorithmic model in the bench
    (bytes or flops per launch), and every recorded ncu traffic entry names a modelled class."""
    import bench
    from interparts_mpich_gb300.cases import channel_case
    from interparts_mpich_gb300.solver import IBMSolver
    case = channel_case()
    for w in (4, 8):
        model = bench.kernel_model(case, w)
        for name in IBMSolver.PROBE_NAMES:
            if name in ("phase", "stats"):  # post1d classes, timed by statistics_timing
                continue
            assert name in model, name
            bound, units = model[name]
            # the gated plain passes of the learned loop do no work unless the gate fell back
            assert bound in ("hbm", "tensor", "fp64") and (units > 0 or name == "gated")
    for form, name in bench.TRAFFIC:
        assert form in ("mixed", "learned", "plain") and name in bench.kernel_model(case, 4)
