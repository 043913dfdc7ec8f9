"""Plane statistics on the GPU (ibm_phase_indicator, ibm_post1d) against the
oracle's restatement of phase_indicator.f90:11-559 and output.f90:13-917.

The phase fields must be bit-identical (same corner arithmetic, and the
reference's order of overwrites recovered exactly); the plane profiles
differ only by the order of the FP64 plane sums."""
import numpy as np
import pytest

from _util import small_case
from interparts_mpich_gb300 import IBM_MODE_MIXED, IBM_MODE_PLAIN_FP64, IBMSolver
from oracle.oracle import OracleSolver

pytestmark = pytest.mark.gpu

# relative to the largest |value| of each profile (sums of ~1e3..1e4 terms in
# another order; the rms subtracts a squared mean from a mean square)
PROFILE_TOL = 1e-10


def _case():
    # spheres across the periodic x and y boundaries and one overlapping pair,
    # which exercises the reference's order of overwrites
    centres = np.array([[0.03, 0.5, 0.5], [0.5, 0.02, 0.4], [0.97, 0.98, 0.6], [0.4, 0.4, 0.3],
                        [0.4 + 0.15, 0.4, 0.3], [0.7, 0.7, 0.75], [0.2, 0.8, 0.2]])
    return small_case(n=48, nsp=len(centres), radius_cells=5.0, seed=5, centres=centres, rotation=1)


def _pair(mode):
    case = _case()
    rng = np.random.default_rng(2)
    ps = case.initial_particles(lagrangian=False)
    for f in ("u", "v", "w", "omx", "omy", "omz"):
        getattr(ps, f)[:] = rng.uniform(-0.5, 0.5, case.np)
    g = IBMSolver(case, mode=mode)
    g.setup(particles=ps)
    o = OracleSolver(case)
    o.setup(particles=ps)
    c = np.asfortranarray(rng.uniform(0.0, 1.0, case.shape))
    for s in (g, o):
        s.set_scalar(c, pran=0.71, bc_c_top_val=0.0, bc_c_bot_val=1.0)
    return g, o, case


@pytest.mark.parametrize("itype", [1, 0])
def test_phase_indicator_bit_identical(gpu_lib, itype):
    g, o, _ = _pair(IBM_MODE_PLAIN_FP64)
    pg, po = g.phase_indicator(itype), o.phase_indicator(itype)
    for name in pg:
        a, b = pg[name], po[name]
        bad = np.argwhere(a != b)
        assert bad.size == 0, (name, len(bad), bad[:3], a[tuple(bad[0])], b[tuple(bad[0])])
    assert (pg["gamp"] < 1).sum() > 1000


def _compare_profiles(pa, pb, sa, sb):
    # divisions by an empty solid phase (N - gum = 0 in planes without
    # particles) give the same inf/nan on both sides; finite values agree to
    # the summation order
    for name in pa:
        a, b = pa[name], pb[name]
        fin = np.isfinite(b)
        assert np.array_equal(np.isfinite(a), fin), name
        assert np.array_equal(a[~fin], b[~fin], equal_nan=True), name
        scale = max(np.abs(b[fin]).max() if fin.any() else 0.0, 1e-300)
        err = np.abs(a[fin] - b[fin]).max() if fin.any() else 0.0
        assert err <= PROFILE_TOL * scale, (name, err, scale)
    for name in sa:
        a, b = sa[name], sb[name]
        if not np.isfinite(b):
            assert a == b or (np.isnan(a) and np.isnan(b)), (name, a, b)
        else:
            assert abs(a - b) <= PROFILE_TOL * max(abs(b), 1e-300), (name, a, b)


@pytest.mark.parametrize("mode", [IBM_MODE_PLAIN_FP64, IBM_MODE_MIXED])
def test_post1d_matches_oracle(gpu_lib, mode):
    g, o, _ = _pair(mode)
    # the oracle evaluates the statistics of the GPU's state (in the mixed
    # form: the FP32 velocities and the double-float pressure)
    f = g.get_fields()
    o.set_fields(f["u"], f["v"], f["w"], f["p"])
    o.set_particles(g.get_particles())
    pa, sa = g.post1d()
    pb, sb = o.post1d()
    _compare_profiles(pa, pb, sa, sb)
    assert np.isfinite(pa["um"][1:-1]).all() and pa["gum"][1:-1].min() > 0


def test_post1d_without_particles(gpu_lib):
    case = small_case(n=32, nsp=0, seed=9)
    g = IBMSolver(case)
    g.setup()
    o = OracleSolver(case)
    o.setup()
    pa, sa = g.post1d()
    pb, sb = o.post1d()
    _compare_profiles(pa, pb, sa, sb)
    assert np.all(pa["gum"] == 0.0)
