"""Restart files in the reference formats (loadd.f90): byte layout and round
trips through the oracle (CPU)."""
import numpy as np

from interparts_mpich_gb300.cases import Case
from interparts_mpich_gb300.checkpoint import (read_allpartdata, read_fld, record_len, write_allpartdata,
                                               write_fld, written_len)
from oracle.oracle import OracleSolver


def test_fld_layout_and_roundtrip(tmp_path):
    c = Case(name="ck", itot=8, jtot=6, ktot=4)
    f = c.initial_fields()
    f["p"][1:-1, 1:-1, 1:-1] = np.arange(8 * 6 * 4).reshape(8, 6, 4, order="F")
    path = write_fld(tmp_path / "fld0000012", f, time=1.5, istep=12, dt=0.01)
    raw = np.fromfile(path, np.float64)
    n = 8 * 6 * 4
    assert raw.size == 5 * n + 3
    # p is the 4th block, Fortran order: element (i,j,k) at i + 8*(j + 6*k)
    assert raw[3 * n + 2 + 8 * (1 + 6 * 3)] == f["p"][3, 2, 4]
    assert np.all(raw[4 * n:5 * n] == 0.0)  # c = 0 (scalar inert)
    assert tuple(raw[-3:]) == (1.5, 12.0, 0.01)
    g, t, istep, dt = read_fld(path, 8, 6, 4)
    for k in "uvwp":
        assert np.array_equal(g[k][1:-1, 1:-1, 1:-1], f[k][1:-1, 1:-1, 1:-1])
    assert (t, istep, dt) == (1.5, 12, 0.01)


def test_allpartdata_stream(tmp_path):
    c = Case(name="ck", itot=16, jtot=16, ktot=16, radius=3.0 / 16, np=3, seed=2)
    o = OracleSolver(c)
    o.setup()
    o.run(1e-3, 1)
    ps = o.get_particles(lagrangian=False)
    ps.qmax[:] = [1, 0, 2]
    ps.firstc[:] = 0
    ps.firstc[0] = 2
    ps.firstc[2 * ps.nq: 2 * ps.nq + 2] = [5, 1]
    path = write_allpartdata(tmp_path / "allpartdata0000001", ps)
    raw = np.fromfile(path, np.float64)
    nq = ps.nq
    assert nq == 5 and raw.size == written_len(nq) * 3
    # the first record starts with x, y, z and its idp sits at 29 + 10*nq + 1
    assert raw[0] == ps.x[0] and raw[2] == ps.z[0]
    assert raw[29 + 10 * nq + 1] == 1.0 and raw[29 + 10 * nq + 2] == 2.0
    back = read_allpartdata(path, 3, nq)
    # records shift by 31+11nq in memory but only 29+11nq per particle are written
    assert record_len(nq) - written_len(nq) == 2
    assert np.array_equal(back.x[:2], ps.x[:2]) and np.array_equal(back.mslv[:2], [1, 2])
    assert back.contact_lists()[0] == [2]


def test_restart_roundtrip_oracle(tmp_path):
    """2 steps, fld/allpartdata written and read back into a fresh context
    (warm start), 2 more steps: identical to 4 uninterrupted steps.  Four
    spheres: the format's lost tail is then only the last particle's qmax,
    idp and firstc, which a particle without contacts does not use."""
    from interparts_mpich_gb300.checkpoint import load_restart, save_restart

    c = Case(name="rs", itot=32, jtot=32, ktot=32, radius=4.0 / 32, np=4, visc=1.0 / 500.0, seed=5)
    a = OracleSolver(c)
    a.setup()
    dt = 0.5 * a.chkdt()
    a.run(dt, 4)
    b = OracleSolver(c)
    b.setup()
    b.run(dt, 2)
    assert all(q == 0 for q in b.get_particles(lagrangian=False).qmax)
    save_restart(b, tmp_path, 2, 2 * dt, dt)
    r = OracleSolver(c)
    time, istep, dt_f = load_restart(r, tmp_path, 2)
    assert (istep, dt_f) == (2, dt)
    r.run(dt, 2)
    fa, fr = a.get_fields(), r.get_fields()
    for n in "uvwp":
        assert np.array_equal(fa[n][1:-1, 1:-1, 1:-1], fr[n][1:-1, 1:-1, 1:-1]), n
    pa, pr = a.get_particles(), r.get_particles()
    for n in ("x", "y", "z", "u", "v", "w", "omx", "intu", "intomz", "xfp", "ul"):
        assert np.array_equal(getattr(pa, n), getattr(pr, n)), n
