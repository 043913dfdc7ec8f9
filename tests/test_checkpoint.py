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
