"""Restart files in the reference's formats (loadd.f90), host side.

fld<istep:7d> (loadflds, loadd.f90:12-68): u, v, w, p, c written by
2DECOMP's decomp_2d_write_var as global interior arrays itot*jtot*ktot in
Fortran order, FP64, native byte order, one after the other, followed by the
scalars (time, istep, dt) (decomp_2d_write_scalar, io.f90:276-301).

allpartdata<istep:7d> (loadpart, loadd.f90:121-694): one record per master
particle of the type particle_restart,
  x y z theta phi u v w omx omy omz omtheta intu intv intw intomx intomy intomz
  flag1 flag2 colfx colfy colfz coltx colty coltz fxltot fyltot fzltot   (29)
  dx dy dz dxt dyt dzt dut dvt dwt psi                                   (10*nqmax)
  qmax idp                                                               (2)
  firstc                                                                 (nqmax)
i.e. 31 + 11*nqmax doubles in memory, but the writer streams only
skip*npmstr doubles with skip = 27 + 10*nqmax + 2 + nqmax = 29 + 11*nqmax
(loadd.f90:143-144, 679-686).  The file therefore holds the first
(29 + 11*nqmax)*np doubles of the record array: the last 2*np doubles of the
records are not written, and a reader that loads the stream back into the
record array (as loadpart does, loadd.f90:195) keeps whatever that memory
held.  Both functions below reproduce that byte stream; the reader returns
the truncated tail as NaN, or with fill_tail as a zero-initialised record
array on one rank leaves it (0, with the particle id idp = index + 1).  For
np <= 4 the tail is only the last particle's qmax, idp and firstc, so a
particle without contacts restarts exactly; larger np lose data of the last
particles in the reference's own format.  The writer fills flag1/flag2 with 0 and
dut..psi with the values given (the reference leaves them unset).
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from ._abi import ParticleState

FLD_FIELDS = ("u", "v", "w", "p", "c")
PART_SCALARS = ["x", "y", "z", "theta", "phi", "u", "v", "w", "omx", "omy", "omz", "omtheta",
                "intu", "intv", "intw", "intomx", "intomy", "intomz", "flag1", "flag2",
                "colfx", "colfy", "colfz", "coltx", "colty", "coltz", "fxltot", "fyltot", "fzltot"]
PART_CONTACT = ["cdx", "cdy", "cdz", "cdxt", "cdyt", "cdzt", "cdut", "cdvt", "cdwt", "cpsi"]


def fld_name(istep: int) -> str:
    return f"fld{istep:07d}"


def allpartdata_name(istep: int) -> str:
    return f"allpartdata{istep:07d}"


def write_fld(path: str | Path, fields: dict, time: float, istep: int, dt: float) -> Path:
    """fields: arrays in the reference layout (0:i1,0:j1,0:k1); c may be absent (zero)."""
    p = Path(path)
    u = fields["u"]
    interior = tuple(slice(1, n - 1) for n in u.shape)
    with open(p, "wb") as f:
        for name in FLD_FIELDS:
            a = fields.get(name)
            block = np.zeros([n - 2 for n in u.shape]) if a is None else np.asarray(a, np.float64)[interior]
            f.write(np.asfortranarray(block).tobytes(order="F"))
        f.write(np.array([time, float(istep), dt], np.float64).tobytes())
    return p


def read_fld(path: str | Path, itot: int, jtot: int, ktot: int) -> tuple[dict, float, int, float]:
    """Returns interior-filled reference-layout arrays (ghosts zero), time, istep, dt."""
    raw = np.fromfile(path, dtype=np.float64)
    n = itot * jtot * ktot
    if raw.size != 5 * n + 3:
        raise ValueError(f"{path}: {raw.size} doubles, expected {5 * n + 3} for {itot}x{jtot}x{ktot}")
    out = {}
    for q, name in enumerate(FLD_FIELDS):
        a = np.zeros((itot + 2, jtot + 2, ktot + 2), order="F")
        a[1:-1, 1:-1, 1:-1] = raw[q * n:(q + 1) * n].reshape((itot, jtot, ktot), order="F")
        out[name] = a
    time, istep, dt = raw[5 * n:]
    return out, float(time), int(istep), float(dt)


def record_len(nq: int) -> int:
    return 31 + 11 * nq


def written_len(nq: int) -> int:
    return 29 + 11 * nq  # skip = skipr + skipi (loadd.f90:143-144)


def pack_records(ps: ParticleState) -> np.ndarray:
    nq = ps.nq
    rec = np.zeros((ps.np, record_len(nq)))
    for q, name in enumerate(PART_SCALARS):
        if name in ("flag1", "flag2"):
            continue
        rec[:, q] = getattr(ps, name)
    base = len(PART_SCALARS)
    for q, name in enumerate(PART_CONTACT):
        rec[:, base + q * nq: base + (q + 1) * nq] = getattr(ps, name).reshape(ps.np, nq)
    base += 10 * nq
    rec[:, base] = ps.qmax
    rec[:, base + 1] = ps.mslv
    rec[:, base + 2: base + 2 + nq] = ps.firstc.reshape(ps.np, nq)
    return rec


def write_allpartdata(path: str | Path, ps: ParticleState) -> Path:
    rec = pack_records(ps)
    stream = rec.ravel()[: written_len(ps.nq) * ps.np]
    p = Path(path)
    stream.tofile(p)
    return p


def read_allpartdata(path: str | Path, np_: int, nq: int, nl: int = 0, fill_tail: bool = False) -> ParticleState:
    raw = np.fromfile(path, dtype=np.float64)
    if raw.size != written_len(nq) * np_:
        raise ValueError(f"{path}: {raw.size} doubles, expected {written_len(nq) * np_}")
    full = np.full(record_len(nq) * np_, 0.0 if fill_tail else np.nan)
    full[: raw.size] = raw
    rec = full.reshape(np_, record_len(nq))
    if fill_tail:  # the id slot of every record whose idp was not written
        idp_col = len(PART_SCALARS) + 10 * nq + 1
        lost = np.arange(np_) * record_len(nq) + idp_col >= raw.size
        rec[lost, idp_col] = np.arange(1, np_ + 1)[lost]
    ps = ParticleState(np_, nq, nl, lagrangian=False)
    for q, name in enumerate(PART_SCALARS):
        if name in ("flag1", "flag2"):
            continue
        setattr(ps, name, rec[:, q].copy())
    base = len(PART_SCALARS)
    for q, name in enumerate(PART_CONTACT):
        setattr(ps, name, rec[:, base + q * nq: base + (q + 1) * nq].ravel().copy())
    base += 10 * nq
    qm = rec[:, base]
    idp = rec[:, base + 1]
    fc = rec[:, base + 2: base + 2 + nq]
    ps.qmax = np.where(np.isnan(qm), -1, qm).astype(np.int32)
    ps.mslv = np.where(np.isnan(idp), -1, idp).astype(np.int32)
    ps.firstc = np.where(np.isnan(fc), -1, fc).astype(np.int32).ravel()
    return ps


def save_restart(solver, directory: str | Path, istep: int, time: float, dt: float) -> tuple[Path, Path]:
    """loadd(1, istep) of the driver (main.f90:495-506): fld<istep> and
    allpartdata<istep> of the solver's current state in `directory`."""
    d = Path(directory)
    f = solver.get_fields()
    pf = write_fld(d / fld_name(istep), f, time, istep, dt)
    pp = d / allpartdata_name(istep)
    if solver.case.np > 0:
        write_allpartdata(pp, solver.get_particles(lagrangian=False))
    return pf, pp


def load_restart(solver, directory: str | Path, istep: int) -> tuple[float, int, float]:
    """Warm start of program interpt (main.f90:155-201) into a fresh solver:
    loadpart and loadflds, the boundary conditions, then coordsfp (the
    Lagrangian points from the centres) without intgr_over_sphere; the
    neighbour flags come from the centres as loadpart sets them.  Returns
    (time, istep, dt) of the file."""
    from .cases import boundp, bounduvw

    c = solver.case
    d = Path(directory)
    f, time, istep_f, dt = read_fld(d / fld_name(istep), c.itot, c.jtot, c.ktot)
    bounduvw(f["u"], f["v"], f["w"], c.bc_top, c.bc_bot)
    boundp(f["p"])
    solver.set_fields(f["u"], f["v"], f["w"], f["p"])
    ps = read_allpartdata(d / allpartdata_name(istep), c.np, solver.nq, fill_tail=True) if c.np else \
        ParticleState(0, solver.nq, 0, lagrangian=False)
    ps.nb = None
    ps.rkp = None
    solver.set_particles(ps)
    return time, istep_f, dt
