"""ibm_chkdiv_noalloc: the divergence check for callers that cannot allocate
device memory (their fields already live on the GPU under their own memory
manager, or they are at a point where cudaMalloc is not allowed).  It must
give the same result as the context's ibm_chkdiv on the same fields, twice in
a row (the shared static scratch keeps the previous call's contents).

This file sorts last so that a run stopping at the first failure has run
every other test before it."""
import ctypes as C

import numpy as np
import pytest

from _util import PLAIN_TOL_CALL
from interparts_mpich_gb300 import IBMSolver
from interparts_mpich_gb300.cases import Case, bounduvw

pytestmark = pytest.mark.gpu


def _random_fields(case, seed):
    rng = np.random.default_rng(seed)
    f = {n: np.asfortranarray(rng.standard_normal(case.shape)) for n in "uvw"}
    bounduvw(f["u"], f["v"], f["w"], case.bc_top, case.bc_bot)
    f["p"] = np.zeros(case.shape, order="F")
    return f


def test_chkdiv_noalloc_matches_chkdiv(gpu_lib):
    import torch

    lib, fn = gpu_lib
    noalloc = fn["chkdiv_noalloc"]
    case = Case(name="noalloc", itot=32, jtot=24, ktot=20, lx=1.0, ly=0.75, lz=0.5)
    solver = IBMSolver(case)
    dxi, dyi, dzi = case.itot / case.lx, case.jtot / case.ly, case.ktot / case.lz
    out = torch.zeros(5, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for call, seed in enumerate((1, 2)):  # two calls in a row on different fields
        f = _random_fields(case, seed)
        solver.set_fields(f["u"], f["v"], f["w"], f["p"])
        solver.set_particles(case.initial_particles(False))
        solver.init_particles()
        tot_ref, max_ref, ijk_ref = solver.chkdiv()
        dev = {n: torch.from_numpy(f[n].ravel(order="F").copy()).cuda() for n in "uvw"}
        p = {n: C.cast(dev[n].data_ptr(), C.POINTER(C.c_double)) for n in "uvw"}
        st = noalloc(p["u"], p["v"], p["w"], case.itot, case.jtot, case.ktot, dxi, dyi, dzi,
                     C.cast(out.data_ptr(), C.POINTER(C.c_double)), C.c_void_p(stream))
        assert st == 0, call
        torch.cuda.synchronize()
        tot, mx, i, j, k = out.cpu().numpy()
        # numpy restatement of the divergence for the tolerance scale
        u, v, w = f["u"], f["v"], f["w"]
        div = ((w[1:-1, 1:-1, 1:-1] - w[1:-1, 1:-1, :-2]) * dzi + (v[1:-1, 1:-1, 1:-1] - v[1:-1, :-2, 1:-1]) * dyi
               + (u[1:-1, 1:-1, 1:-1] - u[:-2, 1:-1, 1:-1]) * dxi)
        assert abs(mx - max_ref) <= PLAIN_TOL_CALL * max_ref, (call, mx, max_ref)
        assert abs(tot - tot_ref) <= PLAIN_TOL_CALL * np.abs(div).sum(), (call, tot, tot_ref)
        assert (int(i), int(j), int(k)) == tuple(ijk_ref), call
        assert abs(mx - np.abs(div).max()) <= PLAIN_TOL_CALL * mx
    solver.close()


def test_chkdiv_noalloc_rejects_oversize(gpu_lib):
    lib, fn = gpu_lib
    dummy = (C.c_double * 8)()
    p = C.cast(dummy, C.POINTER(C.c_double))
    assert fn["chkdiv_noalloc"](p, p, p, 4, 4, 4097, 1.0, 1.0, 1.0, p, None) == -1
