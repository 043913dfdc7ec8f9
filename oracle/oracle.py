"""TEST INFRASTRUCTURE ONLY: Python binding of the CPU oracle (ibm_oracle.cpp).

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline leg may
import this module.  It builds liboracle with the committed Makefile and
exposes the same driver class as the product (IBMSolver) on top of it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from interparts_mpich_gb300._abi import bind  # noqa: E402
from interparts_mpich_gb300.cases import Case  # noqa: E402
from interparts_mpich_gb300.solver import IBMSolver  # noqa: E402

LIB = HERE / "_build" / "libibm_oracle.so"
_lib = None
_fn = None


def build_oracle(verbose: bool = False) -> Path:
    r = subprocess.run(["make", "-C", str(HERE)], capture_output=True, text=True)
    if verbose or r.returncode:
        print(r.stdout, r.stderr)
    if r.returncode:
        raise RuntimeError("oracle build failed")
    return LIB


def load():
    global _lib, _fn
    if _lib is None:
        build_oracle()
        _lib = C.CDLL(str(LIB))
        _fn = bind(_lib, "orc_")
        for name, res, args in [
            ("orc_kernel", C.c_double, [C.c_double]),
            ("orc_kerneltest", C.c_double, []),
            ("orc_vrfft", C.c_int, [C.POINTER(C.c_double), C.c_int, C.c_int]),
            ("orc_nl", C.c_int, [C.c_double, C.c_double]),
            ("orc_set_threads", C.c_int, [C.c_int]),
        ]:
            f = getattr(_lib, name)
            f.restype = res
            f.argtypes = args
    return _lib, _fn


class OracleSolver(IBMSolver):
    """The reference restatement behind the same driver API."""

    def __init__(self, case: Case, threads: int = 0):
        lib, fn = load()
        if threads:
            lib.orc_set_threads(threads)
        super().__init__(case, backend=fn)
