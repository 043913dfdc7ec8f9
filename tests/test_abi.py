"""The C-ABI library builds for sm_103a, loads without a GPU, exports every
entry point declared in include/ibm_rk3.h, and its struct layouts match the
ctypes mirror.  No compute calls are made here."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

from interparts_mpich_gb300 import _abi
from interparts_mpich_gb300 import build as b

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "ibm_rk3.h"


def declared_functions() -> list[str]:
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ibm_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    path = b.build()
    return C.CDLL(str(path))


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binder_covers_header(lib):
    table = _abi.bind(lib, "ibm_")
    for n in declared_functions():
        assert n[len("ibm_"):] in table, n


def test_abi_version(lib):
    lib.ibm_abi_version.restype = C.c_int
    assert lib.ibm_abi_version() == 3


def test_create_rejects_bad_params_before_touching_the_gpu(lib):
    fn = _abi.bind(lib, "ibm_")
    from interparts_mpich_gb300.cases import Case

    case = Case(name="bad", itot=32, jtot=32, ktot=32, radius=4.0 / 32, np=2)
    prm = case.params()
    prm.nl = prm.nl + 1  # the reference aborts when nl != nlmax (main.f90:118-132)
    assert not fn["create"](C.byref(prm))
    assert b"does not match" in fn["last_error"](None)
    prm = case.params()
    prm.itot = 30  # itot/2 = 15 has a factor 5: no FFT plan
    prm.radius = 4.0 / 30
    prm.nl = case.__class__(name="x", itot=30, jtot=32, ktot=32, radius=4.0 / 30, np=2).nl
    assert not fn["create"](C.byref(prm))


def test_struct_layout_matches_header(tmp_path):
    src = tmp_path / "lay.c"
    fields_p = [f for f, _ in _abi.IbmParams._fields_]
    fields_q = [f for f, _ in _abi.IbmParticles._fields_]
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void){",
             'printf("%zu\\n", sizeof(ibm_params));']
    lines += [f'printf("%zu\\n", offsetof(ibm_params, {f}));' for f in fields_p]
    lines += ['printf("%zu\\n", sizeof(ibm_particles));']
    lines += [f'printf("%zu\\n", offsetof(ibm_particles, {f}));' for f in fields_q]
    lines += ["return 0;}"]
    src.write_text("\n".join(lines))
    exe = tmp_path / "lay"
    subprocess.run(["gcc", str(src), "-o", str(exe)], check=True)
    out = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    expect = [C.sizeof(_abi.IbmParams)] + [getattr(_abi.IbmParams, f).offset for f in fields_p]
    expect += [C.sizeof(_abi.IbmParticles)] + [getattr(_abi.IbmParticles, f).offset for f in fields_q]
    assert out == expect
