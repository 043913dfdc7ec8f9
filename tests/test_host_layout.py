"""The reference host layout through the C ABI, checked by a C program that
builds every array by hand from the reference's index arithmetic
(tests/layout_check.c), without the Python structure mirror that the other
tests and the oracle binding share: field round trip, a planted divergence
found at its (i, j, k) by chkdiv, particle centres and the [p*nl + l] order
of the Lagrangian points.  Run against the CPU oracle here and against the
CUDA library on a GPU."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "layout_check.c"


def _build_and_run(tmp_path: Path, prefix: str, libdir: Path, libname: str, extra_rpath=()) -> str:
    exe = tmp_path / f"layout_{prefix}"
    rpaths = [f"-Wl,-rpath,{libdir}"] + [f"-Wl,-rpath,{p}" for p in extra_rpath]
    cmd = ["gcc", "-O1", "-std=c11", f"-DPFX={prefix}", f"-I{ROOT / 'include'}", str(SRC), "-o", str(exe),
           f"-L{libdir}", f"-l{libname}", *rpaths, "-lm"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def test_layout_against_oracle(tmp_path):
    from oracle.oracle import build_oracle

    lib = build_oracle()
    assert "layout ok" in _build_and_run(tmp_path, "orc_", lib.parent, "ibm_oracle")


@pytest.mark.gpu
def test_layout_against_cuda_library(tmp_path, gpu_lib):
    from interparts_mpich_gb300.solver import library_path

    lib = library_path()
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cudalib = Path(nvcc).resolve().parent.parent / "lib64"
    assert "layout ok" in _build_and_run(tmp_path, "ibm_", lib.parent, "ibm_rk3", extra_rpath=[cudalib])
