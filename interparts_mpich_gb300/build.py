"""In-tree build of the CUDA library libibm_rk3.so for sm_103a.

Each translation unit is compiled by nvcc in parallel, then linked into one
shared object under interparts_mpich_gb300/_build/.  No cmake, no torch
extension machinery: the product is a plain C-ABI library.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libibm_rk3.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
          "-Xptxas", "-warn-spills"]
# Sources whose FP64 arithmetic must keep the reference's separate
# multiply/add roundings (stencil indices, contact decisions).
NO_FMA = {"ibm_kernels.cu", "particle_kernels.cu", "stats_kernels.cu"}


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libibm_rk3.so")
    return exe


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False, extra_flags: list[str] | None = None) -> Path:
    """Compile every .cu under csrc/ for sm_103a and link libibm_rk3.so."""
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    exe = nvcc()
    jobs = []
    for src in sources():
        obj = BUILD / (src.stem + ".o")
        if force or _stale(obj, [src, *headers]):
            flags = list(COMMON)
            if src.name in NO_FMA:
                flags.append("-fmad=false")
            cmd = [exe, *ARCH, *flags, *(extra_flags or []), "-c", str(src), "-o", str(obj)]
            jobs.append((src, cmd))

    def run(job):
        src, cmd = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        return src, cmd, r

    failed = []
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for src, cmd, r in ex.map(run, jobs):
            if verbose or r.returncode:
                print(" ".join(cmd))
                if r.stdout:
                    print(r.stdout)
                if r.stderr:
                    print(r.stderr)
            if r.returncode:
                failed.append(src.name)
    if failed:
        raise RuntimeError(f"nvcc failed for {failed}")
    objs = [BUILD / (s.stem + ".o") for s in sources()]
    if force or jobs or _stale(LIB, objs):
        cmd = [exe, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode:
            print(" ".join(cmd), r.stdout, r.stderr)
        if r.returncode:
            raise RuntimeError("link of libibm_rk3.so failed")
    return LIB


if __name__ == "__main__":
    import sys

    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
