"""Generates tests/golden/oracle_small.npz: the oracle's state after two RK3
steps of a small seeded channel with three spheres (two of them pushed into
contact).  The fixture freezes the oracle so that later edits of the
restatement cannot drift unnoticed; it is not a reference output (the
reference cannot be built here).

    python tests/golden/make_golden.py      # rewrites the fixture
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from interparts_mpich_gb300.cases import Case  # noqa: E402


def case() -> Case:
    R = 3.0 / 16
    c = np.array([[0.30, 0.40, 0.50], [0.30 + 2 * R * 0.9995, 0.40, 0.50], [0.70, 0.85, 0.30]])
    v = np.array([[0.4, 0.0, 0.0], [-0.4, 0.0, 0.0], [0.0, 0.0, -0.2]])
    return Case(name="golden", itot=16, jtot=16, ktot=16, radius=R, np=3, visc=1.0 / 200.0, seed=21,
                centres=c, velocities=v, ratiorho=1.5)


def generate() -> dict:
    from oracle.oracle import OracleSolver

    o = OracleSolver(case())
    o.setup()
    dt = 2e-3
    o.run(dt, 2)
    f = o.get_fields()
    ps = o.get_particles()
    out = {k: np.ascontiguousarray(f[k][1:-1, 1:-1, 1:-1]) for k in ("u", "v", "w", "p")}
    for k in ("x", "y", "z", "u", "v", "w", "intu", "intw", "colfx", "fxltot", "rkp"):
        out["p_" + k] = getattr(ps, k).copy()
    out["firstc"] = ps.firstc.copy()
    out["qmax"] = ps.qmax.copy()
    return out


if __name__ == "__main__":
    np.savez_compressed(HERE / "oracle_small.npz", **generate())
    print("wrote", HERE / "oracle_small.npz")
