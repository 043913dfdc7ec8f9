"""Shared helpers of the parity tests."""
from __future__ import annotations

import numpy as np

from interparts_mpich_gb300.cases import Case

# The plain FP64 GPU path must match the FP64 oracle to this relative L2 on
# u, v, w, p and on the particle positions/velocities after 10 RK3 steps.
PLAIN_TOL_10STEP = 1e-10
# per-substep / single-call parity (FMA contraction and summation order only)
PLAIN_TOL_CALL = 1e-12


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    den = np.linalg.norm(b)
    num = np.linalg.norm(a - b)
    if den == 0.0:
        return float(num)
    return float(num / den)


def interior(f: np.ndarray) -> np.ndarray:
    return f[1:-1, 1:-1, 1:-1]


def field_errors(fa: dict, fb: dict, names=("u", "v", "w", "p")) -> dict:
    return {n: rel_l2(interior(fa[n]), interior(fb[n])) for n in names}


def pressure_error(pa: np.ndarray, pb: np.ndarray) -> float:
    """p is defined up to the same constant on both sides; compare as is."""
    return rel_l2(interior(pa), interior(pb))


def particle_errors(pa, pb) -> dict:
    pos_a = np.stack([pa.x, pa.y, pa.z])
    pos_b = np.stack([pb.x, pb.y, pb.z])
    vel_a = np.stack([pa.u, pa.v, pa.w])
    vel_b = np.stack([pb.u, pb.v, pb.w])
    return {"pos": rel_l2(pos_a, pos_b), "vel": rel_l2(vel_a, vel_b)}


def small_case(n=32, nsp=6, radius_cells=4.0, seed=3, **kw) -> Case:
    args = dict(name=f"small{n}", itot=n, jtot=n, ktot=n, radius=radius_cells / n, np=nsp,
                visc=1.0 / 500.0, seed=seed)
    args.update(kw)
    return Case(**args)
