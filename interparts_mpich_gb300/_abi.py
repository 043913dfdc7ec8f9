"""ctypes mirror of include/ibm_rk3.h (structures and function signatures).

The same binder serves any library that exports the header's entry points
under a common prefix.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

c_float_p = C.POINTER(C.c_float)
c_double_p = C.POINTER(C.c_double)
c_int_p = C.POINTER(C.c_int)

IBM_OK = 0
IBM_E_INVALID = -1
IBM_E_CUDA = -2
IBM_E_NOMEM = -3
IBM_E_CONTACT_OVERFLOW = -4
IBM_E_NOT_CONVERGED = -5
IBM_E_DIVERGENCE = -6
IBM_E_STATE = -7

IBM_PREDICTOR_AUTO = 0
IBM_PREDICTOR_PAIRS = 1
IBM_PREDICTOR_CELLS = 2
IBM_PREDICTOR_TMA = 3

IBM_BC_NOSLIP = 0
IBM_BC_FREESLIP = 1
IBM_BC_PERIODIC = 2

IBM_MODE_PLAIN_FP64 = 0
IBM_MODE_MIXED = 1
IBM_MODE_MIXED_LEARNED = 2

IBM_BC_C_DIRICHLET = 0
IBM_BC_C_NEUMANN = 1

# post1d profiles (include/ibm_rk3.h IBM_STAT_*), in order
STAT_NAMES = ("um", "vm", "wm", "pm", "u2", "v2", "w2", "p2", "uv", "uw", "vw", "upm", "vpm", "wpm",
              "up2", "vp2", "wp2", "upvp", "upwp", "vpwp", "gum", "gvm", "gwm", "gpm", "gp2", "guv",
              "guw", "gvw", "ss", "ssp", "cm", "c2", "wc", "cdflx")
STAT_SCALAR_NAMES = ("re_tau", "u_tau", "nu", "re_rbc", "grad_k_wall")


class IbmParams(C.Structure):
    _fields_ = [
        ("itot", C.c_int), ("jtot", C.c_int), ("ktot", C.c_int),
        ("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double),
        ("visc", C.c_double), ("radius", C.c_double), ("ratiorho", C.c_double),
        ("bc_top", C.c_int), ("bc_bot", C.c_int), ("particle_rotation", C.c_int),
        ("np", C.c_int), ("nl", C.c_int),
        ("thetarc", c_double_p), ("phirc", c_double_p), ("radfp", C.c_double),
        ("nb_copies", C.c_int), ("mode", C.c_int), ("radii", c_double_p),
    ]


# per-particle scalar arrays, in header order
PARTICLE_SCALARS = [
    "x", "y", "z", "theta", "phi", "u", "v", "w", "omx", "omy", "omz", "omtheta",
    "intu", "intv", "intw", "intomx", "intomy", "intomz",
    "colfx", "colfy", "colfz", "coltx", "colty", "coltz",
    "fxltot", "fyltot", "fzltot", "torqxltot", "torqyltot", "torqzltot", "torqtheta",
]
CONTACT_ARRAYS = ["cdx", "cdy", "cdz", "cdxt", "cdyt", "cdzt", "cdut", "cdvt", "cdwt", "cpsi"]
LAGRANGIAN_ARRAYS = ["xfp", "yfp", "zfp", "ul", "vl", "wl", "fxl", "fyl", "fzl"]
RKP_FIELDS = ["fxltot", "fyltot", "fzltot", "torqxltot", "torqyltot", "torqzltot", "torqtheta",
              "colfx", "colfy", "colfz", "coltx", "colty", "coltz", "dudt", "dvdt", "dwdt",
              "domxdt", "domydt", "domzdt"]


class IbmScalarParams(C.Structure):
    _fields_ = [("pran", C.c_double), ("beta", C.c_double), ("bc_c_top_val", C.c_double),
                ("bc_c_bot_val", C.c_double), ("bc_c_top_type", C.c_int), ("bc_c_bot_type", C.c_int)]


class IbmParticles(C.Structure):
    _fields_ = ([(n, c_double_p) for n in PARTICLE_SCALARS]
                + [("qmax", c_int_p), ("firstc", c_int_p)]
                + [(n, c_double_p) for n in CONTACT_ARRAYS]
                + [("nb", c_int_p), ("mslv", c_int_p), ("rkp", c_double_p)]
                + [(n, c_double_p) for n in LAGRANGIAN_ARRAYS])


def dptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float64 and (a.flags.c_contiguous or a.flags.f_contiguous)
    return a.ctypes.data_as(c_double_p)


def iptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(c_int_p)


class ParticleState:
    """Host copy of the particle state (SoA numpy arrays) in the header's layout."""

    def __init__(self, np_: int, nq: int, nl: int, lagrangian: bool = True, alloc=None):
        """alloc(n, dtype) -> zeroed 1-D array (default numpy.zeros); a caller
        that moves the state every step passes one returning page-locked
        memory and reuses the object (get_particles(out=...))."""
        z = alloc or (lambda n, dt: np.zeros(n, dt))
        self.np, self.nq, self.nl = np_, nq, nl
        for n in PARTICLE_SCALARS:
            setattr(self, n, z(np_, np.float64))
        self.qmax = z(np_, np.int32)
        self.firstc = z(np_ * nq, np.int32)
        for n in CONTACT_ARRAYS:
            setattr(self, n, z(np_ * nq, np.float64))
        self.nb = z(np_ * 9, np.int32)
        self.mslv = z(np_, np.int32)
        self.mslv[:] = np.arange(1, np_ + 1, dtype=np.int32)
        self.rkp = z(np_ * 19, np.float64)
        for n in LAGRANGIAN_ARRAYS:
            setattr(self, n, z(np_ * nl, np.float64) if lagrangian else None)

    def struct(self) -> IbmParticles:
        s = IbmParticles()
        for n in PARTICLE_SCALARS + CONTACT_ARRAYS + LAGRANGIAN_ARRAYS + ["rkp"]:
            setattr(s, n, dptr(getattr(self, n)))
        for n in ("qmax", "firstc", "nb", "mslv"):
            setattr(s, n, iptr(getattr(self, n)))
        return s

    def nbytes(self) -> int:
        """Bytes of all arrays (what one set or get moves)."""
        return int(sum(a.nbytes for a in vars(self).values() if isinstance(a, np.ndarray)))

    def copy(self) -> "ParticleState":
        o = ParticleState(self.np, self.nq, self.nl, lagrangian=self.xfp is not None)
        for n in PARTICLE_SCALARS + CONTACT_ARRAYS + LAGRANGIAN_ARRAYS + ["qmax", "firstc", "nb", "mslv", "rkp"]:
            a = getattr(self, n)
            setattr(o, n, None if a is None else a.copy())
        return o

    def contact_lists(self) -> list[list[int]]:
        """Partner ids of every particle in slot order (firstc(1:qmax))."""
        fc = self.firstc.reshape(self.np, self.nq)
        return [list(map(int, fc[p, : self.qmax[p]])) for p in range(self.np)]


def bind(lib: C.CDLL, prefix: str) -> dict:
    """Typed function table for the header's entry points under `prefix`."""
    P = C.POINTER
    ctx = C.c_void_p
    sig = {
        "create": (ctx, [P(IbmParams)]),
        "destroy": (C.c_int, [ctx]),
        "last_error": (C.c_char_p, [ctx]),
        "sizes": (C.c_int, [ctx, c_int_p, c_int_p, c_int_p]),
        "set_fields": (C.c_int, [ctx] + [c_double_p] * 7),
        "get_fields": (C.c_int, [ctx] + [c_double_p] * 7),
        "get_intermediate": (C.c_int, [ctx] + [c_double_p] * 3),
        "set_particles": (C.c_int, [ctx, P(IbmParticles)]),
        "get_particles": (C.c_int, [ctx, P(IbmParticles)]),
        "init_particles": (C.c_int, [ctx, c_double_p]),
        "rk_predict": (C.c_int, [ctx, C.c_int, C.c_double]),
        "forcing_loop": (C.c_int, [ctx, C.c_double, C.c_int]),
        "project": (C.c_int, [ctx, C.c_int, C.c_double]),
        "newton_euler": (C.c_int, [ctx, C.c_int, C.c_double]),
        "rk3_step": (C.c_int, [ctx, C.c_double]),
        "run": (C.c_int, [ctx, C.c_double, C.c_int]),
        "chkdiv": (C.c_int, [ctx, c_double_p, c_double_p, c_int_p]),
        "chkdt": (C.c_int, [ctx, c_double_p]),
        "slip_residual": (C.c_int, [ctx, c_double_p, c_double_p]),
        "diagnostics": (C.c_int, [ctx, c_double_p, c_double_p, c_double_p]),
        "set_scalar": (C.c_int, [ctx, P(IbmScalarParams), c_double_p, c_double_p]),
        "get_scalar": (C.c_int, [ctx, c_double_p, c_double_p]),
        "phase_indicator": (C.c_int, [ctx, C.c_int] + [c_double_p] * 7),
        "post1d": (C.c_int, [ctx, c_double_p, c_double_p]),
    }
    optional = {
        "abi_version": (C.c_int, []),
        "set_stream": (C.c_int, [ctx, C.c_void_p]),
        "timed_step": (C.c_int, [ctx, C.c_double]),
        "phase_times": (C.c_int, [ctx, c_double_p]),
        "launch_count": (C.c_longlong, [ctx]),
        "sync": (C.c_int, [ctx]),
        "chkdiv_noalloc": (C.c_int, [c_double_p, c_double_p, c_double_p, C.c_int, C.c_int, C.c_int, C.c_double,
                                     C.c_double, C.c_double, c_double_p, C.c_void_p]),
        "run_adaptive": (C.c_int, [ctx, C.c_int, C.c_int, c_double_p, c_double_p]),
        "fp64_peak": (C.c_int, [c_double_p]),
        "set_projection_solves": (C.c_int, [ctx, C.c_int]),
        "set_predictor_kernel": (C.c_int, [ctx, C.c_int]),
        "set_step_graphs": (C.c_int, [ctx, C.c_int]),
        "prepare_step_graphs": (C.c_int, [ctx, C.c_double]),
        "probe": (C.c_int, [ctx, C.c_uint]),
        "probe_result": (C.c_int, [ctx, c_double_p, c_int_p]),
        "harvest": (C.c_int, [ctx, C.c_int, C.c_int, C.c_int]),
        "harvest_read": (C.c_int, [ctx, c_float_p, c_float_p, C.c_int, c_int_p]),
        "train_forcing_model": (C.c_int, [ctx, C.c_int, C.c_int, C.c_double, C.c_uint, C.c_int, c_double_p]),
        "set_forcing_model": (C.c_int, [ctx, c_float_p, c_float_p]),
        "get_forcing_model": (C.c_int, [ctx, c_float_p, c_float_p]),
        "learned_config": (C.c_int, [ctx, C.c_int, C.c_double, C.c_double]),
        "learned_stats": (C.c_int, [ctx, c_double_p]),
        "learned_calibration": (C.c_int, [ctx, C.c_int]),
        "learned_gate_state": (C.c_int, [ctx, c_double_p]),
        "forcing_perturbation": (C.c_int, [ctx, c_double_p, C.c_uint]),
        "mlp_gradient": (C.c_int, [ctx, c_float_p, c_float_p, c_float_p, C.c_int, c_float_p, c_float_p, c_float_p]),
        "mlp_infer": (C.c_int, [ctx, c_float_p, c_float_p, C.c_int, c_float_p]),
        "mlp_infer_tc": (C.c_int, [ctx, c_float_p, c_float_p, C.c_int, c_float_p]),
        "mlp_fit": (C.c_int, [ctx, c_float_p, c_float_p, c_float_p, C.c_int, C.c_int, C.c_double, c_float_p,
                              c_float_p]),
    }
    table = {}
    for name, (res, args) in list(sig.items()) + list(optional.items()):
        try:
            f = getattr(lib, prefix + name)
        except AttributeError:
            if name in sig:
                raise
            continue
        f.restype = res
        f.argtypes = args
        table[name] = f
    return table
