"""Host-side mirror of the reference driver API over the C ABI.

IBMSolver exposes one method per reference subroutine of the hot path
(rk1/rk2/rk3, the IBM forcing loop, the projection, intgr_nwtn_eulr, chkdiv,
chkdt) with the reference's argument meaning.  Errors from the library raise
IBMError with the library's message.  The CUDA library must be built
(interparts_mpich_gb300.build.build()); there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import _abi
from ._abi import ParticleState, bind, dptr
from .cases import Case

_LIB = None
_FN = None


class IBMError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def library_path() -> Path:
    return Path(__file__).resolve().parent / "_build" / "libibm_rk3.so"


def load_library(path: str | Path | None = None):
    """Load libibm_rk3.so (built in-tree).  Raises if it is missing."""
    global _LIB, _FN
    if _LIB is not None and path is None:
        return _LIB, _FN
    p = Path(path) if path else library_path()
    if not p.exists():
        raise RuntimeError(f"{p} is missing: run interparts_mpich_gb300.build.build() first")
    lib = C.CDLL(str(p))
    fn = bind(lib, "ibm_")
    if path is None:
        _LIB, _FN = lib, fn
    return lib, fn


class IBMSolver:
    """One simulation context (fields + particles) on the current GPU."""

    def __init__(self, case: Case, mode: int = _abi.IBM_MODE_PLAIN_FP64, backend=None):
        self.case = case
        self.mode = mode
        if backend is None:
            _, self.fn = load_library()
        else:
            self.fn = backend
        self._params = case.params(mode)
        self.ctx = self.fn["create"](C.byref(self._params))
        if not self.ctx:
            msg = self.fn["last_error"](None)
            raise IBMError(_abi.IBM_E_INVALID, msg.decode() if msg else "create failed")
        nq, nl, nc = C.c_int(), C.c_int(), C.c_int()
        self._chk(self.fn["sizes"](self.ctx, C.byref(nq), C.byref(nl), C.byref(nc)))
        self.nq, self.nl, self.ncells = nq.value, nl.value, nc.value

    def _chk(self, st: int):
        if st != _abi.IBM_OK:
            msg = self.fn["last_error"](self.ctx)
            raise IBMError(st, msg.decode() if msg else "")
        return st

    def close(self):
        if getattr(self, "ctx", None):
            self.fn["destroy"](self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- state ------------------------------------------------------------------
    def _field_arrays(self):
        return [np.zeros(self.case.shape, order="F") for _ in range(7)]

    def set_fields(self, u, v, w, p, durk=None, dvrk=None, dwrk=None):
        arrs = [np.asfortranarray(a, np.float64) if a is not None else None for a in (u, v, w, p, durk, dvrk, dwrk)]
        for a in arrs:
            if a is not None and a.shape != self.case.shape:
                raise ValueError(f"field shape {a.shape} != {self.case.shape}")
        self._chk(self.fn["set_fields"](self.ctx, *[dptr(a) for a in arrs]))

    def get_fields(self, out: dict | None = None) -> dict[str, np.ndarray]:
        """Fields in the reference layout; `out` may supply (pinned) arrays for
        any of u, v, w, p, durk, dvrk, dwrk (the others are then skipped)."""
        names = ["u", "v", "w", "p", "durk", "dvrk", "dwrk"]
        if out is not None:
            arrs = [out.get(n) for n in names]
            for a in arrs:
                if a is not None and (a.shape != self.case.shape or not a.flags.f_contiguous):
                    raise ValueError("output arrays must be Fortran-ordered with the reference shape")
        else:
            arrs = self._field_arrays()
        self._chk(self.fn["get_fields"](self.ctx, *[dptr(a) for a in arrs]))
        return {n: a for n, a in zip(names, arrs) if a is not None}

    def get_intermediate(self) -> dict[str, np.ndarray]:
        arrs = self._field_arrays()[:3]
        self._chk(self.fn["get_intermediate"](self.ctx, *[dptr(a) for a in arrs]))
        return dict(zip(["dudt", "dvdt", "dwdt"], arrs))

    def set_particles(self, ps: ParticleState):
        s = ps.struct()
        self._chk(self.fn["set_particles"](self.ctx, C.byref(s)))

    def get_particles(self, lagrangian: bool = True, out: ParticleState | None = None) -> ParticleState:
        """The particle state; `out` (e.g. page-locked, reused every step)
        receives it instead of a new object."""
        ps = out if out is not None else ParticleState(self.case.np, self.nq, self.nl, lagrangian=lagrangian)
        s = ps.struct()
        self._chk(self.fn["get_particles"](self.ctx, C.byref(s)))
        return ps

    def init_particles(self) -> float:
        vol = C.c_double()
        self._chk(self.fn["init_particles"](self.ctx, C.byref(vol)))
        return vol.value

    def setup(self, fields: dict | None = None, particles: ParticleState | None = None) -> float:
        """Cold start as program interpt does (main.f90:142-206)."""
        f = fields or self.case.initial_fields()
        self.set_fields(f["u"], f["v"], f["w"], f["p"], f.get("durk"), f.get("dvrk"), f.get("dwrk"))
        ps = particles or self.case.initial_particles(lagrangian=False)
        self.set_particles(ps)
        return self.init_particles()

    # ---- reference subroutines -------------------------------------------------------
    def rk(self, rkiter: int, dt: float):
        """rk1/rk2/rk3 (rk3.f90:13-329)."""
        self._chk(self.fn["rk_predict"](self.ctx, rkiter, dt))

    def forcing_loop(self, dt: float, nl_iter: int = 3):
        """IBM loop of the driver (main.f90:286-338)."""
        self._chk(self.fn["forcing_loop"](self.ctx, dt, nl_iter))

    def project(self, rkiter: int, dt: float):
        """fillps, solver2d, correc and pnew += p (main.f90:356-372)."""
        self._chk(self.fn["project"](self.ctx, rkiter, dt))

    def intgr_nwtn_eulr(self, rkiter: int, dt: float):
        """intgr_nwtn_eulr (intgr_nwtn_eulr.f90:12-1514)."""
        self._chk(self.fn["newton_euler"](self.ctx, rkiter, dt))

    def rk3_step(self, dt: float):
        self._chk(self.fn["rk3_step"](self.ctx, dt))

    def run(self, dt: float, nsteps: int):
        self._chk(self.fn["run"](self.ctx, dt, nsteps))

    def run_adaptive(self, nsteps: int, ioutchk: int, dt: float, time: float = 0.0) -> tuple[float, float]:
        """RK3 steps with the reference's time-step control (main.f90:425-441):
        every ioutchk steps chkdiv and chkdt, dt = 0.75*dtmax.  Returns (dt, time)."""
        if "run_adaptive" in self.fn:
            d, t = C.c_double(dt), C.c_double(time)
            self._chk(self.fn["run_adaptive"](self.ctx, int(nsteps), int(ioutchk), C.byref(d), C.byref(t)))
            return d.value, t.value
        # backends without the entry point (the oracle): the same loop on the host
        for istep in range(1, nsteps + 1):
            self.rk3_step(dt)
            time += dt
            if istep % ioutchk == 0:
                tot, _, _ = self.chkdiv()
                if tot > 1e-3:
                    raise IBMError(-6, "total divergence > 1e-3 (chkdiv.f90:51-58)")
                dt = 0.75 * self.chkdt()
        return dt, time

    def timed_step(self, dt: float) -> list[float]:
        self._chk(self.fn["timed_step"](self.ctx, dt))
        ms = (C.c_double * 4)()
        self._chk(self.fn["phase_times"](self.ctx, ms))
        return list(ms)

    def chkdiv(self) -> tuple[float, float, tuple[int, int, int]]:
        tot, mx = C.c_double(), C.c_double()
        ijk = (C.c_int * 3)()
        st = self.fn["chkdiv"](self.ctx, C.byref(tot), C.byref(mx), ijk)
        if st not in (_abi.IBM_OK, _abi.IBM_E_DIVERGENCE):
            self._chk(st)
        return tot.value, mx.value, tuple(ijk)

    def chkdt(self) -> float:
        d = C.c_double()
        self._chk(self.fn["chkdt"](self.ctx, C.byref(d)))
        return d.value

    def slip_residual(self) -> tuple[float, float]:
        mx, rms = C.c_double(), C.c_double()
        self._chk(self.fn["slip_residual"](self.ctx, C.byref(mx), C.byref(rms)))
        return mx.value, rms.value

    def diagnostics(self) -> dict:
        wn, wo = C.c_double(), C.c_double()
        ft = (C.c_double * 3)()
        self._chk(self.fn["diagnostics"](self.ctx, C.byref(wn), C.byref(wo), ft))
        return {"wallshearnew": wn.value, "wallshearold": wo.value, "forcetot": list(ft)}

    # ---- scalar field and plane statistics (post1d) --------------------------------
    def set_scalar(self, c=None, pran: float = 1.0, beta: float = 0.0, bc_c_top_val: float = 0.0,
                   bc_c_bot_val: float = 0.0, bc_c_top_type: int = _abi.IBM_BC_C_DIRICHLET,
                   bc_c_bot_type: int = _abi.IBM_BC_C_DIRICHLET, dcrk=None):
        """Scalar field cnew and its stored RHS dcrkold in the reference layout
        (None: zero) and the scalar parameters (param.f90:39-47; kappa =
        visc/Pran, init.f90:94).  From then on every substep transports it."""
        arrs = []
        for f in (c, dcrk):
            a = None
            if f is not None:
                a = np.asfortranarray(f, np.float64)
                if a.shape != self.case.shape:
                    raise ValueError(f"field shape {a.shape} != {self.case.shape}")
            arrs.append(a)
        sp = _abi.IbmScalarParams(float(pran), float(beta), float(bc_c_top_val), float(bc_c_bot_val),
                                  int(bc_c_top_type), int(bc_c_bot_type))
        self._chk(self.fn["set_scalar"](self.ctx, C.byref(sp), dptr(arrs[0]), dptr(arrs[1])))

    def get_scalar(self) -> tuple[np.ndarray, np.ndarray]:
        """(cnew, dcrkold) in the reference layout."""
        a = np.zeros(self.case.shape, order="F")
        b = np.zeros(self.case.shape, order="F")
        self._chk(self.fn["get_scalar"](self.ctx, dptr(a), dptr(b)))
        return a, b

    PHASE_NAMES = ("gamu", "gamv", "gamw", "gamp", "upart", "vpart", "wpart")

    def phase_indicator(self, itype: int = 1) -> dict[str, np.ndarray]:
        """phase_indicator (phase_indicator.f90:11-559): fluid fractions and
        rigid-body velocities in the reference layout."""
        arrs = self._field_arrays()
        self._chk(self.fn["phase_indicator"](self.ctx, int(itype), *[dptr(a) for a in arrs]))
        return dict(zip(self.PHASE_NAMES, arrs))

    def post1d(self) -> tuple[dict[str, np.ndarray], dict[str, float]]:
        """post1d (output.f90:13-917) without its files: the plane profiles
        (k = 0..k1) and the derived scalars."""
        nk = self.case.shape[2]
        prof = np.zeros(len(_abi.STAT_NAMES) * nk)
        scal = np.zeros(len(_abi.STAT_SCALAR_NAMES))
        self._chk(self.fn["post1d"](self.ctx, dptr(prof), dptr(scal)))
        prof = prof.reshape(len(_abi.STAT_NAMES), nk)
        return ({n: prof[q] for q, n in enumerate(_abi.STAT_NAMES)},
                {n: float(scal[q]) for q, n in enumerate(_abi.STAT_SCALAR_NAMES)})

    def set_projection_solves(self, solves: int):
        """Mixed forms: 1 FP32 Poisson solve per projection (the default) or
        2 (the solve plus a defect-correction solve)."""
        self._chk(self.fn["set_projection_solves"](self.ctx, int(solves)))

    def set_predictor_kernel(self, kind: int):
        """Mixed forms: the FP32 predictor kernel (_abi.IBM_PREDICTOR_AUTO:
        planes staged by 16-byte loads; _PAIRS: 4-byte loads; _TMA: tensor-
        memory-accelerator copies; all three give identical results;
        _CELLS: one cell per thread)."""
        self._chk(self.fn["set_predictor_kernel"](self.ctx, int(kind)))

    def set_step_graphs(self, enable: bool):
        """CUDA graphs of the RK stages (default on); off: every launch direct."""
        self._chk(self.fn["set_step_graphs"](self.ctx, int(bool(enable))))

    def prepare_step_graphs(self, dt: float):
        """Capture the stage graphs that steps with this dt will replay."""
        self._chk(self.fn["prepare_step_graphs"](self.ctx, float(dt)))

    def set_stream(self, stream_handle: int | None):
        self._chk(self.fn["set_stream"](self.ctx, C.c_void_p(stream_handle or 0)))

    def launch_count(self) -> int:
        return int(self.fn["launch_count"](self.ctx)) if "launch_count" in self.fn else 0

    def sync(self):
        if "sync" in self.fn:
            self._chk(self.fn["sync"](self.ctx))

    # --- per-kernel event timing --------------------------------------------------

    PROBE_NAMES = ("predict", "stencil", "interp", "spread", "fillps_fftx", "ffty", "thomas", "ifftx", "correc",
                   "sphere", "features", "mlp", "phase", "stats", "gated")

    def probe(self, mask: int = (1 << 15) - 1):
        """Time every launch of the selected kernel classes with CUDA events."""
        self._chk(self.fn["probe"](self.ctx, int(mask)))

    def probe_result(self) -> dict:
        """{class: (total ms, launches)} since probe(); stops probing."""
        n = len(self.PROBE_NAMES)
        ms = (C.c_double * n)()
        cnt = (C.c_int * n)()
        self._chk(self.fn["probe_result"](self.ctx, ms, cnt))
        return {name: (ms[q], cnt[q]) for q, name in enumerate(self.PROBE_NAMES)}

    # --- learned forcing (IBM_MODE_MIXED_LEARNED) ------------------------------

    NN_NPARAM = 29315
    NN_NNORM = 198

    def harvest(self, capacity: int, stride: int = 1, passes: int = 0):
        """Collect (features, correction) pairs from the plain passes of the
        following forcing loops; capacity=0 stops and keeps the samples."""
        self._chk(self.fn["harvest"](self.ctx, int(capacity), int(stride), int(passes)))

    def harvest_read(self) -> tuple[np.ndarray, np.ndarray]:
        """The harvested training set: features [n, 96], targets [n, 3]."""
        n = C.c_int()
        self._chk(self.fn["harvest_read"](self.ctx, None, None, 0, C.byref(n)))
        f = np.zeros((n.value, 96), np.float32)
        t = np.zeros((n.value, 3), np.float32)
        if n.value:
            self._chk(self.fn["harvest_read"](self.ctx, _fp(f), _fp(t), n.value, C.byref(n)))
        return f, t

    def train_forcing_model(self, nsteps: int, batch: int = 8192, lr: float = 1e-3, seed: int = 0,
                            reinit: bool = False) -> float:
        loss = C.c_double()
        self._chk(self.fn["train_forcing_model"](self.ctx, int(nsteps), int(batch), float(lr), int(seed) & 0xFFFFFFFF,
                                                 int(reinit), C.byref(loss)))
        return loss.value

    def set_forcing_model(self, params: np.ndarray, norm: np.ndarray):
        p = np.ascontiguousarray(params, np.float32)
        n = np.ascontiguousarray(norm, np.float32)
        assert p.size == self.NN_NPARAM and n.size == self.NN_NNORM
        self._chk(self.fn["set_forcing_model"](self.ctx, _fp(p), _fp(n)))

    def get_forcing_model(self) -> tuple[np.ndarray, np.ndarray]:
        p = np.zeros(self.NN_NPARAM, np.float32)
        n = np.zeros(self.NN_NNORM, np.float32)
        self._chk(self.fn["get_forcing_model"](self.ctx, _fp(p), _fp(n)))
        return p, n

    def learned_config(self, enable: bool = True, fallback_ratio: float = 1.5, plain_rms_ref: float = 0.0):
        self._chk(self.fn["learned_config"](self.ctx, int(enable), float(fallback_ratio), float(plain_rms_ref)))

    def learned_calibration(self, period: int):
        """Calibration loops (plain passes that refresh the gate's per-stage
        reduction factor): after 1, 2, 4 ... learned loops of a stage, at
        most period - 1 (0: only the first loop of each stage)."""
        self._chk(self.fn["learned_calibration"](self.ctx, int(period)))

    def learned_gate_state(self) -> dict:
        g = (C.c_double * 6)()
        self._chk(self.fn["learned_gate_state"](self.ctx, g))
        keys = ("r0_last", "plain_factor", "plain_loops", "reference_last", "plain_r0_last", "plain_rms_last")
        return dict(zip(keys, list(g)))

    def forcing_perturbation(self, sigma, seed: int = 0):
        """Point noise of rms sigma[c] (velocity units) after the plain passes
        of every following forcing loop (mixed forms); zeros switch it off."""
        s = (C.c_double * 3)(*[float(x) for x in sigma])
        self._chk(self.fn["forcing_perturbation"](self.ctx, s, int(seed) & 0xFFFFFFFF))

    def learned_stats(self) -> dict:
        s = (C.c_double * 6)()
        self._chk(self.fn["learned_stats"](self.ctx, s))
        keys = ("last_rms", "plain_rms_ref", "fallback_ratio", "fallbacks", "learned_loops", "harvested")
        return dict(zip(keys, list(s)))

    def mlp_gradient(self, params, x, t):
        """Loss, gradient and outputs of the library's training kernels on one batch."""
        p = np.ascontiguousarray(params, np.float32)
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        nb = x.shape[0]
        g = np.zeros(self.NN_NPARAM, np.float32)
        y = np.zeros((nb, 3), np.float32)
        loss = C.c_float()
        self._chk(self.fn["mlp_gradient"](self.ctx, _fp(p), _fp(x), _fp(t), nb, _fp(g), C.byref(loss), _fp(y)))
        return float(loss.value), g, y

    def mlp_infer(self, params, x):
        """Outputs of the library's inference kernel (the forcing loop's) on one batch."""
        p = np.ascontiguousarray(params, np.float32)
        x = np.ascontiguousarray(x, np.float32)
        y = np.zeros((x.shape[0], 3), np.float32)
        self._chk(self.fn["mlp_infer"](self.ctx, _fp(p), _fp(x), x.shape[0], _fp(y)))
        return y

    def mlp_infer_tc(self, params, x):
        """Outputs of the tcgen05 inference kernel on one batch."""
        p = np.ascontiguousarray(params, np.float32)
        x = np.ascontiguousarray(x, np.float32)
        y = np.zeros((x.shape[0], 3), np.float32)
        self._chk(self.fn["mlp_infer_tc"](self.ctx, _fp(p), _fp(x), x.shape[0], _fp(y)))
        return y

    def mlp_fit(self, params, x, t, nsteps: int, lr: float = 1e-3):
        p = np.ascontiguousarray(params, np.float32)
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        out = np.zeros(self.NN_NPARAM, np.float32)
        losses = np.zeros(max(nsteps, 1), np.float32)
        self._chk(self.fn["mlp_fit"](self.ctx, _fp(p), _fp(x), _fp(t), x.shape[0], int(nsteps), float(lr),
                                     _fp(out), _fp(losses)))
        return out, losses[:nsteps]


def _fp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))
