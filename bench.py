"""Benchmark: ms per RK3 step of the IBM channel (256^3, 1000 spheres D=16dx).

Default run: N=1 GPU, the plain FP64 drop-in path, seeded synthetic inputs
(perturbed Poiseuille channel, random non-overlapping spheres).  Prints one
JSON line.  `--impl reference` times the CPU restatement of the reference
(the oracle, OpenMP on all host cores) on the same workload.

Under torchrun (N>1) every rank runs an independent replica of the case on
its own GPU ("replicas only": the single-GPU step does not shard); timing is
max over ranks after a barrier.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "ms per RK3 step, 256³ channel+1000 spheres: mixed+learned vs plain FP64 GPU"


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        backend = "nccl"
        dist.init_process_group(backend=backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, ws: int) -> float:
    """Max over the replicas (the slowest rank sets the job time)."""
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        sm, smax, reasons = [], [], set()
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    smax.append(float(f[2]))
                except ValueError:
                    continue
                names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
                for n, v in zip(names, f[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
        except Exception:
            pass
        finally:
            try:
                os.unlink(self.path)
            except Exception:
                pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except Exception:
            pass
    return {}


def fp64_peak() -> float | None:
    """Measured FP64 FMA rate of this GPU (TFLOP/s) through the library's
    calibration kernel; None when the library lacks it."""
    import ctypes as C

    from interparts_mpich_gb300.solver import load_library

    _, fn = load_library()
    if "fp64_peak" not in fn:
        return None
    t = C.c_double()
    return t.value if fn["fp64_peak"](C.byref(t)) == 0 else None


def _radii(case):
    import numpy as np
    return np.asarray(case.radii, np.float64) if case.radii is not None else np.array([case.radius])


def sphere_box(case) -> float:
    """Cells of the sphere-integral box (2R/dx + 5)^3, the mean over the
    spheres when they differ."""
    import numpy as np
    return float(np.mean(np.round(2 * _radii(case) * case.dxi + 5) ** 3))


def s_fp(case) -> float:
    """Footprint cells of a sphere's force-point shell, the mean over the
    spheres when they differ."""
    import math
    import numpy as np
    r = (_radii(case) - 0.3 / case.dxi) * case.dxi
    return float(np.mean(4.0 / 3.0 * math.pi * ((r + 1.5) ** 3 - (r - 1.5) ** 3)))


def algorithmic_bytes(case, w: int = 8) -> dict:
    """Reference dataflow model per RK3 step: 3 x [32 N + 27 S_fp np + 3 box np] words."""
    n = case.itot * case.jtot * case.ktot
    dense = 3 * 32 * n * w
    ibm = 3 * 27 * s_fp(case) * case.np * w
    sph = 3 * 3 * sphere_box(case) * case.np * w
    return {"dense": dense, "ibm": ibm, "sphere": sph, "total": dense + ibm + sph,
            "predictor": (10 + 13 + 10) * n * w, "projection": 3 * 21 * n * w}


# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the
# dominant kernels from one ncu capture of the same command (the 256^3 channel
# with 1000 spheres), for the roofline's `traffic` key: {(form, kernel class): bytes}
TRAFFIC = {
    ("learned", "predict"): 282611200 + 352861696,  # k_predict_quad<1, 0> (37-plane z chunks)
    ("mixed", "predict"): 282611200 + 352861696,
    ("learned", "correc"): 402418176 + 284520704,  # k_correc_mixed4
    ("mixed", "correc"): 402418176 + 284520704,
    ("learned", "spread"): 125088000 + 42448384,   # k_ibm_spread_f<1> (the learned spreading)
    ("learned", "interp"): 139311360 + 3998720,    # k_ibm_interp_comp_f<-1, 0> (the gate's residual)
    ("learned", "mlp"): 140372992 + 11529984,      # k_mlp_infer_tc<1> (features formed in the kernel)
    ("learned", "sphere"): 103032576 + 3572992,    # k_sphere_int<float, 1>
    ("mixed", "sphere"): 103032576 + 3572992,
    ("learned", "thomas"): 159725568 + 44540928,   # k_thomas_df
    ("mixed", "thomas"): 159725568 + 44540928,
}


# untimed steps of the learned form between training and the timed steps:
# the gate's calibration loops fall after 1, 2, 4 and 8 learned loops of each
# stage after a new model, then every ninth (calib_period 10)
LEARNED_SETTLE_STEPS = 12


# FP64 flops per cell of the FP64 predictor (momxad/momyad/momzad 3 x 54,
# pressure gradient 6, RK combination 12-18): the plain form's predictor is
# bound by the FP64 pipe, not by HBM
PREDICT_FP64_FLOPS = 183


def kernel_model(case, w: int) -> dict:
    """Algorithmic bytes (or flops) per launch of each probed kernel class, in
    the reference dataflow model (words of distinct compulsory traffic):
    predictor 11 words/cell (stage average), fillps+x FFT 3 reads + 1
    spectrum word, each spectrum pass 2 words, correc 9 words (11 with the
    double-float pressure), IBM interpolation 3 and spreading 6 words per
    footprint cell S_fp, sphere integrals 3 box words per sphere; the MLP in
    flops (2 x 29,184 per point); the FP64 predictor in FP64 flops."""
    n = case.itot * case.jtot * case.ktot
    ibm = s_fp(case) * case.np
    npts = case.np * case.nl
    return {
        "predict": ("fp64", PREDICT_FP64_FLOPS * n) if w == 8 else ("hbm", 11 * n * w),
        "stencil": ("hbm", npts * (24 + (96 if w == 4 else 168))),
        "interp": ("hbm", 3 * ibm * w), "spread": ("hbm", 6 * ibm * w),
        "fillps_fftx": ("hbm", 4 * n * w), "ffty": ("hbm", 2 * n * w), "thomas": ("hbm", 2 * n * w),
        "ifftx": ("hbm", 2 * n * w), "correc": ("hbm", (11 if w == 4 else 9) * n * w),
        "sphere": ("hbm", 3 * sphere_box(case) * case.np * w),
        "features": ("hbm", 3 * ibm * w + npts * 96 * 2), "mlp": ("tensor", 2 * 29184 * npts),
        # the learned loop's plain passes 2..Nl: no work unless the gate fell back
        "gated": ("hbm", 0),
    }


def statistics_timing(solver, case, calls: int) -> dict:
    """post1d on the final state: the phase indicator and the plane sums on
    the device, the O(ktot) epilogue on the host.  Kernel times from the
    event probe; the plane-sum kernel's roofline from its compulsory reads
    per cell (u, v, w, p, the four phase keys, the three winner codes)."""
    solver.post1d()  # first call allocates the phase buffers
    solver.sync()
    solver.probe((1 << 12) | (1 << 13))
    t0 = time.perf_counter()
    for _ in range(calls):
        solver.post1d()
    call_ms = (time.perf_counter() - t0) * 1e3 / calls
    k = solver.probe_result()
    phase_ms = k["phase"][0] / max(k["phase"][1], 1)
    sums_ms = k["stats"][0] / max(k["stats"][1], 1)
    w = 8 if solver.mode == 0 else 4
    ncell = case.itot * case.jtot * case.ktot
    bytes_per_cell = 3 * w + 8 + 4 * 8 + 3 * 4
    ach = ncell * bytes_per_cell / (sums_ms * 1e-3) / 1e9
    hbm = measured_peaks().get("hbm_gbs", 6800.0)
    return {"calls": calls, "ms_per_call": round(call_ms, 4), "phase_indicator_ms": round(phase_ms, 4),
            "plane_sums_ms": round(sums_ms, 4),
            "plane_sums_roofline": {"bound": "hbm", "algorithmic_per_launch": ncell * bytes_per_cell,
                                    "achieved": round(ach, 1), "unit": "GB/s", "frac": round(ach / hbm, 4)}}


def workload_case(args):
    from interparts_mpich_gb300.cases import channel_case, poly_case, wide_channel_case

    if args.workload == "poly":
        return poly_case(3 * args.n, 3 * args.n // 2, args.np if args.np != 1000 else 15000, seed=1234)
    if args.workload == "wide":
        return wide_channel_case(2 * args.n, args.n, args.np if args.np != 1000 else 8000, seed=1234)
    return channel_case(args.n, args.np, seed=1234)


def harvest_and_train(solver, case, dt, args) -> dict:
    """Plain warm-up steps with harvesting (every stride-th point, so that the
    samples span all of them), then the GPU training of the network."""
    hs = max(1, args.harvest_steps)
    stride = max(1, -(-hs * 3 * case.np * case.nl // args.harvest))
    solver.harvest(capacity=args.harvest, stride=stride, passes=args.harvest_passes)
    for _ in range(hs):
        solver.rk3_step(dt)
    solver.harvest(0)
    solver.sync()
    t0 = time.perf_counter()
    loss = solver.train_forcing_model(args.train_steps, batch=args.batch, lr=1e-3, seed=1)
    train_s = time.perf_counter() - t0
    st = solver.learned_stats()
    return {"harvested_samples": int(st["harvested"]), "harvest_steps": hs, "harvest_stride": stride,
            "harvest_passes": args.harvest_passes, "train_steps": args.train_steps, "batch": args.batch,
            "adam_lr": 1e-3, "train_s": round(train_s, 3), "final_loss_std_units": round(loss, 5)}


def run_form(args, ws, rank, local, mode: int, with_e2e: bool):
    """Times one arithmetic form on the channel case: K steps between CUDA
    events on the library's stream, plus the per-phase times of one step."""
    import torch

    from interparts_mpich_gb300 import IBM_MODE_MIXED_LEARNED, IBMSolver
    from interparts_mpich_gb300._abi import ParticleState
    from interparts_mpich_gb300.cases import channel_case

    case = workload_case(args)
    solver = IBMSolver(case, mode=mode)
    if args.proj_solves and mode != 0:
        solver.set_projection_solves(args.proj_solves)
    if mode != 0:
        solver.set_predictor_kernel({"auto": 0, "pairs": 1, "cells": 2, "tma": 3}[args.predictor])
    stream = torch.cuda.Stream()
    solver.set_stream(stream.cuda_stream)
    if args.no_graphs:
        solver.set_step_graphs(False)
    solver.setup(case.initial_fields())
    dt = 0.5 * solver.chkdt()  # frozen dt (0.5 dtmax at t=0, main.f90:151-154)
    if args.workload == "poly":
        # settling from rest: dtmax at t = 0 is the viscous limit, far above
        # what the spheres' fall allows; CFL 0.5 on the gravitational
        # velocity scale sqrt((rho_r - 1) g D) of the mean diameter instead
        import math
        dmean = 2.0 * float(case.radii.mean())
        dt = min(dt, 0.5 / case.dxi / math.sqrt((case.ratiorho - 1.0) * 9.81 * dmean))
    learn = None
    nwarm = args.warmup
    if mode == IBM_MODE_MIXED_LEARNED:
        if args.workload in ("channel", "poly"):
            # the first warm-up steps: plain passes with harvesting; then GPU training
            learn = harvest_and_train(solver, case, dt, args)
            # untimed steps through the gate's early calibration phase after a
            # new model (calibration loops after 1, 2, 4, 8 learned loops of a
            # stage), so that the timed steps hold the settled one loop in ten
            nwarm = max(nwarm, LEARNED_SETTLE_STEPS)
        else:
            # the network is harvested and trained on the 256^3 channel, then
            # runs on this case
            ch = channel_case(256, 1000, seed=1234)
            src = IBMSolver(ch, mode=mode)
            src.setup(ch.initial_fields())
            learn = harvest_and_train(src, ch, 0.5 * src.chkdt(), args)
            learn["trained_on"] = "channel 256^3, 1000 spheres"
            p, nrm = src.get_forcing_model()
            src.close()
            solver.set_forcing_model(p, nrm)
            solver.learned_config(enable=True, fallback_ratio=1.5)
            nwarm = max(nwarm, LEARNED_SETTLE_STEPS)
    for _ in range(nwarm):
        solver.rk3_step(dt)
    solver.sync()
    phases = solver.timed_step(dt)
    # the RK stages run as CUDA graphs: capture every stage graph the timed
    # steps replay now, so that no capture falls inside them
    if not args.no_graphs:
        solver.prepare_step_graphs(dt)
    probe_steps = max(1, args.steps)
    torch.cuda.synchronize()
    launches0 = solver.launch_count()
    barrier(ws)
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        if args.no_graphs:
            solver.probe(args.probe_mask if args.probe_mask > 0 else (1 << len(solver.PROBE_NAMES)) - 1)
        with torch.cuda.stream(stream):
            torch.cuda.nvtx.range_push("timed")  # profilers select the timed steps by this range
            ev0.record(stream)
            solver.run(dt, args.steps)
            ev1.record(stream)
            torch.cuda.nvtx.range_pop()
        ev1.synchronize()
        torch.cuda.synchronize()
        barrier(ws)
        ms = ev0.elapsed_time(ev1) / args.steps
        launches = solver.launch_count() - launches0
        if not args.no_graphs:
            # the kernel table and the roofline kernel: CUDA events around every
            # launch of every kernel class over as many further steps, launched
            # directly (a replayed graph cannot record events per launch); the
            # kernels are the same, at the same point of the run
            solver.probe(args.probe_mask if args.probe_mask > 0 else (1 << len(solver.PROBE_NAMES)) - 1)
            solver.run(dt, probe_steps)
        kernels_all = solver.probe_result()
    ms_max = max_over_ranks(ms, ws)
    solver.sync()
    _, divmax, _ = solver.chkdiv()
    # (the plane statistics are not defined for polydisperse spheres)
    stats = (statistics_timing(solver, case, args.stats_calls)
             if args.stats_calls > 0 and args.workload != "poly" else None)
    if learn is not None:
        st = solver.learned_stats()
        gs = solver.learned_gate_state()
        learn.update({"learned_rms_residual_last": st["last_rms"],
                      "plain_reference_last": st["plain_rms_ref"],
                      "plain_reduction_factor": gs["plain_factor"],
                      "plain_calibration_loops": int(gs["plain_loops"]),
                      "fallbacks": int(st["fallbacks"]), "learned_loops": int(st["learned_loops"])})
        # the same substep from the same state, three ways: rms no-slip residual
        solver.learned_calibration(0)
        res = {}
        for name, nl, on in (("one_sweep", 1, False), ("plain_nl3", 3, False), ("one_sweep_plus_network", 3, True)):
            solver.learned_config(enable=on, fallback_ratio=1e9 if on else 1.5)
            solver.rk(1, dt)
            solver.forcing_loop(dt, nl)
            res[name] = solver.slip_residual()[1]
        solver.learned_config(enable=True, fallback_ratio=1.5)
        learn["rms_residual_same_substep"] = res
    e2e = None
    if with_e2e and args.e2e_steps > 0:
        # end to end through the C ABI with host buffers: u,v,w,p and the
        # particle state from pinned host memory, one step, read back
        pin = {k: torch.empty(case.shape[::-1], dtype=torch.float64, pin_memory=True).numpy().T for k in "uvwp"}
        cur = solver.get_fields()
        for k in "uvwp":
            pin[k][...] = cur[k]
        tdt = {np.float64: torch.float64, np.int32: torch.int32}

        def pinned(n, dt):
            return torch.zeros(n, dtype=tdt[dt], pin_memory=True).numpy()

        ps = ParticleState(case.np, solver.nq, solver.nl, lagrangian=True, alloc=pinned)
        solver.get_particles(out=ps)
        h2d = 4 * pin["u"].nbytes + ps.nbytes()
        d2h = 4 * pin["u"].nbytes + ps.nbytes()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            solver.set_fields(pin["u"], pin["v"], pin["w"], pin["p"])
            solver.set_particles(ps)
            solver.rk3_step(dt)
            solver.get_fields(out=pin)
            solver.get_particles(out=ps)
        torch.cuda.synchronize()
        e2e_ms = (time.perf_counter() - t0) * 1e3 / args.e2e_steps
        e2e = {"value": round(max_over_ranks(e2e_ms, ws), 4), "unit": "ms/step",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)}
    solver.close()
    return {"case": case, "dt": dt, "ms": ms_max, "phases": phases, "launches": launches, "clocks": clk.summary(),
            "e2e": e2e, "ncell": case.itot * case.jtot * case.ktot, "divmax": divmax, "learn": learn,
            "kernels": kernels_all, "probe_steps": probe_steps, "stats": stats}


def cpu_baseline(args, case_fn):
    """The oracle restatement timed on the host cores on one RK3 step of the workload."""
    from oracle.oracle import OracleSolver, load

    lib, _ = load()
    cores = lib.orc_set_threads(os.cpu_count() or 1)
    case = case_fn()
    o = OracleSolver(case)
    o.setup()
    dt = 0.5 * o.chkdt()
    t0 = time.perf_counter()
    o.rk3_step(dt)
    t = (time.perf_counter() - t0) * 1e3
    t0 = time.perf_counter()
    o.post1d()
    t_stats = (time.perf_counter() - t0) * 1e3
    o.close()
    return {"value": round(t, 1), "unit": "ms/step", "cores": int(cores), "kind": "port",
            "sample": f"1 RK3 step of the same {case.itot}^3 / {case.np}-sphere case (oracle restatement, OpenMP)",
            "post1d_ms": round(t_stats, 1)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="channel", choices=["channel", "wide", "poly"],
                    help="channel: n^3, np spheres (the headline case); wide: 2n x 2n x n on a (2, 2, 1) box, "
                         "8000 spheres, the learned network trained on the 256^3 channel; poly: 3n x 3n x 1.5n "
                         "on a (2, 2, 1) box, 15000 settling spheres of D = 12..24 dx (rho_r 2, Ga 200), the "
                         "network harvested and trained on the same case")
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--np", type=int, default=1000)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--form", default="all", choices=["all", "both", "plain", "mixed", "learned"])
    ap.add_argument("--harvest", type=int, default=2_000_000, help="harvest capacity (samples)")
    ap.add_argument("--harvest-steps", type=int, default=6,
                    help="plain warm-up steps harvested (every stride-th point, so that the capacity spans them)")
    ap.add_argument("--harvest-passes", type=int, default=3,
                    help="plain passes of the harvested loops (3: the Nl = 3 correction the network replaces)")
    ap.add_argument("--train-steps", type=int, default=20000)
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--stats-calls", type=int, default=3, help="post1d calls timed after the steps (0: none)")
    ap.add_argument("--probe-mask", type=int, default=-1,
                    help="kernel classes timed with CUDA events (bit per class; default: every class) over as "
                         "many steps as the timed ones, run right after them (with --no-graphs: inside them)")
    ap.add_argument("--predictor", default="auto", choices=["auto", "pairs", "cells", "tma"],
                    help="FP32 predictor kernel of the mixed forms (auto: planes staged by 16-byte loads; "
                         "tma: by tensor-memory-accelerator copies)")
    ap.add_argument("--no-graphs", action="store_true", help="issue every launch directly (no CUDA graphs of the stages)")
    ap.add_argument("--proj-solves", type=int, default=0,
                    help="FP32 Poisson solves per projection in the mixed forms (0: the library default)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    ws, rank, local = dist_init()

    from interparts_mpich_gb300.cases import channel_case

    wl = workload_case(args)
    if args.workload == "poly":
        desc = (f"polydisperse settling {wl.itot}x{wl.jtot}x{wl.ktot} ({wl.lx:g} x {wl.ly:g} x {wl.lz:g}), "
                f"{wl.np} spheres D=12..24dx, rho_r=2, Ga=200, fluid at rest, Nl=3, "
                f"dt=min(0.5 dtmax, 0.5 dx/sqrt((rho_r-1) g D_mean)) frozen")
    else:
        desc = (f"{'channel' if args.workload == 'channel' else 'wide channel'} "
                f"{wl.itot}x{wl.jtot}x{wl.ktot} ({wl.lx:g} x {wl.ly:g} x {wl.lz:g}), {wl.np} spheres "
                f"D=16dx, perturbed Poiseuille Re_b=5600, Nl=3, dt=0.5 dtmax frozen")
    config = {"workload": desc,
              "grid": [wl.itot, wl.jtot, wl.ktot], "spheres": wl.np,
              "l2_policy": "inputs larger than L2 (each field >= 137 MB > 129 MB L2)",
              "launch": "per-kernel launches" if args.no_graphs else "CUDA graphs of the RK stages (captured before the timed steps)"}

    if args.impl == "reference":
        if rank != 0:
            return
        from oracle.oracle import OracleSolver, load
        lib, _ = load()
        cores = lib.orc_set_threads(os.cpu_count() or 1)
        case = workload_case(args)
        o = OracleSolver(case)
        o.setup()
        dt = 0.5 * o.chkdt()
        nsteps = min(args.steps, 2)
        o.rk3_step(dt)  # one untimed warm-up step (bounded sample)
        t0 = time.perf_counter()
        for _ in range(nsteps):
            o.rk3_step(dt)
        ms = (time.perf_counter() - t0) * 1e3 / nsteps
        sample = f"{nsteps} RK3 steps after 1 warm-up step of the same case (oracle restatement, OpenMP)"
        line = {"metric": METRIC, "value": round(ms, 1), "unit": "ms/step", "impl": "reference", "n_gpus": 0,
                "steps": nsteps, "warmup": 1, "ms_per_step": round(ms, 1), "higher_is_better": False,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config,
                "cpu_baseline": {"value": round(ms, 1), "unit": "ms/step", "cores": int(cores), "kind": "port",
                                 "sample": sample},
                "e2e": {"value": round(ms, 1), "unit": "ms/step", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch

    from interparts_mpich_gb300 import IBM_MODE_MIXED, IBM_MODE_MIXED_LEARNED, IBM_MODE_PLAIN_FP64
    from interparts_mpich_gb300 import build as b

    torch.cuda.set_device(local)
    b.build()
    barrier(ws)
    forms = {"plain": IBM_MODE_PLAIN_FP64, "mixed": IBM_MODE_MIXED, "learned": IBM_MODE_MIXED_LEARNED}
    wanted = {"all": ["plain", "mixed", "learned"], "both": ["plain", "learned"]}.get(args.form, [args.form])
    head = next(f for f in ("learned", "mixed", "plain") if f in wanted)
    res = {f: run_form(args, ws, rank, local, forms[f], with_e2e=True) for f in wanted}
    if rank != 0:
        return
    r = res[head]
    case = r["case"]
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs", 6800.0)
    tflops = peaks.get("bf16_tflops", 1900.0)
    fp64 = fp64_peak()
    peak_of = {"hbm": hbm, "tensor": tflops, "fp64": fp64 or float("nan")}
    unit_of = {"hbm": "GB/s", "tensor": "TFLOP/s", "fp64": "TFLOP/s"}
    w = 8 if head == "plain" else 4

    def kernel_table(x, wb, key="kernels", steps=1):
        """Per kernel class: launches and mean duration (CUDA events), the
        algorithmic bytes or flops per launch and the fraction of the peak.
        key "kernels": the probed steps (every class)."""
        model = kernel_model(x["case"], wb)
        out = {}
        for name, (tot_ms, cnt) in x[key].items():
            if cnt == 0:
                continue
            bound, units = model[name]
            per = tot_ms / cnt
            ach = units / (per * 1e-3) / (1e9 if bound == "hbm" else 1e12)
            peak = peak_of[bound]
            out[name] = {"launches_per_step": round(cnt / steps, 2), "ms_per_launch": round(per, 4),
                         "share_of_step": round(tot_ms / steps / x["ms"], 4), "bound": bound,
                         "algorithmic_per_launch": int(units), "achieved": round(ach, 3 if bound == "fp64" else 1),
                         "unit": unit_of[bound], "frac": round(ach / peak, 4)}
        return out
    ab = algorithmic_bytes(case, w)
    names = ["predictor", "ibm", "projection", "newton_euler"]
    ktab = kernel_table(r, w, "kernels", r["probe_steps"])
    # the roofline kernel: the class with the largest share of the step
    ttab = {k: v for k, v in ktab.items() if v["algorithmic_per_launch"] > 0}
    dom = max(ttab, key=lambda k: ttab[k]["share_of_step"])
    dk = ttab[dom]
    # the ncu bytes were captured on the 256^3 channel with 1000 spheres only
    measured_case = args.workload == "channel" and args.n == 256 and args.np == 1000
    traffic = TRAFFIC.get((head, dom)) if measured_case else None
    line = {
        "metric": METRIC, "value": round(r["ms"], 4), "unit": "ms/step", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(r["ms"], 4), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": {"plain": "f64", "mixed": "f32+f64", "learned": "f32+f64 (bf16/f16 MLP)"}[head], "data": "synthetic",
        "config": config,
        "form": {"plain": "plain FP64 (drop-in)", "mixed": "mixed FP32/FP64",
                 "learned": "mixed FP32/FP64 + learned forcing"}[head],
        "forms": {f: {"ms_per_step": round(x["ms"], 4),
                      "mcell_steps_per_s": round(args.gpus * x["ncell"] / (x["ms"] * 1e-3) / 1e6, 1),
                      "phases_ms": {n: round(t, 4) for n, t in zip(names, x["phases"])},
                      "chkdiv_max": x["divmax"], "gpu_launches": int(x["launches"]),
                      "kernels": kernel_table(x, 8 if f == "plain" else 4, "kernels", x["probe_steps"]),
                      **({"e2e": x["e2e"]} if x["e2e"] else {}),
                      **({"post1d": x["stats"]} if x["stats"] else {}),
                      **({"learned_forcing": x["learn"]} if x["learn"] else {})} for f, x in res.items()},
        "mcell_steps_per_s": round(args.gpus * r["ncell"] / (r["ms"] * 1e-3) / 1e6, 1),
        "hbm_roofline_frac_step": round(ab["total"] / (r["ms"] * 1e-3) / 1e9 / hbm, 4),
        "roofline": {"bound": dk["bound"], "kernel": dom, "achieved": dk["achieved"],
                     "peak": peak_of[dk["bound"]], "unit": dk["unit"], "frac": dk["frac"],
                     "traffic": traffic,
                     # the DRAM bandwidth the kernel's measured traffic implies (its honest
                     # roof when it is not bound by its own unit, e.g. the gather-bound MLP)
                     **({"dram_gbs": round(traffic / (dk["ms_per_launch"] * 1e-3) / 1e9, 1),
                         "dram_frac": round(traffic / (dk["ms_per_launch"] * 1e-3) / 1e9 / hbm, 4)}
                        if traffic else {}),
                     "algorithmic_per_launch": dk["algorithmic_per_launch"], "ms_per_launch": dk["ms_per_launch"],
                     "timing": ("CUDA events around every launch of every kernel class over as many steps as "
                                "the timed ones, run directly right after them (the timed steps replay CUDA "
                                "graphs of the RK stages, which cannot record events per launch)"
                                if not args.no_graphs else "CUDA events around every launch inside the timed steps"),
                     "peak_source": ("ibm_fp64_peak, FMA chains on all SMs (of measured)" if dk["bound"] == "fp64"
                                     else ("MEASURED_PEAKS.json " + ("hbm_gbs" if dk["bound"] == "hbm" else "bf16_tflops")
                                           + " (of measured)") if peaks else "fallback (of fallback)")},
        "fp64_peak_tflops": round(fp64, 4) if fp64 else None,
        "kernels": ktab,
        "gpu_launches": int(r["launches"]),
        "clocks": r["clocks"],
        "dt": r["dt"],
    }
    for f in ("mixed", "learned"):
        if "plain" in res and f in res:
            line[f"speedup_{f}_vs_plain"] = round(res["plain"]["ms"] / res[f]["ms"], 3)
    if r["e2e"]:
        line["e2e"] = r["e2e"]
    if not args.no_cpu_baseline:
        try:
            line["cpu_baseline"] = cpu_baseline(args, lambda: workload_case(args))
        except Exception as ex:  # the baseline is reported, never required
            line["cpu_baseline"] = {"value": None, "error": str(ex)[:200]}
    print(json.dumps(line))


if __name__ == "__main__":
    main()
