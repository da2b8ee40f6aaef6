#!/usr/bin/env python3
"""Benchmark: PISO time steps of the 128^3 channel on one GB300.

Metric: PISO steps/s and the p'-solve time to a 1e-6
relative residual.  A "step" is one PISO time step of main.f90:134-207:
time-level shift, CourantNo.h, ghost-cell update, calcuvw (gradients,
fluxuvw x3, wall terms, three sipsol solves), PISO_multiple_correction
(2 correctors, PCG-SIP p solves to sor(ip)=0.1 then 1e-6).

  value        steps/s with every field resident in HBM (device-timed with
               CUDA events on the library's stream)
  e2e          the same steps through the C ABI with host buffers: each
               step copies u,v,w,p,f1,f2,f3 from pinned host memory, runs
               cappgpu_piso_steps(1), and copies them back
  roofline     the SIP forward substitution (the hottest unit of the p
               solve) against the measured HBM copy bandwidth, with the
               FP64 issue rate measured in the same run beside it
  cpu_baseline the C oracle (the reference's algorithm restated,
               single-threaded as the reference's recurrences are) on the
               first steps of the timed window, continued from the GPU's
               post-warm-up state, on this machine's host
  fp32_refined / fp32_learned  precision modes 1 and 2 over the same steps
               from the same state; forms_summary repeats their headline
               figures at the end of the line

--impl reference times the oracle (the reference's CPU algorithm) on the
same config and the same window (--warmup steps untimed, then --steps
timed); the reference itself is Fortran and no Fortran compiler exists in
the build image.

Multi-GPU: the step has no data-parallel split (the SIP recurrences are
global), so N GPUs run N independent replicas (weak scaling), launched
with torch.distributed.run; the barrier/max use a gloo group.
"""
import argparse
import json
import os
import pathlib
import subprocess
import sys
import threading
import time

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_DEFAULT = 128
METRIC = "PISO steps/s & p'-solve ms to 1e-6 res: FP64 plain vs FP32+learned, 1 GB300"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Group:
    """Barrier and max-reduce across replica ranks (gloo); no-ops at N=1."""

    def __init__(self, ws):
        self.ws = ws
        self.dist = None
        if ws > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, x):
        if not self.dist:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(n)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs"), "measured"
    return 6800.0, "fallback"


def measured_bf16_peak():
    """Dense BF16 TFLOP/s (burst: the net's kernels are timed alone)."""
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        if d.get("bf16_tflops"):
            return d["bf16_tflops"], "measured"
    return 1900.0, "fallback"


FP32_PARTS_DEFAULT = 11   # the library's default FP32 parts in precision modes 1-2
CPU_SAMPLE = 2            # oracle steps of the cpu_baseline leg
LEARN_STEPS = 20     # PISO steps whose pressure solves are recorded as training pairs
LEARN_EPOCHS = 20
LEARN_BLOCK = 64     # training window (cells per axis)


def snapshot(lib):
    """Every field and the parameters (outside any timed region)."""
    import cappgpu
    return {n: lib.get_field(n) for n in cappgpu.FIELD_NAMES}, lib.get_params()


def restore(lib, snap):
    fields, params = snap
    for n, a in fields.items():
        lib.set_field(n, a)
    lib.set_params(params)


def result_state(lib):
    """Velocity, pressure and the continuity residual after a run (host copies)."""
    p = lib.get_params()
    return {"u": lib.get_field("u"), "v": lib.get_field("v"), "w": lib.get_field("w"), "p": lib.get_field("p"),
            "continuity": float(p.sumlocalconterr)}


def state_errors(x, ref):
    """Relative L2 differences of the velocity vector (normalised by |U| of the
    reference), of u, v, w, p (each by its own norm) and the continuity
    residuals of two runs."""
    import numpy as np
    out = {}
    du = sum(float(np.linalg.norm(x[k] - ref[k])) ** 2 for k in ("u", "v", "w")) ** 0.5
    nu = sum(float(np.linalg.norm(ref[k])) ** 2 for k in ("u", "v", "w")) ** 0.5
    out["velocity_rel_l2"] = du / nu if nu else None
    for k in ("u", "v", "w", "p"):
        den = float(np.linalg.norm(ref[k]))
        out[k + "_rel_l2"] = float(np.linalg.norm(x[k] - ref[k])) / den if den else None
    out["continuity"] = x["continuity"]
    out["continuity_fp64"] = ref["continuity"]
    return out


def profiled_traffic(n):
    """DRAM bytes per launch of the forward sweep from the committed ncu
    capture of the same workload (profiles/), or None."""
    f = ROOT / "profiles" / "k_wave_sip_sweeps_channel128.md"
    if n != 128 or not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith("dram_bytes_per_launch_fwd"):
            return float(line.split("=")[1])
    return None


def make_case(n):
    import cappgpu
    return cappgpu.cases.channel(N=(n, n, n))


def cpu_case_state(case):
    """Oracle state of the case (geometry by the oracle itself)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    import cappgpu
    oracle.build()
    st = oracle.State.from_case(case)
    for n in ("ar1x", "ar1y", "ar1z", "ar2x", "ar2y", "ar2z", "ar3x", "ar3y", "ar3z", "fx", "fy", "fz"):
        case.fields[n] = st.field(n).copy()
    for n, a in cappgpu.cases.initial_face_fluxes(case).items():
        st.set_field(n, a)
    return st


def time_oracle_steps(n, steps, warmup):
    case = make_case(n)
    st = cpu_case_state(case)
    for _ in range(warmup):
        st.piso_steps(1)
    t0 = time.perf_counter()
    for _ in range(steps):
        st.piso_steps(1)
    return time.perf_counter() - t0


def oracle_from_snapshot(lib, case, snap):
    """An oracle state holding the library's state `snap` (every field, the
    BC codes of the case and the parameters): the oracle continues the run
    from where the device left it."""
    import ctypes
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    oracle.build()
    fields, params = snap
    st = oracle.State(case.ni, case.nj, case.nk)
    for name, a in fields.items():
        st.set_field(name, a)
    for face, codes in case.bc.items():
        st.bc(face)[:] = codes
    ctypes.memmove(ctypes.addressof(st.params), ctypes.addressof(params), ctypes.sizeof(params))
    return st


def run_reference(args, ws, rank):
    if rank != 0:
        return
    # the GPU arm's window: the same warm-up steps, then the same timed steps,
    # each one PISO step of the same 128^3 case (about 5 s per step on one
    # host core)
    steps = max(1, args.steps)
    warm = max(0, args.warmup)
    t = time_oracle_steps(args.n, steps, warm)
    v = steps / t
    out = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "steps/s", "n_gpus": ws,
        "steps": steps, "warmup": warm, "ms_per_step": 1e3 * t / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"channel {args.n}^3 PISO (2 correctors, PCG-SIP p to 1e-6)",
                   "cells": args.n ** 3},
        "cpu_baseline": {"value": v, "unit": "steps/s", "cores": 1, "kind": "port",
                         "sample": f"steps {warm + 1}-{warm + steps} of the {args.n}^3 channel "
                                   f"(the GPU arm's timed window), C oracle, 1 thread"},
        "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference is Fortran (no compiler in the image); its algorithm restated in C "
                "(oracle/) and run single-threaded, as its sequential SIP recurrences run",
    }
    print(json.dumps(out), flush=True)


def run_gpu(args, ws, rank, local):
    import cappgpu
    group = Group(ws)
    lib = cappgpu.Library()
    case = make_case(args.n)
    lib.load_case(case)
    cells = args.n ** 3
    for _ in range(args.warmup):
        lib.piso_steps(1)
    snap = snapshot(lib)
    # FP64 issue rate of this GPU (the ceiling of the FP64-bound kernels)
    ms_rate, ops_rate = lib.profile_kernel(11, reps=3)
    fp64_peak = ops_rate / (ms_rate / 1e3)
    clocks = ClockSampler(local)
    launches0 = lib.stats().launches
    # CUDA events around every SIP forward substitution of the timed steps
    # (the roofline's kernel, timed inside the timed region)
    lib.set_option("sweep_timing", 1)
    lib.sweep_stats(reset=True)
    group.barrier()
    clocks.start()
    lib.timer_start()
    lib.piso_steps(args.steps)
    ms = lib.timer_stop()
    clk = clocks.stop()
    group.barrier()
    sweep_ms, sweep_n = lib.sweep_stats(reset=True)
    lib.set_option("sweep_timing", 0)
    launches = lib.stats().launches - launches0
    st = lib.stats()
    ref_state = result_state(lib)   # FP64 plain result of the timed steps
    ms = group.max(ms)
    value = ws * args.steps / (ms / 1e3)

    # end to end through the C ABI with host buffers, from the same state
    # as the device-timed steps
    restore(lib, snap)
    names = ["u", "v", "w", "p", "f1", "f2", "f3"]
    host = {n: lib.pinned(lib.nijk) for n in names}
    for n in names:
        host[n][:] = lib.get_field(n)
    e2e_steps = args.steps
    group.barrier()
    lib.timer_start()
    for _ in range(e2e_steps):
        for n in names:
            lib.set_field(n, host[n])
        lib.piso_steps(1)
        for n in names:
            lib.get_field(n, out=host[n])
    e2e_ms = group.max(lib.timer_stop())
    lib.free_pinned()
    nbytes = len(names) * lib.nijk * 8

    # the FP32 + FP64-refinement form of the pressure solve (precision mode
    # 1), same steps from the same state
    restore(lib, snap)
    lib.precision(1)
    lib.piso_steps(1)   # warm-up of the FP32 buffers and kernels
    restore(lib, snap)
    group.barrier()
    lib.timer_start()
    lib.piso_steps(args.steps)
    ms32 = group.max(lib.timer_stop())
    st32 = lib.stats()
    lib.precision(0)
    errs = state_errors(result_state(lib), ref_state)
    fp32 = {"value": ws * args.steps / (ms32 / 1e3), "unit": "steps/s", "ms_per_step": ms32 / args.steps,
            "p_solve_ms": st32.p_solve_ms, "p_iters": st32.p_report.iters,
            "p_rel_residual": st32.p_report.resl / st32.p_report.res0 if st32.p_report.res0 else None,
            "form": "FP32 SIP-preconditioned CG inside FP64 iterative refinement (exit test on the FP64 residual); "
                    "the FP32 SIP block-local per i-slab (every 8-line block column along i a slab)",
            "errors_vs_fp64": errs}

    # precision mode 2: the refinement form starting from the learned guess.
    # The net is trained on pairs the solver records during steps of the
    # refinement form from the same start, then the same timed steps run.
    restore(lib, snap)
    t0 = time.perf_counter()
    lib.learn_reset(2 * LEARN_STEPS, seed=20261203)
    lib.learn_collect(True)
    lib.precision(1)
    lib.piso_steps(LEARN_STEPS)
    lib.learn_collect(False)
    t1 = time.perf_counter()
    loss = lib.learn_train(LEARN_EPOCHS, block=LEARN_BLOCK, lr=1e-3)
    t2 = time.perf_counter()
    restore(lib, snap)
    lib.precision(2)
    lib.piso_steps(1)   # warm-up of the inference buffers
    restore(lib, snap)
    s0 = lib.learn_stats()
    group.barrier()
    lib.timer_start()
    lib.piso_steps(args.steps)
    msl = group.max(lib.timer_stop())
    stl = lib.stats()
    s1 = lib.learn_stats()
    lib.precision(0)
    # the net's own kernels: one forward pass on this grid (the guess) and one
    # training pass (forward + backward) on a 64^3 window, against the
    # measured dense BF16 peak
    bf16_peak, bf16_kind = measured_bf16_peak()
    net = {}
    for w, name in ((9, "inference"), (10, "train_pass")):
        m, fl = lib.profile_kernel(w, reps=3)
        tf = fl / (m / 1e3) / 1e12
        net[name] = {"ms": m, "gflop": fl / 1e9, "tflops": tf, "frac_of_bf16_peak": tf / bf16_peak}
    net["bf16_peak_tflops"] = bf16_peak
    net["peak_source"] = bf16_kind
    learned = {"value": ws * args.steps / (msl / 1e3), "unit": "steps/s", "ms_per_step": msl / args.steps,
               "p_solve_ms": stl.p_solve_ms, "p_iters": stl.p_report.iters,
               "p_rel_residual": stl.p_report.resl / stl.p_report.res0 if stl.p_report.res0 else None,
               "guesses_kept": s1["guesses"] - s0["guesses"], "guesses_discarded": s1["fallbacks"] - s0["fallbacks"],
               "train": {"pairs": 2 * LEARN_STEPS, "epochs": LEARN_EPOCHS, "block": LEARN_BLOCK, "loss": loss,
                         "loss_kind": "residual norm |A d - r|^2/|r|^2 on the window", "collect_s": t1 - t0,
                         "train_s": t2 - t1},
               "net": net,
               "form": "as fp32_refined, each pressure solve starting from the learned guess when it lowers the "
                       "FP64 residual",
               "errors_vs_fp64": state_errors(result_state(lib), ref_state)}

    # Arithmetic errors of the two reduced-precision forms.  The reference
    # solves p to sor = 0.1 only in the first corrector, and where that
    # solve stops moves the step's result by far more than FP32 rounding
    # (fp64_first_corrector_spread below: FP64 with the first corrector
    # solved to the last one's tolerance against the reference's FP64).  So
    # the three forms are also compared with every corrector solved to the
    # last one's tolerance (the "tight_correctors" option), untimed.
    # The momentum solves (sipsol to sor = 1e-3, at most nsw = 20 sweeps)
    # are solved to 1e-9 in these runs for the same reason.
    def converged_solves(p_factor=1.0):
        pr = lib.get_params()
        for q in range(3):
            pr.sor[q] = 1e-9
            pr.nsw[q] = 400
        pr.sor[3] = pr.sor[3] * p_factor
        pr.nsw[3] = max(pr.nsw[3], 4000)
        lib.set_params(pr)

    lib.set_option("tight_correctors", 1)
    tight = {}
    for mode in (0, 1, 2):
        restore(lib, snap)
        converged_solves()
        lib.precision(mode)
        lib.piso_steps(args.steps)
        tight[mode] = result_state(lib)
    lib.precision(0)
    # every part in FP32, the coefficient assembly included (not the default:
    # FP32 coefficients change the FP64 system the refinement solves)
    restore(lib, snap)
    converged_solves()
    lib.set_option("fp32_parts", 31)
    lib.precision(1)
    lib.piso_steps(args.steps)
    tight_all32 = result_state(lib)
    lib.precision(0)
    lib.set_option("fp32_parts", FP32_PARTS_DEFAULT)
    # FP64 with the pressure solves 100x tighter: how far the 1e-6 tolerance
    # itself lets a solution lie from the converged one
    restore(lib, snap)
    converged_solves(1e-2)
    lib.piso_steps(args.steps)
    tight_fine = result_state(lib)
    # mode 1 at the same tighter tolerance: the arithmetic's own error
    restore(lib, snap)
    converged_solves(1e-2)
    lib.precision(1)
    lib.piso_steps(args.steps)
    tight_fine32 = result_state(lib)
    lib.precision(0)
    lib.set_option("tight_correctors", 0)
    restore(lib, snap)
    precision_check = {
        "steps": args.steps,
        "fp64_first_corrector_spread": state_errors(tight[0], ref_state),
        "fp64_vs_fp64_solved_100x_tighter": state_errors(tight[0], tight_fine),
        "fp32_refined_vs_fp64": state_errors(tight[1], tight[0]),
        "fp32_learned_vs_fp64": state_errors(tight[2], tight[0]),
        "fp32_refined_vs_fp64_solved_100x_tighter": state_errors(tight[1], tight_fine),
        "fp32_refined_vs_fp64_both_solved_100x_tighter": state_errors(tight_fine32, tight_fine),
        "fp32_all_parts_vs_fp64": state_errors(tight_all32, tight[0]),
        "fp32_parts": {"default": FP32_PARTS_DEFAULT, "meaning": "1 pressure solve, 2 momentum solves, "
                       "8 velocity gradients in FP32; 4 momentum assembly, 16 pressure assembly FP64"},
        "note": "every pressure corrector solved to the last one's tolerance and the momentum solves to 1e-9 "
                "in all runs",
    }

    # roofline of the SIP forward substitution on the current state
    peak, peak_kind = measured_peaks()
    ms_alone, bytes_fwd = lib.profile_kernel(0, reps=10)   # the same launch timed alone, for comparison
    ms_fwd = sweep_ms / sweep_n if sweep_n else ms_alone
    achieved = bytes_fwd / (ms_fwd / 1e3) / 1e9
    units = {}
    for w, name in ((1, "sip_backward"), (2, "spmv_dot"), (6, "sip_factor"), (3, "grad_gauss"),
                    (7, "sip_forward_fp32"), (8, "sip_backward_fp32")):
        m, b = lib.profile_kernel(w, reps=3)
        units[name] = {"ms": m, "GBps": b / (m / 1e3) / 1e9}
    # FP64 instructions per interior cell, counted from the kernels' source:
    # the SIP forward substitution 7 (3 multiplies, 3 subtractions, 1
    # multiply), the 7-point product with its dot 15 (7 multiplies, 6
    # subtractions, 1 multiply and 1 add)
    fp64 = {"peak_lane_ops_per_s": fp64_peak, "peak_source": "measured in this run (profile unit 11)"}
    for name, ms_u, per_cell in (("sip_forward", ms_fwd, 7), ("spmv_dot", units["spmv_dot"]["ms"], 15)):
        rate = per_cell * cells / (ms_u / 1e3)
        fp64[name] = {"fp64_ops_per_cell": per_cell, "lane_ops_per_s": rate, "frac": rate / fp64_peak}

    out = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"channel {args.n}^3 PISO (2 correctors, PCG-SIP p to 1e-6, FP64 plain)",
                   "cells": cells, "parallelism": f"replicas{ws}",
                   "l2": "working set (~80 fields x 19 MB) far larger than the 129 MB L2"},
        "cell_updates_per_s": value * cells,
        "p_solve_ms": st.p_solve_ms, "p_iters": st.p_report.iters,
        "p_rel_residual": st.p_report.resl / st.p_report.res0 if st.p_report.res0 else None,
        "e2e": {"value": ws * e2e_steps / (e2e_ms / 1e3), "unit": "steps/s",
                "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes},
        "roofline": {"bound": "hbm", "kernel": "SIP forward substitution (pcg-sip.f90:98-106)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": profiled_traffic(args.n),
                     "algorithmic_bytes": bytes_fwd, "ms_per_launch": ms_fwd,
                     "timed": (f"CUDA events around each of the {sweep_n} pcgsip forward substitutions of the "
                               f"timed steps" if sweep_n else "the launch timed alone"),
                     "ms_per_launch_alone": ms_alone, "fp64_issue": fp64},
        "units": units,
        "fp32_refined": fp32,
        "fp32_learned": learned,
        "precision_check": precision_check,
        "gpu_launches": launches,
        "clocks": clk,
    }
    if rank == 0 and not args.no_cpu_baseline:
        # the oracle continues from the GPU's post-warm-up state: the first
        # CPU_SAMPLE steps of the timed window (about 10 s of one core)
        st_cpu = oracle_from_snapshot(lib, case, snap)
        t0 = time.perf_counter()
        for _ in range(CPU_SAMPLE):
            st_cpu.piso_steps(1)
        t = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": CPU_SAMPLE / t, "unit": "steps/s", "cores": 1, "kind": "port",
                               "sample": f"steps {args.warmup + 1}-{args.warmup + CPU_SAMPLE} of the {args.n}^3 "
                                         f"channel from the GPU's post-warm-up state (C oracle, 1 thread)"}
    # the forms' headline figures once more at the end of the line
    out["forms_summary"] = {
        "fp64_ms_per_step": ms / args.steps, "fp64_p_solve_ms": st.p_solve_ms,
        "fp32_refined_steps_per_s": fp32["value"], "fp32_refined_ms_per_step": fp32["ms_per_step"],
        "fp32_refined_p_solve_ms": fp32["p_solve_ms"],
        "fp32_learned_steps_per_s": learned["value"], "fp32_learned_ms_per_step": learned["ms_per_step"],
        "fp32_learned_p_solve_ms": learned["p_solve_ms"],
        "speedup_fp32_refined": (ms / args.steps) / fp32["ms_per_step"],
        "speedup_fp32_learned": (ms / args.steps) / learned["ms_per_step"],
        "fp32_refined_errors": {k: v for k, v in precision_check["fp32_refined_vs_fp64"].items()
                                if k.endswith("rel_l2")},
        "fp64_tolerance_spread": {k: v for k, v in precision_check["fp64_vs_fp64_solved_100x_tighter"].items()
                                  if k.endswith("rel_l2")},
        "fp32_refined_errors_at_equal_tighter_tolerance": {
            k: v for k, v in precision_check["fp32_refined_vs_fp64_both_solved_100x_tighter"].items()
            if k.endswith("rel_l2")},
    }
    group.close()
    lib.finalize()
    if rank == 0:
        print(json.dumps(out), flush=True)


def run_profile(args):
    """Small fixed workloads for ncu captures (no bench line): one PISO step
    of the channel in FP64 or in the FP32 form after one warm-up step, or
    the learned guess's net (one forward pass on the grid, one training pass
    on a 64^3 window of a recorded pair)."""
    import cappgpu
    lib = cappgpu.Library()
    lib.load_case(make_case(args.n))
    out = {"profile": args.profile, "size": args.n}
    if args.profile in ("step64", "step32"):
        lib.precision(0 if args.profile == "step64" else 1)
        lib.piso_steps(1)
        lib.timer_start()
        lib.piso_steps(1)
        out["ms"] = lib.timer_stop()
    else:
        lib.precision(1)
        lib.learn_reset(2, seed=1)
        lib.learn_collect(True)
        lib.piso_steps(1)
        lib.learn_collect(False)
        for w, name in ((9, "inference"), (10, "train_pass")):
            m, fl = lib.profile_kernel(w, reps=1)
            out[name] = {"ms": m, "tflops": fl / (m / 1e3) / 1e12}
    lib.finalize()
    print(json.dumps(out), flush=True)


def run_learned_config(args):
    """The learned-guess configuration as specified: 2000 (RHS, p') pairs,
    random 64^3 windows of the pressure solves of 200 steps of the 128^3
    channel in precision 1 (two solves a step, five windows a solve),
    normalised by the RMS of the solve's initial residual; the 16/32/64
    U-Net trained with Adam at lr 1e-3 for 20 epochs on the residual-norm
    loss; then inference on a 192^3 channel: per step and per solve the
    PCG iterations and the p'-solve time to the same tolerance with the
    guess (precision 2) and without it (precision 1) from the same state,
    and the fallback rate (guesses discarded because they did not lower
    the FP64 residual).  --learn-loss supervised / energy trains on the
    recorded converged corrections instead (all: the three losses from the
    same start and pairs).  Prints one JSON line (no bench line)."""
    import cappgpu
    steps_rec, per_solve, block, epochs, pairs = 200, 5, 64, 20, 2000
    kinds = {"residual": 0, "supervised": 1, "energy": 2}
    chosen = list(kinds) if args.learn_loss == "all" else [args.learn_loss]
    out = {"learned_config": True, "seed": 20261203}
    lib = cappgpu.Library()
    lib.load_case(make_case(128))
    lib.learn_reset(pairs, seed=20261203)
    p0 = lib.learn_params()
    lib.learn_windows(block, per_solve)
    lib.precision(1)
    lib.learn_collect(True)
    t0 = time.perf_counter()
    lib.piso_steps(steps_rec)
    lib.learn_collect(False)
    t1 = time.perf_counter()
    out["train"] = {"grid": [128, 128, 128], "steps": steps_rec, "pairs": lib.learn_stats()["samples"],
                    "window": block, "epochs": epochs, "lr": 1e-3, "collect_s": t1 - t0}
    params = {}
    for name in chosen:
        lib.learn_params(p0)
        lib.set_option("learn_loss", kinds[name])
        t2 = time.perf_counter()
        loss = lib.learn_train(epochs, block=block, lr=1e-3)
        out["train"][name] = {"loss_last_epoch": loss, "train_s": time.perf_counter() - t2}
        params[name] = lib.learn_params()
    lib.set_option("learn_loss", 0)
    lib.finalize()

    n = args.learned_size
    lib = cappgpu.Library()
    lib.load_case(make_case(n))
    lib.learn_reset(0, seed=20261203)
    lib.precision(0)
    lib.piso_steps(args.warmup)
    snap = snapshot(lib)
    forms = {}
    for mode, name in [(1, None)] + [(2, q) for q in chosen]:
        if name:
            lib.learn_params(params[name])
        restore(lib, snap)
        lib.precision(mode)
        lib.piso_steps(1)   # warm-up of the buffers of the form
        restore(lib, snap)
        s0 = lib.learn_stats()
        per_step = []
        for _ in range(args.steps):
            lib.timer_start()
            lib.piso_steps(1)
            ms = lib.timer_stop()
            st = lib.stats()
            per_step.append({"ms": ms, "p_solve_ms": st.p_solve_ms, "p_iters": st.p_report.iters,
                             "p_rel_residual": st.p_report.resl / st.p_report.res0 if st.p_report.res0 else None})
        s1 = lib.learn_stats()
        kept, dropped = s1["guesses"] - s0["guesses"], s1["fallbacks"] - s0["fallbacks"]
        forms[f"fp32_learned_{name}" if name else "fp32_refined"] = {
            "ms_per_step": sum(q["ms"] for q in per_step) / len(per_step),
            "last_p_solve_ms": sum(q["p_solve_ms"] for q in per_step) / len(per_step),
            "last_p_iters": [q["p_iters"] for q in per_step],
            "guesses_kept": kept if name else None, "guesses_discarded": dropped if name else None,
            "fallback_rate": (dropped / (kept + dropped)) if name and kept + dropped else None,
            "per_step": per_step}
    lib.precision(0)
    lib.finalize()
    out["inference"] = {"grid": [n, n, n], "warmup_fp64_steps": args.warmup, "steps": args.steps, **forms}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--size", dest="n", type=int, default=N_DEFAULT, help="interior cells per axis")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile", choices=["step64", "step32", "net"],
                    help="run a small fixed workload for an ncu capture instead of the bench")
    ap.add_argument("--learned-config", action="store_true",
                    help="train the learned guess as its configuration specifies and compare it at --learned-size")
    ap.add_argument("--learned-size", type=int, default=192)
    ap.add_argument("--learn-loss", default="residual", choices=["residual", "supervised", "energy", "all"],
                    help="training loss of --learned-config (residual: the configuration's)")
    args = ap.parse_args()
    if args.learned_config:
        run_learned_config(args)
        return
    if args.profile:
        run_profile(args)
        return
    ws, rank, local = dist_env()
    if ws > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        run_gpu(args, ws, rank, local)


if __name__ == "__main__":
    main()
