#!/usr/bin/env python
"""Throughput of the StrangSplitting hot path on GB300, one JSON line.

Workload: the two-component exciton-polariton problem on a 512 x 512 grid (L = 256,
2x2 matrix dispersion, G = diag(0, g|u2|^2), Gaussian photon pump with a linear
ramp, dt = 0.05), FP64 fields.  One "step" is one full Strang step of every
trajectory in the batch.  The batch holds independent copies of the field so that
the working set (fields + tables) is more than twice the 129 MB L2: every pass
streams from HBM.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--dtype c128|c64]

value      : grid-point-steps/s over all ranks, inputs resident in HBM, CUDA-event timed
e2e        : the same through the C ABI with host buffers: H2D of the state from pinned
             memory, K steps, D2H of the final state, wall-clock timed
roofline   : dominant kernel, algorithmic bytes per launch / its mean event-timed
             duration, against the measured HBM copy bandwidth
cpu_baseline: the FP64 CPU restatements (C/OpenMP and numpy/scipy.fft, all host threads) on
             bounded samples; the faster is the baseline
plain_gpu  : the plain GPU split step on the same workload (cuFFT transforms + unfused
             torch elementwise kernels, the reference's step order): its rate, the rate
             of its transforms alone, and the fused passes' speed-up over both
--impl reference: the reference's algorithm on the host cores (the Julia reference
             cannot run here; its C/OpenMP restatement in oracle/ is the reference arm)
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_GRID, L_BOX, DT = 512, 256.0, 0.05
POL = dict(hbar=0.6582, m=1 / 6, dc=-0.5, dx=0.0, gc=0.05, gx=0.005, Om=5.07, g=0.003, A=5.0, ramp=200.0, w=50.0)
L2_BYTES = 129 * 2 ** 20


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def polariton_closures():
    p = POL

    def disp(k, _):
        k2 = k[0] ** 2 + k[1] ** 2
        return [[p["hbar"] * k2 / (2 * p["m"]) - p["dc"] - 1j * p["gc"], p["Om"]], [p["Om"], -p["dx"] - 1j * p["gx"]]]

    def nonl(u, _):
        return [0 * u[0], p["g"] * np.abs(u[1]) ** 2]

    def pump(r, _, t):
        a = p["A"] * min(t / p["ramp"], 1.0)
        return [a * np.exp(-((r[0] - L_BOX / 2) ** 2 + (r[1] - L_BOX / 2) ** 2) / p["w"] ** 2), 0]

    return disp, nonl, pump


def batch_for(dtype) -> int:
    per = 2 * N_GRID * N_GRID * (16 if dtype == np.complex128 else 8)
    return int(2 ** math.ceil(math.log2(2 * L2_BYTES / per)))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = "clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown," \
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 6:
                continue
            try:
                sm.append(float(parts[0]))
                mx = max(mx, float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[2:6]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_model() -> str:
    """The host CPU's model name (lscpu), or the architecture when it is not reported."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    import platform
    return platform.machine()


def _time_cpu_form(form: str, seconds: float):
    """Steps per second of one FP64 CPU form of the reference's algorithm on one 512^2
    two-component polariton trajectory, all host threads, about `seconds` of work:
    "c" = the C/OpenMP restatement (oracle/gpe_ref.c), "numpy" = the numpy/scipy.fft one."""
    from oracle import gpe_oracle as O
    prob = oracle_problem(O)
    cores = os.cpu_count() or 1
    if form == "c":
        from oracle import gpe_oracle_c as OC
        it = OC.CIterator(prob, (0.0, 200.0), DT, 100, threads=cores)
        it.step(2)  # warm-up
        n, t0 = 0, time.perf_counter()
        while time.perf_counter() - t0 < seconds and n < 4000:
            it.step(10)
            n += 10
        return n, time.perf_counter() - t0
    it = O.OracleIterator(prob, (0.0, 200.0), DT, 100, fft_workers=cores)
    t = DT
    it.step(t, DT)  # warm-up
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds and n < 4000:
        t += DT
        it.step(t, DT)
        n += 1
    return n, time.perf_counter() - t0


def cpu_baseline(seconds: float = 10.0):
    """The FP64 CPU restatements of the reference's algorithm on the host cores, each on a
    bounded sample (~`seconds` of work): the faster is the baseline, the other is listed."""
    cores = os.cpu_count() or 1
    P = N_GRID * N_GRID
    forms = {}
    for form in ("c", "numpy"):
        n, el = _time_cpu_form(form, seconds)
        forms[form] = {"value": P * n / el, "steps": n, "seconds": el}
    best = max(forms, key=lambda f: forms[f]["value"])
    other = "numpy" if best == "c" else "c"
    name = {"c": "C/OpenMP restatement with its own radix-2 FFT (oracle/gpe_ref.c)",
            "numpy": "numpy restatement with scipy.fft"}
    return {"value": forms[best]["value"], "unit": "grid-point-steps/s", "cores": cores, "cpu": cpu_model(),
            "kind": "port",
            "sample": f"{forms[best]['steps']} Strang steps of one 512^2 two-component trajectory, FP64, "
                      f"{name[best]}, {cores} threads, {forms[best]['seconds']:.1f} s",
            "other_form": {"form": name[other], "value": forms[other]["value"],
                           "sample": f"{forms[other]['steps']} steps, {forms[other]['seconds']:.1f} s"}}


def oracle_problem(O):
    p = POL
    dg, rg = O.grids((L_BOX, L_BOX), (N_GRID, N_GRID))
    X, Y = O.mesh(dg)
    prof = np.exp(-((X - L_BOX / 2) ** 2 + (Y - L_BOX / 2) ** 2) / p["w"] ** 2)

    def disp(k, _):
        k2 = k[0] ** 2 + k[1] ** 2
        one = np.ones_like(k2)
        return np.array([[p["hbar"] * k2 / (2 * p["m"]) - p["dc"] - 1j * p["gc"], p["Om"] * one],
                         [p["Om"] * one, (-p["dx"] - 1j * p["gx"]) * one]])

    z = np.zeros((N_GRID, N_GRID), np.complex128)
    return O.OracleProblem(u0=(z, z.copy()), lengths=(L_BOX, L_BOX), dispersion=disp,
                           nonlin_g=np.array([[0, 0], [0, p["g"]]], np.complex128),
                           pump_profile=np.stack([prof, 0 * prof]).astype(np.complex128),
                           pump_amp=lambda t: np.array([p["A"] * min(t / p["ramp"], 1.0), 0.0]))


def run_reference(args, rank, world):
    """The reference arm: the reference's algorithm on the host cores, in its faster CPU
    restatement (the C/OpenMP one; the Julia reference has no julia binary here)."""
    if rank != 0:
        return
    from oracle import gpe_oracle as O
    from oracle import gpe_oracle_c as OC
    prob = oracle_problem(O)
    cores = os.cpu_count() or 1
    it = OC.CIterator(prob, (0.0, 200.0), DT, 100, threads=cores)
    it.step(args.warmup)
    t0 = time.perf_counter()
    it.step(args.steps)
    el = time.perf_counter() - t0
    P = N_GRID * N_GRID
    v = P * args.steps / el
    line = {"metric": "grid-point-steps/s", "value": v, "unit": "grid-point-steps/s", "impl": "reference",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_dict(np.complex128, batch_for(np.complex128), world),
            "cpu_baseline": {"value": v, "unit": "grid-point-steps/s", "cores": cores, "cpu": cpu_model(), "kind": "port",
                             "sample": f"each step = one Strang step of one 512^2 two-component trajectory "
                                       f"(FP64, the C/OpenMP restatement oracle/gpe_ref.c, {cores} threads); the "
                                       f"Julia reference has no julia binary on this box, so its algorithm runs as "
                                       f"this restatement"},
            "e2e": {"value": v, "unit": "grid-point-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def config_dict(dtype, B, world):
    fb = 2 * N_GRID * N_GRID * B * (16 if dtype == np.complex128 else 8)
    return {"workload": f"2-component exciton-polariton {N_GRID}x{N_GRID}, L={L_BOX:g}, 2x2 matrix dispersion, "
                        f"pumped photon, dt={DT}; {B} independent copies per GPU",
            "grid": [N_GRID, N_GRID], "components": 2, "batch_per_gpu": B, "global_batch": B * world,
            "field_bytes_per_gpu": fb,
            "l2_policy": f"inputs larger than L2: fields {fb / 2**20:.0f} MiB + tables per GPU vs 129 MB L2",
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU"}


def algorithmic_bytes(dtype, B: int):
    """Bytes per grid point (of one copy) per launch of each pass: both components read
    and written once, plus the tables every copy shares read once per launch (the photon
    pump profile, r bytes a point; the 2x2 k-space table, 4c bytes a point) and so
    divided over the B copies.  c = complex size, r = real size."""
    c = 16 if dtype == np.complex128 else 8
    r = c // 2
    row = 2 * 2 * c + r / B
    col = 2 * 2 * c + 4 * c / B
    return {"row": row, "col": col}


def binding_limit(dtype, fp64: str) -> str:
    """What bounds the passes of this precision (from ncu captures of the same passes)."""
    if dtype == np.complex128 and fp64 == "bfp":
        return ("row pass: FP64 pipe (the pointwise half steps; GB300 issues FP64 at 1/64 of the FP32 rate) "
                "overlapped with the block floating point transforms on the integer pipes; column pass: integer "
                "ALU pipe (transforms and FP64 <-> fixed point conversions) and issue; DRAM below 10 % of peak")
    if dtype == np.complex128 and fp64 == "native":
        return ("FP64 pipe: 82-83 % active in both passes (GB300 issues FP64 at 1/64 of the FP32 rate, about "
                "1.2 TFLOP/s); DRAM stays below 10 % of peak")
    if dtype == np.complex128:
        return ("FP32-pipe instruction issue: double-word arithmetic, about 1900 + 1300 instructions per point "
                "(row + column), 70 % of issue slots busy, DRAM 9-14 % of peak")
    return "instruction issue (row: ALU pipe 43 %, 68 % of issue slots) and global-load latency (column)"


def arith_name(dtype, fp64: str) -> str:
    if dtype == np.complex64:
        return "f32"
    if fp64 == "bfp":
        return ("f64 (FP64 pointwise steps; line transforms and the k-space table between them in block floating "
                "point: 64-bit integers under one exponent a line)")
    return "f64" if fp64 == "native" else "f64-dw (double-word f32 pairs, 2^-48 unit roundoff)"


def measure_fused(pkg, lib, L, args, dtype, fp64: str, B: int, local_rank: int, world: int, dist, with_e2e: bool):
    """Device-resident throughput of the fused passes on the polariton workload (and, with
    with_e2e, the same through gpe_set_field / gpe_run with pinned host buffers)."""
    disp, nonl, pump = polariton_closures()
    u0 = np.zeros((N_GRID, N_GRID, B), dtype, order="F")
    prob = pkg.GrossPitaevskiiProblem((u0, u0.copy()), (L_BOX, L_BOX), dispersion=disp, nonlinearity=nonl, pump=pump)
    total = args.warmup + 3 * args.steps + 8
    it = pkg.StrangSplittingIterator(prob, (0.0, 200.0), dt=DT, nsaves=100, total_steps=max(total, 4000),
                                     device=local_rank, fp64=fp64)
    h = it.h
    P = N_GRID * N_GRID
    it.step(args.warmup)

    def barrier():
        if dist:
            dist.barrier()

    # clocks sampled over both runs: the per-launch-event run (kernel times for the
    # roofline) and the clean run that `value` times
    with ClockSampler(local_rank) as clk:
        L.check(lib, h, lib.gpe_set_timing(h, 1))
        barrier()
        L.check(lib, h, lib.gpe_run(h, args.steps, 0, None, None))
        barrier()
        kms = np.zeros(3)
        kn = np.zeros(3, np.int64)
        L.check(lib, h, lib.gpe_kernel_times(h, L.ptr(kms), L.ptr(kn)))
        L.check(lib, h, lib.gpe_set_timing(h, 0))
        L.check(lib, h, lib.gpe_run(h, args.steps, 0, None, None))
        ms_clean = lib.gpe_last_run_ms(h)
        launches = lib.gpe_last_run_launches(h)  # the kernels of the run that `value` times
    if dist:
        import torch
        t = torch.tensor([ms_clean], device=f"cuda:{local_rank}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_clean = float(t.item())
    value = P * B * args.steps * world / (ms_clean * 1e-3)
    out = {"value": value, "ms_clean": ms_clean, "launches": int(launches), "kms": kms, "kn": kn,
           "clocks": clk.summary()}
    if with_e2e:
        # the state in and the result out both live in pinned host memory
        try:
            import torch
            rt = torch.float64 if dtype == np.complex128 else torch.float32
            pinned = [torch.zeros(B * P * 2, dtype=rt).pin_memory() for _ in range(2)]
            hbufs = [pb.numpy().view(dtype) for pb in pinned]
            out_pinned = torch.empty(2 * B * P * 2, dtype=rt).pin_memory()
            res = out_pinned.numpy().view(dtype).reshape(2, 1, B * P)
        except Exception:
            hbufs = [np.zeros(B * P, dtype) for _ in range(2)]
            res = np.empty((2, 1, B * P), dtype)
        for m in range(2):
            hbufs[m][:] = 0
        barrier()
        t0 = time.perf_counter()
        for m in range(2):
            L.check(lib, h, lib.gpe_set_field(h, m, L.ptr(hbufs[m])))
        L.check(lib, h, lib.gpe_run(h, args.steps, args.steps, L.ptr(res), None))
        e2e_s = time.perf_counter() - t0
        barrier()
        if dist:
            import torch
            t = torch.tensor([e2e_s], device=f"cuda:{local_rank}")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            e2e_s = float(t.item())
        out["e2e_value"] = P * B * args.steps * world / e2e_s
        out["state_bytes"] = 2 * B * P * np.dtype(dtype).itemsize
    it.close()
    return out


def fp64_roof(m: dict, B: int, sm_mhz):
    """The FP64-pipe roof of the native FP64 passes: nominal flops per grid point and launch
    (5 log2 N per point of each complex line transform, the conventional FFT count; 32 for
    the 2x2 complex k-space mat-vec; 30 per half step for the density, phase, rotation and
    pump) over the mean event-timed launch duration, against GB300's FP64 peak (two FP64
    FMAs a clock per SM, as ncu reports it, at the clock sampled during the run)."""
    try:
        import torch
        nsm = torch.cuda.get_device_properties(0).multi_processor_count
    except Exception:
        nsm = 152
    mhz = sm_mhz or 2070.0
    peak = 2 * 2 * nsm * mhz * 1e6 / 1e12
    P = N_GRID * N_GRID
    lg = int(math.log2(N_GRID))
    flops = {"row": 2 * 2 * 5 * lg + 2 * 30, "col": 2 * 2 * 5 * lg + 32}  # two components
    out = {}
    for i, k in enumerate(["row", "col"]):
        ms = m["kms"][i] / max(m["kn"][i], 1)
        tf = flops[k] * P * B / (ms * 1e-3) / 1e12
        out[k] = {"flops_per_point": flops[k], "achieved_tflops": tf, "frac": tf / peak}
    return {"bound": "fp64 pipe", "unit": "TFLOP/s", "peak": peak,
            "peak_source": f"2 FP64 FMA per clock per SM x {nsm} SMs x {mhz:.0f} MHz", "kernels": out}


def fp64_issue_roof(m: dict, B: int, sm_mhz):
    """The FP64-pipe roof of the default FP64 row pass, whose FP64 work is its two half
    steps (the transforms run on the integer pipes): FP64 instructions per grid point by
    construction of the polariton's compile-time specialised half step at its shortest
    phase polynomial (the workload's phases stay below 2^-10) -- per half step the exciton
    density 2, phase 1, polynomial 6, rotation 4, the photon's merged pump 2 -- over the
    mean event-timed launch, against two FP64 instructions a clock per SM at the sampled
    clock.  The column pass holds no FP64 work."""
    try:
        import torch
        nsm = torch.cuda.get_device_properties(0).multi_processor_count
    except Exception:
        nsm = 152
    mhz = sm_mhz or 2070.0
    peak = 2 * nsm * mhz * 1e6 / 1e12  # tera-instructions/s
    P = N_GRID * N_GRID
    per_point = 2 * (2 + 1 + 6 + 4 + 2)
    ms = m["kms"][0] / max(m["kn"][0], 1)
    ach = per_point * P * B / (ms * 1e-3) / 1e12
    return {"bound": "fp64 pipe (row pass)", "unit": "FP64 Tinst/s", "peak": peak,
            "peak_source": f"2 FP64 instructions per clock per SM x {nsm} SMs x {mhz:.0f} MHz",
            "fp64_inst_per_point": per_point, "achieved": ach, "frac": ach / peak}


def roofline_of(m: dict, dtype, fp64: str, B: int):
    """Dominant kernel's algorithmic bytes per launch over its mean event-timed duration,
    against the measured HBM copy bandwidth (and, for native FP64, the FP64-pipe roof)."""
    P = N_GRID * N_GRID
    kms, kn = m["kms"], m["kn"]
    ab = algorithmic_bytes(dtype, B)
    peak, peak_kind = measured_peaks()
    per_launch = {"row": (kms[0] / max(kn[0], 1), ab["row"]), "col": (kms[1] / max(kn[1], 1), ab["col"])}
    dom = "row" if kms[0] >= kms[1] else "col"
    d_ms, d_b = per_launch[dom]
    achieved = d_b * P * B / (d_ms * 1e-3) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": None, "kernel": f"{dom} pass", "peak_source": f"{peak_kind} hbm_gbs",
            "traffic_note": "DRAM bytes per launch come from separate ncu captures of the same passes, not from "
                            "this run",
            "algorithmic_bytes_per_point": d_b, "launch_ms": d_ms,
            "kernels": {k: {"launches": int(kn[i]), "total_ms": float(kms[i]),
                            "mean_ms": float(kms[i] / max(kn[i], 1)),
                            "achieved_gbs": float(ab[k] * P * B / (kms[i] / max(kn[i], 1) * 1e-3) / 1e9)}
                        for i, k in enumerate(["row", "col"])},
            "binding_limit": binding_limit(dtype, fp64),
            **({"compute_roof": fp64_roof(m, B, (m.get("clocks") or {}).get("sm_mhz"))}
               if dtype == np.complex128 and fp64 == "native" else {}),
            **({"compute_roof": fp64_issue_roof(m, B, (m.get("clocks") or {}).get("sm_mhz"))}
               if dtype == np.complex128 and fp64 == "bfp" else {})}


def run_gpu(args, rank, world, local_rank):
    import __graft_entry__ as G
    pkg = G.load_package()
    L = sys.modules["gpe_gb300._lib"]
    lib = pkg.load_library()
    dist = None
    if world > 1:
        import torch
        import torch.distributed as tdist
        torch.cuda.set_device(local_rank)
        tdist.init_process_group("nccl")
        dist = tdist
    dtype = np.complex128 if args.dtype == "c128" else np.complex64
    B = args.batch or batch_for(dtype)
    P = N_GRID * N_GRID
    m = measure_fused(pkg, lib, L, args, dtype, args.fp64, B, local_rank, world, dist, with_e2e=True)
    value = m["value"]
    dw = fl = None
    if dtype == np.complex128 and args.fp64 == "bfp" and not args.no_dw:
        # FP64 floating point throughout (the reference's arithmetic, transforms included)
        mfl = measure_fused(pkg, lib, L, args, dtype, "native", B, local_rank, world, dist, with_e2e=False)
        fl = {"dtype": arith_name(dtype, "native"), "value": mfl["value"], "unit": "grid-point-steps/s",
              "ms_per_step": mfl["ms_clean"] / args.steps, "gpu_launches": mfl["launches"],
              "headline_speedup": value / mfl["value"], "roofline": roofline_of(mfl, dtype, "native", B),
              "clocks": mfl["clocks"]}
    if dtype == np.complex128 and args.fp64 in ("bfp", "native") and not args.no_dw:
        # the opt-in double-word mode on the same workload, reported beside the FP64 headline
        mdw = measure_fused(pkg, lib, L, args, dtype, "dw", B, local_rank, world, dist, with_e2e=False)
        dw = {"dtype": arith_name(dtype, "dw"), "value": mdw["value"], "unit": "grid-point-steps/s",
              "ms_per_step": mdw["ms_clean"] / args.steps, "gpu_launches": mdw["launches"],
              "speedup_vs_f64": mdw["value"] / value, "roofline": roofline_of(mdw, dtype, "dw", B),
              "clocks": mdw["clocks"]}
    plain = None
    if args.plain_steps > 0:
        plain = run_plain_gpu(dtype, B, args.plain_steps, 3, local_rank, value / world)
        if dtype == np.complex128 and rank == 0:
            plain["rel_l2_fused_vs_plain_f64"] = plain_vs_fused_rel_l2(pkg, local_rank, fp64=args.fp64)
            plain["rel_l2_case"] = (f"one pumped 512^2 field from u = 0, 200 steps, fused "
                                    f"{ {'bfp': 'FP64 (block floating point transforms)', 'native': 'FP64'}.get(args.fp64, 'double-word')} "
                                    f"vs plain FP64")

    if rank != 0:
        return
    line = {
        "metric": "grid-point-steps/s", "value": value, "unit": "grid-point-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": m["ms_clean"] / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": arith_name(dtype, args.fp64),
        "data": "synthetic (zero initial field, pumped; the reference's polariton parameters)",
        "config": config_dict(dtype, B, world),
        "e2e": {"value": m["e2e_value"], "unit": "grid-point-steps/s",
                "h2d_bytes_per_step": m["state_bytes"] / args.steps,
                "d2h_bytes_per_step": m["state_bytes"] / args.steps},
        "gpu_launches": m["launches"],
        "roofline": roofline_of(m, dtype, args.fp64, B),
        "clocks": m["clocks"],
    }
    if fl is not None:
        line["fp64_float_transforms"] = fl
    if dw is not None:
        line["double_word"] = dw
    if plain is not None:
        line["plain_gpu"] = plain
    if args.anchor_steps > 0:
        line["kerr1024"] = run_kerr1024(pkg, lib, L, local_rank, args.anchor_steps)
    if args.solve_run:
        line["polariton_solve"] = run_polariton_solve(pkg, lib, local_rank)
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline()
    if args.twa_steps > 0:
        line["twa"] = run_twa(pkg, args.twa_steps, tune=not args.no_tune)
    print(json.dumps(line), flush=True)


def run_polariton_solve(pkg, lib, device):
    """The polariton configuration exactly as specified, through solve(): one 512^2
    two-component field, tspan (0, 200), dt 0.05 (4000 steps), nsaves 100 returned to the
    host (the save ring streams every save out while the next steps run).  Wall-clock
    time of the whole call (closure sampling, set-up, steps, saves, result assembly) and
    of the stepping alone; FP64 (double-word) and FP32."""
    disp, nonl, pump = polariton_closures()
    out = []
    for dtype, fp64 in ((np.complex128, "bfp"), (np.complex128, "native"), (np.complex128, "dw"),
                        (np.complex64, "native")):
        z = np.zeros((N_GRID, N_GRID), dtype, order="F")
        prob = pkg.GrossPitaevskiiProblem((z, z.copy()), (L_BOX, L_BOX), dispersion=disp, nonlinearity=nonl,
                                          pump=pump)
        t0 = time.perf_counter()
        it = pkg.StrangSplittingIterator(prob, (0.0, 200.0), dt=DT, nsaves=100, device=device, fp64=fp64)
        t1 = time.perf_counter()
        ts, res = it.solve()
        t2 = time.perf_counter()
        it.close()
        steps = 4000
        save_bytes = 100 * 2 * N_GRID * N_GRID * np.dtype(dtype).itemsize
        out.append({"dtype": {"bfp": "f64-bfp", "dw": "f64-dw"}.get(fp64, "f64") if dtype == np.complex128 else "f32",
                    "steps": steps, "saves": 100,
                    "setup_s": t1 - t0, "solve_s": t2 - t1, "total_s": t2 - t0,
                    "point_steps_per_s": N_GRID * N_GRID * steps / (t2 - t1),
                    "saved_bytes": save_bytes, "result_shape": list(res[0].shape),
                    "plain_gpu_ms_per_step": plain_single_field_ms(dtype, device)})
    return {"workload": "2-component polariton 512x512, one field, tspan (0, 200), dt 0.05, nsaves 100, via solve()",
            "runs": out}


def run_kerr1024(pkg, lib, L, device, steps):
    """Scalar Kerr at 1024^2 (L=32, u0 = exp(-|r - r0|^2 / 4), r0 = (16, 16), D = |k|^2/2,
    G = |u|^2, dt = 0.005), FP64 fields: a single field (16 MiB, L2-resident) and 16
    independent copies (256 MiB, streamed from HBM), double-word and native FP64.
    Algorithmic bytes per point-step: two passes each reading and writing the field
    (4 x 16 B) plus the scalar k-space table (16 B) = 80 B."""
    N, Lb, dt = 1024, 32.0, 0.005
    x = np.arange(N) * (Lb / N)
    X, Y = np.meshgrid(x, x, indexing="ij")
    base = np.exp(-((X - 16) ** 2 + (Y - 16) ** 2) / 4.0).astype(np.complex128)
    peak, _ = measured_peaks()
    out = []
    for B, fp64 in ((1, "dw"), (16, "dw"), (16, "native"), (16, "bfp")):
        u0 = np.asfortranarray(np.repeat(base[:, :, None], B, axis=2)) if B > 1 else np.asfortranarray(base)
        prob = pkg.GrossPitaevskiiProblem((u0,), (Lb, Lb), dispersion=lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2,
                                          nonlinearity=lambda u, p: np.abs(u[0]) ** 2)
        it = pkg.StrangSplittingIterator(prob, (0.0, 1e3 * dt), dt=dt, nsaves=1, device=device, fp64=fp64)
        it.step(5)
        L.check(lib, it.h, lib.gpe_run(it.h, steps, 0, None, None))
        ms = lib.gpe_last_run_ms(it.h)
        it.close()
        v = N * N * B * steps / (ms * 1e-3)
        gbs = 80.0 * v / 1e9
        out.append({"batch": B, "arith": {"dw": "f64-dw", "bfp": "f64-bfp"}.get(fp64, "f64"), "steps": steps,
                    "ms_per_step": ms / steps, "value": v, "unit": "grid-point-steps/s",
                    "algorithmic_gbs": gbs, "frac_of_hbm": gbs / peak,
                    "l2": "field L2-resident (16 MiB)" if B == 1 else "256 MiB of fields, streamed from HBM"})
    return {"workload": "scalar Kerr 1024x1024 FP64, L=32, G=|u|^2, dt=0.005 (80 algorithmic B per point-step)",
            "runs": out}


def expm2_np(A):
    """exp(A) for a field of 2x2 complex matrices A[i, j][...] (closed form: e^{tr/2}
    [cosh(s) I + sinh(s)/s (A - tr/2 I)], s^2 = ((a-d)/2)^2 + bc, series for sinh(s)/s
    near s = 0)."""
    ht = (A[0][0] + A[1][1]) / 2
    hd = (A[0][0] - A[1][1]) / 2
    s = np.sqrt(hd * hd + A[0][1] * A[1][0])
    small = np.abs(s) < 1e-3
    s2 = s * s
    shs = np.where(small, 1 + s2 / 6 + s2 * s2 / 120, np.sinh(s) / np.where(small, 1.0, s))
    e = np.exp(ht)
    ch = np.cosh(s)
    return [[e * (ch + shs * (A[0][0] - ht)), e * shs * A[0][1]], [e * shs * A[1][0], e * (ch + shs * (A[1][1] - ht))]]


class PlainSplitStep:
    """The plain GPU form of the reference's Strang step for the polariton workload, the
    comparator of the fused passes: cuFFT transforms (torch.fft.fft2 over every component
    and copy at once) and the per-point work as separate elementwise torch operations, in
    the reference's order (src/strang_splitting.jl:69-90): at each half-step time the pump
    is evaluated over the whole grid into the `next` buffer after `now` takes the old one
    (src/misc.jl:22-42), then u <- cis(-dt/2 G(u)) (u + dt/4 F_now) + dt/4 F_next
    (src/kernels.jl:37-54); between the half steps the 2x2 table exp(-i dt D(k)) (built in
    FP64 on the host, src/misc.jl:14-20) is applied per k between the forward and the
    normalised inverse transform.  State: torch tensor (2, B, N, N), [component][copy][y][x]."""

    def __init__(self, N: int, L: float, B: int, dtype, device, u0=None, dt: float = DT, prm=None):
        import torch
        self.torch = torch
        p = prm or POL
        self.p, self.dt, self.N, self.B = p, dt, N, B
        c64 = dtype == np.complex64
        self.cdt = torch.complex64 if c64 else torch.complex128
        rdt = torch.float32 if c64 else torch.float64
        x = np.arange(N) * (L / N)
        k = 2 * np.pi * np.fft.fftfreq(N, L / N)
        KY, KX = np.meshgrid(k, k, indexing="ij")
        Y, X = np.meshgrid(x, x, indexing="ij")
        k2 = KX ** 2 + KY ** 2
        one = np.ones_like(k2)
        D = [[p["hbar"] * k2 / (2 * p["m"]) - p["dc"] - 1j * p["gc"], p["Om"] * one],
             [p["Om"] * one, (-p["dx"] - 1j * p["gx"]) * one]]
        E = expm2_np([[-1j * dt * D[i][j] for j in range(2)] for i in range(2)])
        dev = torch.device(device)
        self.T = [[torch.tensor(E[i][j], dtype=self.cdt, device=dev) for j in range(2)] for i in range(2)]
        prof = np.exp(-((X - L / 2) ** 2 + (Y - L / 2) ** 2) / p["w"] ** 2)
        self.prof = torch.tensor(prof, dtype=rdt, device=dev)
        self.u = (torch.zeros((2, B, N, N), dtype=self.cdt, device=dev) if u0 is None
                  else torch.tensor(np.asarray(u0), dtype=self.cdt, device=dev))
        self.t = 0.0
        self.nxt = self.prof * self.amp(0.0)  # init evaluates F(t0) into `next`
        self.now = torch.empty_like(self.nxt)

    def amp(self, t: float) -> float:
        return self.p["A"] * min(t / self.p["ramp"], 1.0)

    def half(self, t_pump: float):
        torch = self.torch
        self.now, self.nxt = self.nxt, self.now
        torch.mul(self.prof, self.amp(t_pump), out=self.nxt)
        dth = self.dt / 2
        u0, u1 = self.u[0], self.u[1]
        u0.add_(self.now, alpha=dth / 2)   # G_0 = 0: cis(0) (u + dt/4 F_now) + dt/4 F_next
        u0.add_(self.nxt, alpha=dth / 2)
        dens = torch.view_as_real(u1).square().sum(-1)
        u1.mul_(torch.exp(dens.mul(-1j * dth * self.p["g"])))

    def diffusion(self):
        torch = self.torch
        U = torch.fft.fft2(self.u)
        V = torch.empty_like(U)
        for i in range(2):
            torch.mul(self.T[i][0], U[0], out=V[i])
            V[i].addcmul_(self.T[i][1], U[1])
        self.u = torch.fft.ifft2(V)

    def step(self, n: int = 1):
        for _ in range(n):
            self.t = self.t + self.dt
            self.half(self.t + self.dt / 2)
            self.diffusion()
            self.half(self.t + self.dt)

    def fft_only(self, n: int = 1):
        """The transforms of n steps alone (forward and inverse of both components)."""
        torch = self.torch
        for _ in range(n):
            self.u = torch.fft.ifft2(torch.fft.fft2(self.u))


def run_plain_gpu(dtype, B: int, steps: int, warmup: int, device: int, fused_value: float):
    """Times the plain cuFFT form (PlainSplitStep) on the same workload and batch as the
    fused passes: whole steps, and the transforms alone (a lower bound for any split step
    built on cuFFT), CUDA events on torch's stream, inputs larger than L2."""
    import torch
    dev = f"cuda:{device}"
    ps = PlainSplitStep(N_GRID, L_BOX, B, dtype, dev)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    ps.step(warmup)
    torch.cuda.synchronize()
    ev[0].record()
    ps.step(steps)
    ev[1].record()
    ps.fft_only(warmup)
    ev[2].record()
    ps.fft_only(steps)
    ev[3].record()
    torch.cuda.synchronize()
    ms = ev[0].elapsed_time(ev[1]) / steps
    ms_fft = ev[2].elapsed_time(ev[3]) / steps
    P = N_GRID * N_GRID
    v, vf = P * B / (ms * 1e-3), P * B / (ms_fft * 1e-3)
    del ps
    torch.cuda.empty_cache()
    return {"impl": "plain GPU split step: cuFFT (torch.fft.fft2 / ifft2 over both components and all copies) "
                    "and unfused torch elementwise kernels for the pump evaluation, half steps and 2x2 table",
            "dtype": "f64" if dtype == np.complex128 else "f32", "batch": B, "steps": steps,
            "ms_per_step": ms, "value": v, "unit": "grid-point-steps/s",
            "fft_only_ms_per_step": ms_fft, "fft_only_value": vf,
            "speedup": fused_value / v, "speedup_vs_fft_only": fused_value / vf}


def plain_single_field_ms(dtype, device: int, steps: int = 200) -> float:
    """ms per step of the plain cuFFT form on one 512^2 polariton field (no saves)."""
    import torch
    ps = PlainSplitStep(N_GRID, L_BOX, 1, dtype, f"cuda:{device}")
    ps.step(10)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    ps.step(steps)
    e1.record()
    torch.cuda.synchronize()
    del ps
    return e0.elapsed_time(e1) / steps


def plain_vs_fused_rel_l2(pkg, device: int, steps: int = 200, fp64: str = "native"):
    """rel L2 between the plain cuFFT form in FP64 and the fused passes (native FP64 or
    double-word) after `steps` steps of one pumped polariton field from u = 0."""
    import torch
    disp, nonl, pump = polariton_closures()
    z = np.zeros((N_GRID, N_GRID), np.complex128, order="F")
    prob = pkg.GrossPitaevskiiProblem((z, z.copy()), (L_BOX, L_BOX), dispersion=disp, nonlinearity=nonl, pump=pump)
    it = pkg.StrangSplittingIterator(prob, (0.0, steps * DT), dt=DT, nsaves=1, device=device, fp64=fp64)
    it.step(steps)
    got = np.stack([np.ascontiguousarray(f.T) for f in it.get_fields()])
    it.close()
    ps = PlainSplitStep(N_GRID, L_BOX, 1, np.complex128, f"cuda:{device}")
    ps.step(steps)
    ref = ps.u[:, 0].cpu().numpy()
    del ps
    torch.cuda.empty_cache()
    return float(np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-300))


TWA_GROUPS = [(64, 342), (128, 341), (256, 341)]  # 1024 trajectories over three grids


def run_twa(pkg, steps: int, tune: bool):
    """Batched truncated-Wigner ensemble: 1024 trajectories of the damped-driven scalar
    field split 342/341/341 over 64^2, 128^2 and 256^2 grids (L=64, D=|k|^2/2 - 0.1i,
    g=0.01, F=1, eta=sqrt(gamma/(2 dV)), Philox noise, FP32 fields with FP64-built tables),
    advanced by one CUDA graph.  Against: the plain per-trajectory form (one trajectory per
    handle, two-pass path, run one after another) timed on a sample and scaled."""
    T = sys.modules.get("gpe_gb300.twa") or __import__("gpe_gb300.twa", fromlist=["Ensemble"])
    A = __import__("gpe_gb300.autotune", fromlist=["tune"])
    prm = T.DampedDrivenParams()
    chunk = 50
    tuned_chunks = []
    choices = {}
    its = []
    for N, B in TWA_GROUPS:
        resident, variant = True, 0
        if tune:
            k = A.key(N, 1, "c64", B, A.gpu_name())
            resident, variant, chunk_n, timings = A.tune(
                lambda r, v, N=N, B=B: T.make_group(N, B, prm, 400, seed=N, resident=r, variant=v), k,
                trial_steps=200, variants=(0, 1), resident_ok=A.resident_fits(N, 1, 8))
            # each candidate timed alone (the group by itself in a graph, 200 steps)
            choices[f"{N}x{N}"] = {"resident": resident, "variant": variant, "steps_per_graph": chunk_n,
                                   "ms_per_step_alone": {c: ms / 200 for c, ms in timings.items()}}
            tuned_chunks.append(chunk_n)
        its.append(T.make_group(N, B, prm, steps + 400, seed=N, resident=resident, variant=variant))
    if tuned_chunks and steps % min(tuned_chunks) == 0:
        chunk = min(tuned_chunks)  # one graph serves every group: the shortest tuned chunk
    ens = T.Ensemble(its)
    ens.run(chunk, chunk)  # capture + warm-up
    ens.run(steps, chunk)
    ms = ens.last_run_ms()
    launches = ens.last_run_launches()
    ens.close()
    for it in its:
        it.close()
    ntraj = sum(B for _, B in TWA_GROUPS)
    value = ntraj * steps / (ms * 1e-3)
    # plain per-trajectory form on a sample: 3 trajectories x 100 steps per grid size
    t_plain = 0.0
    for N, B in TWA_GROUPS:
        rate = T.plain_per_trajectory_rate(N, prm, 3, 100, seed=N)
        t_plain += B * steps / rate
    plain_value = ntraj * steps / t_plain
    return {"metric": "traj-steps/s", "value": value, "unit": "traj-steps/s", "steps": steps,
            "ms": ms, "gpu_launches": int(launches), "trajectories": ntraj,
            "groups": [{"grid": [N, N], "trajectories": B} for N, B in TWA_GROUPS],
            "dtype": "f32 (tables built in FP64)", "steps_per_graph": chunk, "autotune": choices or None,
            "plain_per_trajectory": {"value": plain_value, "unit": "traj-steps/s",
                                     "sample": "3 trajectories x 100 steps per grid, one handle each, two-pass path"},
            "speedup_vs_plain_per_trajectory": value / plain_value,
            "statistics_vs_fp64_cpu_ensemble": twa_c2_statistics(pkg, steps)}


def twa_c2_statistics(pkg, steps: int = 2000, N: int = 64, ntraj: int = 342):
    """The ensemble statistics of the batched truncated-Wigner configuration, checked
    against an FP64 CPU ensemble: the 64^2 group (342 trajectories, FP32 fields, Philox
    noise) after `steps` steps on the GPU, and the same trajectories advanced in FP64 by
    the C oracle on the host cores with the same initial states and the same Philox draws
    (FP32 draws evaluated in FP64).  Reported: the per-site mean and variance of |u|^2 over
    the trajectories, their rel L2 difference between the two ensembles, and the largest
    per-trajectory rel L2 difference."""
    import math as _m
    T = sys.modules.get("gpe_gb300.twa") or __import__("gpe_gb300.twa", fromlist=["Ensemble"])
    from oracle import gpe_oracle as O
    from oracle import gpe_oracle_c as OC
    prm = T.DampedDrivenParams()
    seed = N
    it = T.make_group(N, ntraj, prm, steps, seed=seed)
    it.step(steps)
    g = it.get_fields()[0].astype(np.complex128)  # (x, y, b)
    it.close()
    u0 = T.wigner_initial(N, 0, ntraj, prm, seed, np.complex64)
    dV = (prm.L / N) ** 2
    prob = O.OracleProblem(u0=(np.ascontiguousarray(np.transpose(u0, (2, 1, 0))).astype(np.complex128),),
                           lengths=(prm.L, prm.L),
                           dispersion=lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2 - 0.5j * prm.gamma,
                           nonlin_g=np.array([[prm.g]]), pump_profile=np.ones((1, N, N), np.complex128),
                           pump_amp=lambda t: np.array([prm.F]), eta=np.array([_m.sqrt(prm.gamma / (2 * dV))]))
    t0 = time.perf_counter()
    cit = OC.CIterator(prob, (0.0, steps * prm.dt), prm.dt, 1, philox_seed=seed + 1, draw32=True)
    cit.step(steps)
    cpu_s = time.perf_counter() - t0
    c = np.transpose(cit.u[0], (2, 1, 0))  # (x, y, b)
    ng, nc = np.abs(g) ** 2, np.abs(c) ** 2
    mg, mc, vg, vc = ng.mean(-1), nc.mean(-1), ng.var(-1), nc.var(-1)
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    per_traj = max(rel(g[..., b], c[..., b]) for b in range(ntraj))
    return {"group": f"{N}x{N}, {ntraj} trajectories, {steps} steps", "gpu": "FP32 fields, Philox FP32 draws",
            "cpu": f"FP64 C oracle on {os.cpu_count()} host threads, the same initial states and Philox draws "
                   f"({cpu_s:.1f} s)",
            "mean_density_gpu": float(mg.mean()), "mean_density_cpu": float(mc.mean()),
            "density_variance_gpu": float(vg.mean()), "density_variance_cpu": float(vc.mean()),
            "rel_l2_mean_density_field": rel(mg, mc), "rel_l2_variance_field": rel(vg, vc),
            "max_rel_l2_per_trajectory": per_traj}


def run_precision_sweep(args):
    """Precision sweep: 2D Kerr on 2048^2 (L=32, u0 = exp(-|r - r0|^2 / 2^2), r0 = (16, 16),
    D = |k|^2/2, G = g|u|^2, g = +1 and -2, dt = 0.005, 1000 steps, 20 saves) in FP32,
    double-word FP64 and native FP64 on the GPU, against the FP64 oracle advanced in
    lockstep on the host: rel L2 error, norm drift and energy drift at every save."""
    import __graft_entry__ as G
    pkg = G.load_package()
    from oracle import gpe_oracle as O
    N, Lb, dt, nsteps, nsaves = args.sweep_n, 32.0, 0.005, args.sweep_steps, 20
    per = nsteps // nsaves
    dg, _ = O.grids((Lb, Lb), (N, N))
    X, Y = O.mesh(dg)
    u0c = np.exp(-((X - 16) ** 2 + (Y - 16) ** 2) / 4.0).astype(np.complex128)
    disp = lambda k, p: (k[0] ** 2 + k[1] ** 2) / 2
    report = {"metric": "precision sweep", "grid": [N, N], "steps": nsteps, "saves": nsaves, "dt": dt, "cases": []}
    cores = os.cpu_count() or 1
    for g in (1.0, -2.0):
        orc = O.OracleProblem(u0=(u0c,), lengths=(Lb, Lb), dispersion=disp, nonlin_g=np.array([[g]]))
        oit = O.OracleIterator(orc, (0.0, nsteps * dt), dt, nsaves, fft_workers=cores)
        modes = [("f32", np.complex64, "dw"), ("f64-dw", np.complex128, "dw"), ("f64-native", np.complex128, "native")]
        its = {}
        for name, dtype, fp64 in modes:
            prob = pkg.GrossPitaevskiiProblem((np.asfortranarray(u0c.T).astype(dtype),), (Lb, Lb), dispersion=disp,
                                              nonlinearity=lambda u, p, g=g: g * np.abs(u[0]) ** 2)
            its[name] = pkg.init(prob, pkg.StrangSplitting(), (0.0, nsteps * dt), dt=dt, nsaves=nsaves, fp64=fp64)
        e0 = {n: it.energy().sum() for n, it in its.items()}
        n0 = {n: it.norm()[0] for n, it in its.items()}
        rows = {n: [] for n in its}
        t = 0.0
        for s in range(nsaves):
            for _ in range(per):
                t += dt
                oit.step(t, dt)
            ref = oit.u[0]
            for n, it in its.items():
                it.step(per)
                u = np.ascontiguousarray(it.get_fields()[0].T).astype(np.complex128)
                rows[n].append({"t": round(t, 6), "rel_l2": O.rel_l2(u, ref),
                                "norm_drift": float(it.norm()[0] / n0[n] - 1),
                                "energy_drift": float((it.energy().sum() - e0[n]) / abs(e0[n]))})
        for n, it in its.items():
            it.close()
        report["cases"].append({"g": g, "modes": rows})
    print(json.dumps(report), flush=True)


def run_fno(args):
    """Learned surrogate: train the FNO (4 spectral layers, width 32, 16 modes per axis,
    BF16 GEMM operands on tcgen05, FP32 accumulation) on polariton windows (128^2, L=256,
    window = args.fno_window steps of dt=0.05) the solver generates for random constant pump
    amplitudes in [0, 6], then roll out to steady state with a plain-solver check every 10
    windows, and time that rollout against the plain solver over the same span."""
    import __graft_entry__ as G
    G.load_package()
    F = __import__("gpe_gb300.fno", fromlist=["FNO"])
    import torch
    W = args.fno_window
    t0 = time.perf_counter()
    amps, saves = F.generate_pairs(args.fno_traj, args.fno_windows, steps_per_window=W, seed=1)
    t_gen = time.perf_counter() - t0
    scale = float(np.abs(saves).max()) or 1.0
    X, Y = F.pairs_to_tensors(amps, saves, scale)
    cfg = F.FNOConfig()
    model = F.FNO(cfg, seed=0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    losses = F.train(model, X, Y, epochs=args.fno_epochs, batch=16, lr=2e-3,
                     log=lambda m: print(m, file=sys.stderr, flush=True))
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    # held-out windows: rel L2 of one surrogate window against the solver's, and of
    # persistence (u(t + W dt) ~ u(t)) for scale
    va, vs = F.generate_pairs(4, max(10, args.fno_windows // 4), steps_per_window=W, seed=99)
    VX, VY = F.pairs_to_tensors(va, vs, scale)
    with torch.no_grad():
        pred = torch.cat([model.forward(VX[i:i + 16].contiguous()) for i in range(0, VX.shape[0], 16)])
    win_err = float(torch.linalg.norm(pred - VY) / torch.linalg.norm(VY))
    persist = float(torch.linalg.norm(VX[:, :4] - VY) / torch.linalg.norm(VY))
    results = []
    for A in (2.7, 4.9):
        h1, h2, st = F.hybrid_rollout(model, A, args.fno_rollout, scale, steps_per_window=W)
        p1, p2, ms_plain = F.plain_rollout(A, args.fno_rollout, steps_per_window=W)
        ref = np.concatenate([p1.ravel(), p2.ravel()])
        got = np.concatenate([h1.ravel(), h2.ravel()])
        err = float(np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-30))
        results.append({"pump_amplitude": A, "windows": args.fno_rollout, "steps": args.fno_rollout * W,
                        "hybrid_ms": st["ms"], "plain_ms": ms_plain, "speedup_to_end_state": ms_plain / st["ms"],
                        "final_rel_l2_vs_plain": err, "checks": st["checks"], "fallbacks": st["fallbacks"],
                        "restarts": st["restarts"], "max_check_rel_l2": st["max_check_err"]})
    per_window = {}
    for B in (1, 64):
        per_window[str(B)] = {"surrogate_ms": F.surrogate_window_ms(model, B),
                              "plain_ms": F.plain_window_ms(B, steps_per_window=W)}
    print(json.dumps({"metric": "FNO surrogate hybrid rollout", "steps_per_window": W, "pairs": int(X.shape[0]),
                      "generation_s": t_gen, "train_s": t_train, "epochs": args.fno_epochs,
                      "loss_per_epoch": losses, "heldout_window_rel_l2": win_err,
                      "heldout_persistence_rel_l2": persist, "rollouts": results,
                      "window_cost_by_batch": per_window}), flush=True)


def run_gemm_bench(args):
    """Throughput of the surrogate's tcgen05 GEMM (gpe_fno_gemm: BF16 operands staged from
    FP32, FP32 accumulation in tensor memory) on the shapes the network runs at a batch of
    64 windows (pointwise channel mixing: M = 64 x 128^2 points, N = K = 32; the truncated
    DFT along x: M = 64 x 32 x 128 rows, N = 32 modes, K = 128) and on a square 8192^3
    product, against the measured cuBLAS BF16 peak.  CUDA events, after warm-up."""
    import torch
    import __graft_entry__ as G
    G.load_package()
    F = __import__("gpe_gb300.fno", fromlist=["FNO"])
    peak = None
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peak = float(json.loads(pk.read_text())["bf16_tflops"])
    shapes = [("channel mix, 64 windows", 64 * 128 * 128, 32, 32), ("x DFT, 64 windows", 64 * 32 * 128, 32, 128),
              ("square", 8192, 8192, 8192)]
    out = []
    for name, M, N, K in shapes:
        A = torch.randn(M, K, device="cuda")
        B = torch.randn(K, N, device="cuda")
        C = torch.empty(M, N, device="cuda")
        run = lambda: F.gemm(A, B, C, M, N, K, (K, 1), (N, 1), (N, 1))
        for _ in range(3):
            run()
        reps = 20 if M * N * K < 1e11 else 5
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            run()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        tf = 2.0 * M * N * K / (ms * 1e-3) / 1e12
        gbs = 4.0 * (M * K + K * N + M * N) / (ms * 1e-3) / 1e9
        out.append({"shape": name, "M": M, "N": N, "K": K, "ms": ms, "tflops": tf, "operand_gbs": gbs,
                    "frac_of_bf16_peak": (tf / peak) if peak else None})
        del A, B, C
    assert F.take_status() == 0
    print(json.dumps({"metric": "tcgen05 GEMM throughput", "bf16_peak_tflops": peak, "runs": out}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--dtype", default="c128", choices=["c128", "c64"])
    ap.add_argument("--batch", type=int, default=0)
    ap.add_argument("--fp64", default="bfp", choices=["bfp", "native", "dw"],
                    help="ComplexF64 arithmetic: FP64 with block floating point line transforms (default), FP64 "
                         "floating point throughout, or double-word on the FP32 pipes")
    ap.add_argument("--no-dw", action="store_true",
                    help="skip the FP64-floating-point and double-word measurements beside the FP64 headline")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--twa-steps", type=int, default=2000,
                    help="steps of the batched truncated-Wigner ensemble measurement (0 skips it)")
    ap.add_argument("--no-tune", action="store_true", help="skip the ensemble autotuner")
    ap.add_argument("--no-solve-run", dest="solve_run", action="store_false",
                    help="skip the full-length polariton solve() measurement")
    ap.add_argument("--plain-steps", type=int, default=20,
                    help="steps of the plain cuFFT split step timed beside the fused passes (0 skips it)")
    ap.add_argument("--anchor-steps", type=int, default=200,
                    help="steps of the scalar Kerr 1024^2 FP64 measurement (0 skips it)")
    ap.add_argument("--precision-sweep", action="store_true",
                    help="print the FP32 / FP64 precision sweep on 2D Kerr instead of the throughput line")
    ap.add_argument("--sweep-n", type=int, default=2048)
    ap.add_argument("--sweep-steps", type=int, default=1000)
    ap.add_argument("--fno", action="store_true", help="train the FNO surrogate and time the hybrid rollout")
    ap.add_argument("--fno-traj", type=int, default=100)
    ap.add_argument("--fno-windows", type=int, default=200)
    ap.add_argument("--fno-epochs", type=int, default=10)
    ap.add_argument("--fno-rollout", type=int, default=400)
    ap.add_argument("--fno-window", type=int, default=20, help="solver steps one surrogate window replaces")
    ap.add_argument("--gemm-bench", action="store_true", help="time the surrogate's tcgen05 GEMM on its shapes")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    rank, world, local_rank = dist_env()
    if args.precision_sweep:
        if rank == 0:
            run_precision_sweep(args)
        return
    if args.fno:
        if rank == 0:
            run_fno(args)
        return
    if args.gemm_bench:
        if rank == 0:
            run_gemm_bench(args)
        return
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    run_gpu(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
