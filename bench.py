"""Benchmark: einsum TFLOP/s on the CCD W intermediates (o=32, v=160), split-BF16
vs plain FP64, with the error of every result against FP64 and a sampled
CPU-oracle check.

One step = the four contractions of the CCD configuration on one GPU:
    Wmnij += 0.25 t_ijef g_mnef      (GEMM)
    Wabef += 0.25 g_mnef t_mnab      (GEMM; Wabef is 25600 x 25600, 5.24 GB)
    Wmbej += -0.5 t_jnfb g_mnef      (GENERIC)
    E      = 0.25 sum t_ijab g_ijab  (DOT, always FP64)
``value`` is the algorithmic FLOP count of a step (2*|C|*|links| per
contraction) divided by the device time of the step, for the headline
precision (split-BF16 when built, else FP64).  Inputs are larger than L2
(129 MB), so no flush is needed between steps.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Under torchrun (N > 1) each rank runs an independent replica (the path has no
exchange step); value sums the replicas' work over the max time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

O_DEF, V_DEF = 32, 160
METRIC = "einsum TFLOP/s, split-BF16 vs plain FP64 at <=1e-10 rel err; % of roofline"


def flops(o, v):
    return {"Wmnij": 2.0 * o ** 4 * v ** 2, "Wabef": 2.0 * v ** 4 * o ** 2, "Wmbej": 2.0 * o ** 3 * v ** 3,
            "E": 2.0 * o ** 2 * v ** 2}


# ncu dram__bytes_read.sum + dram__bytes_write.sum of the tensor kernel on the
# o=32, v=160 workload, mean over the step's three launches (Wmnij 3.32 GB,
# Wabef 18.17 GB, Wmbej 6.37 GB), from a separate capture of this workload.
TC_TRAFFIC_O32_V160 = 9.44e9


def tc_algorithmic_bytes(o, v, S):
    """Mean DRAM bytes per tensor-kernel launch of one step at the algorithmic
    minimum: both operands' S BF16 digit planes read once, C read and written
    once in FP64.  (M, N, K) of Wmnij, Wabef and Wmbej."""
    shapes = [(o * o, o * o, v * v), (v * v, v * v, o * o), (o * v, o * v, o * v)]
    return sum(2 * 8 * M * N + 2 * S * (M + N) * K for M, N, K in shapes) / 3


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p, "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


# ------------------------------------------------------------------ clocks --
class ClockSampler:
    """Samples nvidia-smi during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    INTERVAL_MS = 50

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", str(self.INTERVAL_MS)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # nvidia-smi takes a while to print its first line: start the work only once it samples
            t0 = time.time()
            while not self.lines and self.proc.poll() is None and time.time() - t0 < 3.0:
                time.sleep(0.01)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            parts = [p.strip() for p in l.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------------- our arm --
def ccd_step(eg, T, W, precision, slices, timers=None, report=None, only=None):
    """The four contractions (results stay on the device).  When ``report`` is
    a dict it receives the split-form accounting of the Wabef contraction;
    ``only`` names a single contraction to run."""
    import torch
    t, g = T["t"], T["g_oovv"]

    def run(name, fn):
        if only is not None and name != only:
            return
        if timers is not None:
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            timers.setdefault(name, []).append((e0, e1))
        else:
            fn()

    run("Wmnij", lambda: eg.einsum(1.0, "mnij", W["Wmnij"], 0.25, "ijef", t, "mnef", g, precision=precision,
                                   slices=slices))
    run("Wabef", lambda: eg.einsum(1.0, "abef", W["Wabef"], 0.25, "mnef", g, "mnab", t, precision=precision,
                                   slices=slices))
    if report is not None and only in (None, "Wabef"):
        report.update(eg.last_split_report())
    run("Wmbej", lambda: eg.einsum(1.0, "mbej", W["Wmbej"], -0.5, "jnfb", t, "mnef", g, precision=precision,
                                   slices=slices))
    run("E", lambda: eg.einsum(0.0, "", W["E"], 0.25, "ijab", t, "ijab", g))


def fresh_W(T):
    import torch
    return {"Wmnij": T["g_oooo"].clone(), "Wabef": T["g_vvvv"].clone(), "Wmbej": T["g_ovvo"].clone(),
            "E": torch.zeros((), dtype=torch.float64, device="cuda")}


def rel_err(x, ref):
    import torch
    num = torch.linalg.vector_norm((x - ref).reshape(-1))
    den = torch.linalg.vector_norm(ref.reshape(-1))
    return float(num / den) if float(den) > 0 else float(num)


def oracle_sample_check(T, Ws, rows=4):
    """CPU-oracle values of the first `rows` rows of each W's increment (the contraction
    term, C_prefactor 0), against the increment each GPU result in `Ws` (name -> W dict)
    made: rows m < 4 of 32 (Wmnij, Wmbej) and a < 4 of 160 (Wabef), plus the energy."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    t = T["t"].cpu().numpy()
    g = T["g_oovv"].cpu().numpy()
    init = {"Wmnij": "g_oooo", "Wabef": "g_vvvv", "Wmbej": "g_ovvo"}
    refs = {}
    ref = np.zeros_like(T["g_oooo"][:rows].cpu().numpy())
    oracle.einsum("mnij", ref, 0.0, 0.25, "ijef", t, "mnef", np.ascontiguousarray(g[:rows]))
    refs["Wmnij"] = ref
    ref = np.zeros_like(T["g_vvvv"][:rows].cpu().numpy())
    oracle.einsum("abef", ref, 0.0, 0.25, "mnef", g, "mnab", np.ascontiguousarray(t[:, :, :rows]))
    refs["Wabef"] = ref
    ref = np.zeros_like(T["g_ovvo"][:rows].cpu().numpy())
    oracle.einsum("mbej", ref, 0.0, -0.5, "jnfb", t, "mnef", np.ascontiguousarray(g[:rows]))
    refs["Wmbej"] = ref
    e = np.zeros(())
    oracle.einsum("", e, 0.0, 0.25, "ijab", t, "ijab", g)
    out = {}
    for name, W in Ws.items():
        res = {}
        for k, ref in refs.items():
            got = (W[k][:rows] - T[init[k]][:rows]).cpu().numpy()
            res[k] = oracle.rel_fro(got, ref)
        res["E"] = abs(float(W["E"].item()) - float(e)) / max(abs(float(e)), 1e-300)
        out[name] = res
    out["rows"] = rows
    return out


def oracle_threads():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    return int(oracle.lib().oracle_num_threads())


def cpu_sample(o, v, seed=0, cores=None, b_rows=None, a_rows=None):
    """The oracle's CCD step on a bounded sample; returns (seconds, algorithmic
    flops of the sample, description).

    The reference's generic loop runs OpenMP over the outermost target index
    only (Backends/BaseAlgebra.hpp:70-80), so the Wmnij and Wmbej slabs keep at
    least as many rows of m as the host has cores (all of them on a box with
    o or fewer cores): every core works, as it would on the whole step.
    Wmbej may also be cut along b, Wabef (a dgemm, threaded by OpenBLAS) along
    a; E is computed whole."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from einsums_gb300 import workloads
    cores = cores or host_cores()
    T = workloads.ccd_inputs(o, v, seed=seed, backend="numpy", with_vvvv=False)
    t, g = T["t"], T["g_oovv"]
    m_rows = min(o, max(1, cores))
    b_rows = min(v, b_rows or v)
    a_rows = min(v, a_rows or max(1, v // 32))
    W1 = np.zeros((m_rows, o, o, o))
    W2 = np.zeros((a_rows, v, v, v))
    W3 = np.zeros((m_rows, b_rows, v, o))
    E = np.zeros(())
    g_m = np.ascontiguousarray(g[:m_rows])
    t_a = np.ascontiguousarray(t[:, :, :a_rows])
    t_b = np.ascontiguousarray(t[:, :, :, :b_rows])
    t0 = time.perf_counter()
    oracle.einsum("mnij", W1, 1.0, 0.25, "ijef", t, "mnef", g_m)
    oracle.einsum("abef", W2, 1.0, 0.25, "mnef", g, "mnab", t_a)
    oracle.einsum("mbej", W3, 1.0, -0.5, "jnfb", t_b, "mnef", g_m)
    oracle.einsum("", E, 0.0, 0.25, "ijab", t, "ijab", g)
    dt = time.perf_counter() - t0
    f = flops(o, v)
    fl = f["Wmnij"] * m_rows / o + f["Wabef"] * a_rows / v + f["Wmbej"] * m_rows / o * b_rows / v + f["E"]
    full = sum(f.values())
    desc = (f"oracle CCD step on a sample of {100 * fl / full:.1f}% of the step's flops: Wmnij rows m<{m_rows} "
            f"of {o} ({100 * m_rows / o:.0f}%), Wabef rows a<{a_rows} of {v} ({100 * a_rows / v:.1f}%), Wmbej rows "
            f"m<{m_rows}, b<{b_rows} ({100 * m_rows * b_rows / (o * v):.1f}%), full E; numpy OpenBLAS dgemm + "
            f"OpenMP generic loop over m on {oracle_threads()} threads")
    return dt, fl, desc


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def host_cpu():
    """The host CPU the baseline ran on: architecture, model (or the Arm implementer/part ids), cores usable."""
    import platform
    info = {"machine": platform.machine(), "cores_usable": host_cores(), "cores_online": os.cpu_count()}
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                key, _, val = line.partition(":")
                key, val = key.strip(), val.strip()
                if key in ("model name", "CPU implementer", "CPU part") and key not in info:
                    info[key] = val
    except OSError:
        pass
    return info


def reduce_max_ms(ms, world, device):
    """Max over ranks of a per-rank time: the job is as slow as its slowest rank."""
    if world == 1:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_tflops(step_flops, ms, world):
    """Whole-job throughput: every rank processed one step of ``step_flops`` per ``ms``."""
    return world * step_flops / (ms * 1e-3) / 1e12


def run_ours(args, rank, world):
    import torch

    import einsums_gb300 as eg
    from einsums_gb300 import _lib, core, workloads

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    lib = _lib.load()
    o, v = args.o, args.v
    F = flops(o, v)
    step_flops = sum(F.values())

    # FP64 roofline denominator, measured on this device.
    import ctypes
    dfma, dmma, probe_mhz = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    _lib.check(lib.eg_measure_fp64_peak_clock(ctypes.byref(dfma), ctypes.byref(dmma), ctypes.byref(probe_mhz)))
    # The FP64 pipe retires one DFMA warp instruction per 16 SM clocks (2 lanes,
    # 4 flop per clock per SM: ncu instruction counts over pipe-active cycles,
    # for the DFMA probe and for k_contract_f64 alike); the probe loops keep it
    # 84-97 % busy, so the roofline takes that rate at the probe's clock.
    n_sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    fp64_pipe = 4.0 * n_sms * probe_mhz.value * 1e6 / 1e12
    fp64_peak = max(dfma.value, dmma.value, fp64_pipe)

    T = workloads.ccd_inputs(o, v, seed=args.seed, backend="cuda")
    torch.cuda.synchronize()

    # Which precision is the headline: split-BF16 when the library has it.
    headline = "split_bf16"
    try:
        Wt = fresh_W(T)
        ccd_step(eg, T, Wt, "split_bf16", args.slices)
        torch.cuda.synchronize()
        del Wt
    except _lib.NotSupportedError:
        headline = "fp64"

    # Accuracy: one step each precision from the same initial W.
    W64 = fresh_W(T)
    ccd_step(eg, T, W64, "fp64", 0)
    errors = {}
    split_report = None
    checked = {"fp64": W64}
    if headline == "split_bf16":
        Ws = fresh_W(T)
        split_report = {}
        ccd_step(eg, T, Ws, "split_bf16", args.slices, report=split_report)
        for k in ("Wmnij", "Wabef", "Wmbej"):
            errors[k] = rel_err(Ws[k] - T[{"Wmnij": "g_oooo", "Wabef": "g_vvvv", "Wmbej": "g_ovvo"}[k]],
                                W64[k] - T[{"Wmnij": "g_oooo", "Wabef": "g_vvvv", "Wmbej": "g_ovvo"}[k]])
        checked["split_bf16"] = Ws
    torch.cuda.synchronize()
    oracle_err = oracle_sample_check(T, checked) if rank == 0 else None
    del checked
    Ws = None

    def timed(precision, steps, warmup, timers=None):
        W = fresh_W(T)
        for _ in range(warmup):
            ccd_step(eg, T, W, precision, args.slices)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        n0 = ctypes.c_uint64()
        _lib.check(lib.eg_kernel_launches(ctypes.byref(n0)))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            ccd_step(eg, T, W, precision, args.slices, timers)
        e1.record()
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        n1 = ctypes.c_uint64()
        _lib.check(lib.eg_kernel_launches(ctypes.byref(n1)))
        del W
        return e0.elapsed_time(e1) / steps, int(n1.value - n0.value)

    # Plain FP64 reference timing (fewer steps: it is ~100x slower).
    fp64_steps = 1 if headline == "split_bf16" else args.steps
    fp64_timers = {}
    ms_fp64, _ = timed("fp64", fp64_steps, 1, fp64_timers)

    timers = {}
    gpu_idx = int(os.environ.get("LOCAL_RANK", 0))
    lib.eg_profile_enable(1)
    lib.eg_profile_reset()
    with ClockSampler(gpu_idx) as clk:
        ms, launches = timed(headline, args.steps, args.warmup, timers)
    buf = ctypes.create_string_buffer(1 << 16)
    _lib.check(lib.eg_profile_summary(buf, len(buf)))
    lib.eg_profile_enable(0)
    kernels = {}
    for line in buf.value.decode().strip().split("\n"):
        if line:
            name, cnt, tot = line.split(",")
            kernels[name] = {"launches": int(cnt), "total_ms": float(tot)}

    ms = reduce_max_ms(ms, world, "cuda")

    per_contraction = {k: sum(a.elapsed_time(b) for a, b in vals) / len(vals) for k, vals in timers.items()}
    per_contraction_fp64 = {k: sum(a.elapsed_time(b) for a, b in vals) / len(vals) for k, vals in fp64_timers.items()}
    value = job_tflops(step_flops, ms, world)
    fp64_value = step_flops / (ms_fp64 * 1e-3) / 1e12

    # Dominant kernel roofline.
    pk, pk_kind = peaks()
    if headline == "split_bf16":
        dom = max((k for k in kernels if k.startswith("k_tc")), key=lambda k: kernels[k]["total_ms"], default=None)
    else:
        dom = "k_contract_f64" if "k_contract_f64" in kernels else max(kernels, key=lambda k: kernels[k]["total_ms"])
    roof = None
    if dom:
        d = kernels[dom]
        avg_ms = d["total_ms"] / d["launches"]
        if headline == "split_bf16":
            pairs = (split_report or {}).get("slice_pairs", 0)
            # bf16 flops issued by the tensor kernel per launch (slice pairs x 2MNK over the GEMM-shaped W's);
            # the kernel profile spans the warm-up and the timed steps
            launches_per_step = d["launches"] / (args.steps + args.warmup)
            alg = pairs * (F["Wmnij"] + F["Wabef"] + F["Wmbej"]) / launches_per_step
            ach = alg / (avg_ms * 1e-3) / 1e12
            # the burst peak (cuBLAS timed alone) unless the clock record shows the
            # power cap, then the sustained one measured under it
            capped = "sw_power_cap" in (clk.summary().get("reasons") or [])
            peak = pk.get("bf16_tflops_sustained" if capped else "bf16_tflops", 1700.0 if capped else 1900.0)
            roof = {"kernel": dom, "bound": "tensor", "achieved": ach, "peak": peak, "unit": "TFLOP/s",
                    "frac": ach / peak, "traffic": None,
                    "peak_source": f"bf16 {'sustained (power cap seen)' if capped else 'burst'}, {pk_kind}"}
            if (o, v) == (32, 160) and (split_report or {}).get("slices") == 5:
                # DRAM bytes per tensor-kernel launch, mean over the step's three
                # launches, from one ncu capture of this workload
                # (dram__bytes_read.sum + dram__bytes_write.sum); algorithmic bytes
                # per launch (digit planes read once, C read and written once) are
                # 4.16 GB; the kernel moves 2.3x that (digit-plane panels re-read
                # through L2 by the output tiles that share them).
                roof["traffic"] = TC_TRAFFIC_O32_V160
                roof["traffic_unit"] = ("bytes per launch, mean of the step's 3 launches, from an ncu capture of "
                                        "this workload (dram__bytes_read.sum + dram__bytes_write.sum), "
                                        "not measured in this run")
                roof["algorithmic_bytes"] = tc_algorithmic_bytes(o, v, 5)
        else:
            alg = F["Wabef"]
            ach = alg / (per_contraction["Wabef"] * 1e-3) / 1e12
            roof = {"kernel": dom, "bound": "tensor", "achieved": ach, "peak": fp64_peak, "unit": "TFLOP/s",
                    "frac": ach / fp64_peak, "traffic": None,
                    "peak_source": "fp64: FP64 pipe rate (4 flop per clock per SM) at the probe's measured SM clock"}

    # End to end through the public API: host inputs in, host results out.
    # every rank runs it (replicas), timed between barriers; the slowest rank sets the time
    e2e = run_e2e(eg, T, headline, args, o, v, step_flops, world=world)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        # three runs of the sample (10-30 s of CPU work on the GPU machine's host); the median rate
        runs = [cpu_sample(o, v, seed=args.seed) for _ in range(3)]
        dt = statistics.median(r[0] for r in runs)
        fl, desc = runs[0][1], runs[0][2]
        cpu = {"value": fl / dt / 1e12, "unit": "TFLOP/s", "cores": oracle_threads(), "kind": "port",
               "sample": desc + "; median of 3 runs", "seconds": dt, "cpu": host_cpu()}

    # The other configurations at their full sizes, after the timed region, with
    # their oracle parity checks (rank 0 of a single-GPU run only).
    suites = None
    if rank == 0 and world == 1 and not args.no_suites:
        del T, W64
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        suites = run_suites_inline(eg)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64 (split into bf16 slices, fp32 tensor accumulate)"
            if headline == "split_bf16" else "f64",
            "data": "synthetic (seeded torch generator on device; CCD amplitudes/integrals as specified)",
            "config": {"workload": f"CCD W intermediates o={o} v={v}: Wmnij, Wabef (GEMM), Wmbej (GENERIC), E (DOT)",
                       "precision": headline, "slices": (split_report or {}).get("slices"),
                       "l2": f"inputs larger than L2 (Wabef {v ** 4 * 8 / 1e9:.2f} GB read+written per step); no flush"
                       if v ** 4 * 8 > 129e6 else "inputs smaller than L2 (129 MB): a reduced case, not the headline",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "plain_fp64": {"value": fp64_value, "ms_per_step": ms_fp64, "per_contraction_ms": per_contraction_fp64,
                           "fp64_peak_tflops": fp64_peak, "dfma_tflops": dfma.value, "dmma_tflops": dmma.value,
                           "fp64_pipe_tflops": fp64_pipe, "fp64_probe_sm_mhz": probe_mhz.value},
            "split_vs_fp64_speedup": value / world / fp64_value if headline == "split_bf16" else None,
            "per_contraction_ms": per_contraction, "kernels": kernels, "kernels_steps": args.steps + args.warmup,
            "error_vs_fp64": errors, "error_vs_oracle_sample": oracle_err, "split_report": split_report,
            "roofline": roof, "cpu_baseline": cpu, "clocks": clk.summary(), "e2e": e2e, "gpu_launches": launches,
            "suites": suites,
        }
        print(json.dumps(line))


def run_e2e(eg, T, precision, args, o, v, step_flops, chunks=8, return_outputs=False, world=1):
    """Same step through the public API with host buffers: every step copies all
    of its inputs in from pinned host memory and all four results back, inside
    the timed region.  The copies are pipelined the way a caller of the API
    would, on three streams (uploads, contractions, read-backs):

    * t, g_oovv, g_oooo and g_ovvo (0.6 GB) go to one of three device sets;
      Wmnij, Wmbej and E are computed from them and read back.
    * Wabef's 5.2 GB initial value g_vvvv and its result move in ``chunks``
      slabs of rows a: slab j uploads into one of four device slab buffers, its
      contraction W[a0:a1] += 0.25 g_mnef t_mn[a0:a1]b runs as soon as it has
      landed, and it is read back as soon as that is done.  Each output element
      is computed exactly as in the whole contraction (its row and column and
      the K sum are unchanged), so the slabs reproduce it bit for bit.

    A set or slab buffer is refilled only after the read-back of its previous
    contents has finished.  With several ranks (replicas) every rank runs this
    between barriers; the slowest rank's time and all ranks' work and bytes make
    the reported figures."""
    import torch
    small = ("t", "g_oovv", "g_oooo", "g_ovvo")
    host = {k: T[k].cpu().pin_memory() for k in small + ("g_vvvv",)}
    out = {"Wmnij": torch.empty_like(host["g_oooo"]).pin_memory(),
           "Wmbej": torch.empty_like(host["g_ovvo"]).pin_memory(),
           "Wabef": torch.empty_like(host["g_vvvv"]).pin_memory(),
           "E": torch.empty((), dtype=torch.float64).pin_memory()}
    nv = host["g_vvvv"].shape[0]
    chunks = max(1, min(chunks, nv))
    bounds = [(nv * j // chunks, nv * (j + 1) // chunks) for j in range(chunks)]
    rows_max = max(a1 - a0 for a0, a1 in bounds)
    sets = []
    for _ in range(3):
        dev = {k: torch.empty_like(T[k]) for k in small}
        W = {"Wmnij": dev["g_oooo"], "Wmbej": dev["g_ovvo"], "E": torch.zeros((), dtype=torch.float64, device="cuda")}
        sets.append((dev, W, torch.cuda.Event()))  # event: the set's last use has finished
    slabs = [(torch.empty((rows_max,) + tuple(host["g_vvvv"].shape[1:]), dtype=torch.float64, device="cuda"),
              torch.cuda.Event()) for _ in range(4)]
    h2d = sum(x.numel() * 8 for x in host.values())
    d2h = sum(x.numel() * 8 for x in out.values())
    s_in, s_cmp, s_out = torch.cuda.Stream(), torch.cuda.Stream(), torch.cuda.Stream()
    inputs_of = {"Wmnij": ("t", "g_oovv", "g_oooo"), "Wmbej": ("t", "g_oovv", "g_ovvo"), "E": ("t", "g_oovv")}
    counter = [0]

    def step(i):
        dev, W, freed = sets[i % 3]
        landed, done = {}, {}
        s_in.wait_event(freed)
        with torch.cuda.stream(s_in):
            for k in small:
                dev[k].copy_(host[k], non_blocking=True)
                landed[k] = torch.cuda.Event()
                landed[k].record(s_in)
        with torch.cuda.stream(s_cmp):
            for w in ("Wmnij", "Wmbej", "E"):
                for k in inputs_of[w]:
                    s_cmp.wait_event(landed[k])
                ccd_step(eg, {"t": dev["t"], "g_oovv": dev["g_oovv"]}, W, precision, args.slices, only=w)
                done[w] = torch.cuda.Event()
                done[w].record(s_cmp)
        with torch.cuda.stream(s_out):
            for w in ("Wmnij", "Wmbej", "E"):
                s_out.wait_event(done[w])
                out[w].copy_(W[w], non_blocking=True)
        for a0, a1 in bounds:
            buf, buf_free = slabs[counter[0] % len(slabs)]
            counter[0] += 1
            wc = buf[:a1 - a0]
            s_in.wait_event(buf_free)
            with torch.cuda.stream(s_in):
                wc.copy_(host["g_vvvv"][a0:a1], non_blocking=True)
                ev_in = torch.cuda.Event()
                ev_in.record(s_in)
            with torch.cuda.stream(s_cmp):
                s_cmp.wait_event(ev_in)
                eg.einsum(1.0, "abef", wc, 0.25, "mnef", dev["g_oovv"], "mnab", dev["t"][:, :, a0:a1, :],
                          precision=precision, slices=args.slices)
                ev_c = torch.cuda.Event()
                ev_c.record(s_cmp)
            with torch.cuda.stream(s_out):
                s_out.wait_event(ev_c)
                out["Wabef"][a0:a1].copy_(wc, non_blocking=True)
                buf_free.record(s_out)
        freed.record(s_out)

    steps = max(1, min(args.steps, 3)) if precision == "fp64" else args.steps
    for i in range(max(1, args.warmup if precision != "fp64" else 1)):
        step(i)
    torch.cuda.synchronize()
    # the link rates, before the timed steps: they write into the result buffers,
    # which the timed steps then fill with the results
    link = link_rates(host["g_vvvv"], out["Wabef"], [b for b, _ in slabs], rows_max, s_in, s_out)
    if world > 1:
        torch.distributed.barrier()
    # Three passes of `steps` steps each; the reported time is the median pass.  The
    # host link of this machine is shared, and single passes have been seen to take
    # twice the link floor while the copy rates measured just before were normal.
    passes = []
    for _ in range(1 if precision == "fp64" else 3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s_in)
        for i in range(steps):
            step(i)
        e1.record(s_out)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        passes.append(reduce_max_ms(e0.elapsed_time(e1) / steps, world, "cuda"))
    ms = sorted(passes)[len(passes) // 2]
    floor_ms = (h2d + d2h) / (link["both_gbs"] * 1e9) * 1e3
    res = {"value": job_tflops(step_flops, ms, world), "unit": "TFLOP/s", "h2d_bytes_per_step": world * h2d,
           "d2h_bytes_per_step": world * d2h, "ms_per_step": ms, "steps": steps, "passes_ms_per_step": passes,
           "link_gbs": link, "link_floor_ms": floor_ms, "frac_of_link_floor": floor_ms / ms,
           "pipelining": f"uploads, contractions and read-backs on three streams; three sets of the 0.6 GB inputs; "
                         f"Wabef in {chunks} slabs of rows a through four slab buffers"}
    if return_outputs:
        return res, out
    return res


def link_rates(h_in, h_out, bufs, rows, s_in, s_out, reps=2):
    """Host-link copy rates (GB/s) measured just before the timed e2e steps with the same
    pinned buffers and streams: Wabef's initial value up in row slabs, its result down,
    and both at once -- the e2e step's floor is its bytes over the concurrent rate."""
    import torch
    nv = h_in.shape[0]
    bounds = [(a0, min(a0 + rows, nv)) for a0 in range(0, nv, rows)]

    def up(k):
        for j, (a0, a1) in enumerate(bounds):
            bufs[(j + k) % len(bufs)][:a1 - a0].copy_(h_in[a0:a1], non_blocking=True)

    def down(k):
        for j, (a0, a1) in enumerate(bounds):
            h_out[a0:a1].copy_(bufs[(j + k + 2) % len(bufs)][:a1 - a0], non_blocking=True)

    def timed(fn_in, fn_out):
        torch.cuda.synchronize()
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(s_in)
        s_out.wait_event(e0)
        for k in range(reps):
            if fn_in:
                with torch.cuda.stream(s_in):
                    fn_in(k)
            if fn_out:
                with torch.cuda.stream(s_out):
                    fn_out(k)
        e1.record(s_in)
        e2.record(s_out)
        torch.cuda.synchronize()
        return max(e0.elapsed_time(e1), e0.elapsed_time(e2)) / reps

    nbytes = h_in.numel() * 8
    t_up = timed(up, None)
    t_down = timed(None, down)
    t_both = timed(up, down)
    return {"h2d_gbs": nbytes / t_up / 1e6, "d2h_gbs": nbytes / t_down / 1e6, "both_gbs": 2 * nbytes / t_both / 1e6,
            "bytes": nbytes}


# --------------------------------------------------------- reference arm --
def run_reference(args, rank, world):
    if rank != 0:
        return
    o, v = args.o, args.v
    for _ in range(args.warmup):
        cpu_sample(o, v, seed=args.seed)
    times, fl, desc = [], 0.0, ""
    for _ in range(args.steps):
        dt, fl, desc = cpu_sample(o, v, seed=args.seed)
        times.append(dt)
    dt = sum(times) / len(times)
    val = fl / dt / 1e12
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": val, "unit": "TFLOP/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (numpy PCG64, seeded)",
        "config": {"workload": f"CCD W intermediates o={o} v={v}: Wmnij, Wabef (GEMM), Wmbej (GENERIC), E (DOT)",
                   "precision": "fp64 (reference CPU einsum restated: OpenBLAS dgemm + OpenMP generic loop)"},
        "cpu_baseline": {"value": val, "unit": "TFLOP/s", "cores": host_cores(), "kind": "port", "sample": desc,
                         "cpu": host_cpu()},
        "e2e": {"value": val, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


# ------------------------------------------------------------ config suite --
def _events():
    import torch
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def _time(fn, reps=3, warm=1):
    import torch
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    e0, e1 = _events()
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def suite_fock(eg, n=100):
    """Config 1: F = 2 J - K with J = einsum(pq <- pqrs, rs) (GEMV) and K = einsum(pq <- prqs, rs) (GENERIC)."""
    import numpy as np
    import torch
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from einsums_gb300 import workloads
    g_np, D_np = workloads.fock_inputs(n, seed=0)
    g, D = torch.tensor(g_np, device="cuda"), torch.tensor(D_np, device="cuda")
    F = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    out = {"config": f"Fock two-electron build n={n}"}
    flop = 2.0 * n ** 4
    for prec in ("fp64", "split_bf16"):
        algJ = eg.einsum(0.0, "pq", F, 2.0, "pqrs", g, "rs", D, precision=prec)
        msJ = _time(lambda: eg.einsum(0.0, "pq", F, 2.0, "pqrs", g, "rs", D, precision=prec))
        msK = _time(lambda: eg.einsum(1.0, "pq", F, -1.0, "prqs", g, "rs", D, precision=prec))
        F.zero_()
        eg.einsum(0.0, "pq", F, 2.0, "pqrs", g, "rs", D, precision=prec)
        algK = eg.einsum(1.0, "pq", F, -1.0, "prqs", g, "rs", D, precision=prec)
        # J and K are GEMV-shaped (N = 1): a split request runs the FP64 kernels (0 slices reported)
        slices = eg.last_split_report()["slices"]
        out[prec] = {"J_ms": msJ, "K_ms": msK, "J_alg": algJ, "K_alg": algK, "split_slices": slices,
                     "J_tflops": flop / msJ / 1e9, "K_tflops": flop / msK / 1e9,
                     "J_gbs": 8.0 * n ** 4 / msJ / 1e6, "K_gbs": 8.0 * n ** 4 / msK / 1e6,
                     "F": F.cpu().numpy().copy()}
    Fref = np.zeros((n, n))
    t0 = time.perf_counter()
    oracle.einsum("pq", Fref, 0.0, 2.0, "pqrs", g_np, "rs", D_np)
    tJ = time.perf_counter() - t0
    t0 = time.perf_counter()
    oracle.einsum("pq", Fref, 1.0, -1.0, "prqs", g_np, "rs", D_np)
    tK = time.perf_counter() - t0
    for prec in ("fp64", "split_bf16"):
        out[prec]["error_vs_oracle"] = oracle.rel_fro(out[prec].pop("F"), Fref)
    # the whole F = 2 J - K: the two einsum calls against the symmetric-integral entry point
    # (reads the canonical eighth of g; 0.75 n^4 FP64 multiply-adds against 2 n^4)
    def two_calls():
        eg.einsum(0.0, "pq", F, 2.0, "pqrs", g, "rs", D)
        eg.einsum(1.0, "pq", F, -1.0, "prqs", g, "rs", D)
    ms_two = _time(two_calls, reps=20, warm=3)
    Fs = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    sym = {"two_einsum_calls_ms": ms_two, "canonical_bytes": 8.0 * n ** 4 / 8, "fma": 0.75 * n ** 4,
           "note": "equiv TFLOP/s counts the 4 n^4 flops of the two general contractions"}
    for prec in ("fp64", "split_bf16"):
        ms_sym = _time(lambda: eg.fock_jk_symmetric(Fs, g, D, F_prefactor=0.0, precision=prec), reps=20, warm=3)
        sym[prec] = {"ms": ms_sym, "speedup_vs_two_calls": ms_two / ms_sym,
                     "error_vs_oracle": oracle.rel_fro(Fs.cpu().numpy(), Fref),
                     "equiv_tflops": 4.0 * n ** 4 / ms_sym / 1e9}
        if prec == "split_bf16":
            sym[prec]["split_report"] = eg.last_split_report()
    out["F_2J_minus_K_symmetric"] = sym
    out["cpu_oracle"] = {"J_ms": tJ * 1e3, "K_ms": tK * 1e3, "cores": host_cores()}
    return out


def _graph_ms(fns):
    """Device time per call of the calls in `fns`, captured once into a CUDA graph
    and replayed (no host overhead per call)."""
    import torch
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        for fn in fns:
            fn()
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        for fn in fns:
            fn()
    g.replay()
    torch.cuda.synchronize()
    e0, e1 = _events()
    e0.record()
    g.replay()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / len(fns)


def suite_permute(eg, sizes=(32, 64, 128, 256)):
    """Config 3a: all 24 rank-4 permutations at n^4, bit-exact.  Each permutation is
    timed through the API (host work included) and, as a compiled plan, on the device
    alone (a CUDA graph of plan executions over buffers that together exceed L2)."""
    import itertools

    import numpy as np
    import torch
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    res = {"config": "rank-4 permute sweep, all 24 permutations", "sizes": {}}
    pk, _ = peaks()
    for n in sizes:
        gen = torch.Generator(device="cuda")
        gen.manual_seed(n)
        A = torch.randn((n, n, n, n), generator=gen, dtype=torch.float64, device="cuda")
        C = torch.empty_like(A)
        back = torch.empty_like(A) if n >= 128 else None
        times, dev_times, exact = [], [], True
        A_np = A.cpu().numpy() if n <= 64 else None
        # rotating (A, C) pairs so that the replayed plan streams from HBM, not L2
        nbuf = max(1, -(-320 * 2 ** 20 // (16 * n ** 4)))
        rot = [(A, C)] + [(A.clone(), torch.empty_like(A)) for _ in range(nbuf - 1)]
        for perm in itertools.permutations(range(4)):
            Cl = "".join("abcd"[p] for p in perm)
            ms = _time(lambda: eg.permute(0.0, Cl, C, 1.0, "abcd", A), reps=3, warm=1)
            times.append(ms)
            plan = eg.compile_permute(0.0, Cl, C, 1.0, "abcd", A)
            dev_times.append(_graph_ms([lambda a=a, c=c: plan.execute(c, a) for a, c in rot] * max(1, 8 // nbuf)))
            plan.close()
            if A_np is not None:
                ref = np.empty([n] * 4)
                oracle.permute(Cl, ref, 0.0, 1.0, "abcd", A_np)
                exact &= bool(np.array_equal(C.cpu().numpy().view(np.uint64), ref.view(np.uint64)))
            else:
                # size-independent property: the inverse permutation restores A bit for bit
                eg.permute(0.0, "abcd", back, 1.0, Cl, C)
                exact &= bool(torch.equal(back.view(torch.int64), A.view(torch.int64)))
        bytes_ = 16.0 * n ** 4
        dev_mean = sum(dev_times) / len(dev_times)
        res["sizes"][str(n)] = {"api_mean_ms": sum(times) / len(times), "api_min_ms": min(times),
                                "api_max_ms": max(times), "api_mean_gbs": bytes_ / (sum(times) / len(times)) / 1e6,
                                "device_mean_ms": dev_mean, "device_max_ms": max(dev_times),
                                "device_mean_gbs": bytes_ / dev_mean / 1e6,
                                "device_worst_gbs": bytes_ / max(dev_times) / 1e6, "bit_exact": exact,
                                "frac_of_hbm": bytes_ / dev_mean / 1e6 / pk["hbm_gbs"]}
        del A, C, back, rot
        torch.cuda.empty_cache()
    return res


def suite_contraction(eg, sizes=(64, 128)):
    """Config 3b: C[i,k,j,l] = sum_mn A[i,m,j,n] B[m,k,n,l]; FP64 and split S = 3..6."""
    import numpy as np
    import torch
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from einsums_gb300 import workloads
    res = {"config": "generic contraction ikjl <- imjn * mknl", "sizes": {}}
    for n in sizes:
        A, B = workloads.sweep_contraction_inputs(n, seed=n, backend="cuda")
        C64 = torch.zeros((n, n, n, n), dtype=torch.float64, device="cuda")
        flop = 2.0 * n ** 6
        alg = eg.einsum(0.0, "ikjl", C64, 1.0, "imjn", A, "mknl", B)
        ms64 = _time(lambda: eg.einsum(0.0, "ikjl", C64, 1.0, "imjn", A, "mknl", B), reps=1, warm=0)
        entry = {"algorithm": alg, "fp64": {"ms": ms64, "tflops": flop / ms64 / 1e9}}
        # the oracle on a slab of C (rows i < ri, k < rk): the reference's generic loop
        ri, rk = (16, n) if n <= 64 else (1, 8)
        ref = np.zeros((ri, rk, n, n))
        oracle.einsum("ikjl", ref, 0.0, 1.0, "imjn", np.ascontiguousarray(A[:ri].cpu().numpy()), "mknl",
                      np.ascontiguousarray(B[:, :rk].cpu().numpy()))
        entry["fp64"]["error_vs_oracle_slab"] = oracle.rel_fro(C64[:ri, :rk].cpu().numpy(), ref)
        entry["fp64"]["oracle_slab"] = f"i<{ri}, k<{rk}"
        C = torch.zeros_like(C64)
        for S in (3, 4, 5, 6):
            ms = _time(lambda: eg.einsum(0.0, "ikjl", C, 1.0, "imjn", A, "mknl", B, precision="split_bf16",
                                         slices=S), reps=2, warm=1)
            err = float(torch.linalg.vector_norm(C - C64) / torch.linalg.vector_norm(C64))
            entry[f"split_S{S}"] = {"ms": ms, "tflops": flop / ms / 1e9, "error_vs_fp64": err,
                                    "speedup_vs_fp64": ms64 / ms}
        res["sizes"][str(n)] = entry
        del A, B, C, C64
        torch.cuda.empty_cache()
    return res


def suite_batched(eg, count=2048):
    """Config 4: 2048 contractions C_k[a,b] = sum_ij A_k[i,j,a] B_k[i,j,b], uneven extents."""
    import numpy as np
    import torch
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from einsums_gb300 import workloads
    shapes = workloads.batched_shapes(count, seed=0)
    As, Bs = workloads.batched_inputs(shapes, seed=1, backend="cuda")
    Cs = [torch.zeros((a, b), dtype=torch.float64, device="cuda") for (i, j, a, b) in shapes]
    flop = sum(2.0 * i * j * a * b for (i, j, a, b) in shapes)
    res = {"config": f"{count} uneven contractions ab <- ija * ijb", "gflop": flop / 1e9}
    As_np = [x.cpu().numpy() for x in As]
    Bs_np = [x.cpu().numpy() for x in Bs]
    refs = []
    for k in range(count):
        ref = np.zeros(Cs[k].shape)
        oracle.einsum("ab", ref, 0.0, 1.0, "ija", As_np[k], "ijb", Bs_np[k])
        refs.append(ref)
    for prec in ("fp64", "split_bf16"):
        t0 = time.perf_counter()
        plan = eg.GroupedPlan(0.0, "ab", Cs, 1.0, "ija", As, "ijb", Bs, precision=prec)
        t_plan = time.perf_counter() - t0
        ms_graph = _time(plan.execute, reps=5, warm=2)
        errs = [oracle.rel_fro(c.cpu().numpy(), ref) for c, ref in zip(Cs, refs)]
        plan.close()

        def per_item():
            for k in range(count):
                eg.einsum(0.0, "ab", Cs[k], 1.0, "ija", As[k], "ijb", Bs[k], precision=prec)
        ms_loop = _time(per_item, reps=1, warm=1)
        res[prec] = {"grouped_graph_ms": ms_graph, "grouped_tflops": flop / ms_graph / 1e9,
                     "plan_build_s": t_plan, "one_launch_per_contraction_ms": ms_loop,
                     "speedup_vs_per_item": ms_loop / ms_graph, "items_checked_vs_oracle": len(errs),
                     "max_error_vs_oracle": max(errs)}
    return res


def suite_autograd(eg, o=24, v=96):
    """Config 5: L = ||einsum(mbej <- jnfb, mnef)(t, g) - R||^2 with adjoint kernels."""
    import numpy as np
    import torch
    from einsums_gb300 import autograd, workloads
    T = workloads.ccd_inputs(o, v, seed=0, backend="cuda", with_vvvv=False)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(9)
    R = torch.randn((o, v, v, o), generator=gen, dtype=torch.float64, device="cuda")
    flop = 3 * 2.0 * o ** 3 * v ** 3
    res = {"config": f"autograd Wmbej o={o} v={v}", "gflop_fwd_bwd": flop / 1e9}
    grads = {}
    for prec in ("fp64", "split_bf16"):
        t = T["t"].clone().requires_grad_(True)
        g = T["g_oovv"].clone().requires_grad_(True)

        def step():
            t.grad = None
            g.grad = None
            C = autograd.einsum_ag("mbej", "jnfb", "mnef", t, g, precision=prec)
            ((C - R) ** 2).sum().backward()
        ms = _time(step, reps=3, warm=1)
        grads[prec] = (t.grad.clone(), g.grad.clone())
        res[prec] = {"fwd_bwd_ms": ms, "tflops": flop / ms / 1e9}
    for name, a, b in (("dt", grads["split_bf16"][0], grads["fp64"][0]), ("dg", grads["split_bf16"][1], grads["fp64"][1])):
        res[f"split_error_{name}"] = float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))
    # central differences (h = 1e-6) on 64 seeded entries of t and of g
    rng = np.random.default_rng(4)
    h = 1e-6
    worst = 0.0
    tt, gg = T["t"], T["g_oovv"]
    for which, X in ((0, tt), (1, gg)):
        grad = grads["fp64"][which]
        gmax = float(grad.abs().max())
        for f in rng.choice(X.numel(), size=64, replace=False):
            idx = np.unravel_index(int(f), tuple(X.shape))
            Xp, Xm = X.clone(), X.clone()
            Xp[idx] += h
            Xm[idx] -= h
            args_p = (Xp, gg) if which == 0 else (tt, Xp)
            args_m = (Xm, gg) if which == 0 else (tt, Xm)
            Cp = autograd.einsum_ag("mbej", "jnfb", "mnef", *args_p).detach()
            Cm = autograd.einsum_ag("mbej", "jnfb", "mnef", *args_m).detach()
            fd = float(((Cp - Cm) * (Cp + Cm - 2.0 * R)).sum()) / (2 * h)
            an = float(grad[idx])
            worst = max(worst, abs(fd - an) / max(abs(an), 1e-3 * gmax))
    res["fd_worst_relative_error"] = worst
    res["fd_entries"] = {"t": 64, "g": 64, "h": h}
    # the reference CPU einsum of the forward and the two adjoint patterns
    # (every index of these patterns is in C or in both operands, so the C++
    # generic loop and the Python plan semantics agree)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    t_np, g_np, R_np = tt.cpu().numpy(), gg.cpu().numpy(), R.cpu().numpy()
    Cn = np.zeros((o, v, v, o))
    oracle.einsum("mbej", Cn, 0.0, 1.0, "jnfb", t_np, "mnef", g_np)
    dC = 2.0 * (Cn - R_np)
    dt_ref = np.zeros_like(t_np)
    oracle.einsum("jnfb", dt_ref, 0.0, 1.0, "mbej", dC, "mnef", g_np)
    dg_ref = np.zeros_like(g_np)
    oracle.einsum("mnef", dg_ref, 0.0, 1.0, "mbej", dC, "jnfb", t_np)
    res["fp64_vs_oracle"] = {"dt": oracle.rel_fro(grads["fp64"][0].cpu().numpy(), dt_ref),
                             "dg": oracle.rel_fro(grads["fp64"][1].cpu().numpy(), dg_ref)}
    res["split_vs_oracle"] = {"dt": oracle.rel_fro(grads["split_bf16"][0].cpu().numpy(), dt_ref),
                              "dg": oracle.rel_fro(grads["split_bf16"][1].cpu().numpy(), dg_ref)}
    return res


def suite_gemm(eg, m=8192, k=1024, c_along_m=True, reps=3):
    """One split-BF16 GEMM-shaped contraction C[b,a] (or C[a,b]) = sum_k A[a,k] B[b,k],
    M = N = m: the Wabef shape at a chosen size, for timing the tensor kernel and for
    profiling it on a case smaller than the CCD step.  Not part of the default line."""
    import torch
    gen = torch.Generator(device="cuda")
    gen.manual_seed(m + k)
    A = torch.randn((m, k), generator=gen, dtype=torch.float64, device="cuda")
    B = torch.randn((m, k), generator=gen, dtype=torch.float64, device="cuda")
    C = torch.zeros((m, m), dtype=torch.float64, device="cuda")
    Cl = "ba" if c_along_m else "ab"
    run = lambda: eg.einsum(1.0, Cl, C, 1.0, "ak", A, "bk", B, precision="split_bf16")
    ms = _time(run, reps=reps, warm=1)
    pairs = eg.last_split_report()["slice_pairs"]
    return {"config": f"split-BF16 GEMM M=N={m} K={k}, C contiguous along {'M' if c_along_m else 'N'}",
            "ms": ms, "bf16_tflops_incl_splitting": pairs * 2.0 * m * m * k / ms / 1e9}


SUITES = ("fock", "permute", "contraction", "batched", "autograd")


def run_suites_inline(eg):
    """Every other configuration at its full size; a failing suite records its
    error instead of losing the headline line."""
    import torch
    out = {}
    for name in SUITES:
        t0 = time.perf_counter()
        try:
            r = SUITE_FNS[name](eg)
        except Exception as exc:  # noqa: BLE001 -- reported in the line
            r = {"error": f"{type(exc).__name__}: {exc}"}
        r["wall_s"] = time.perf_counter() - t0
        out[name] = r
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
    return out


def run_suite(args):
    import torch

    import einsums_gb300 as eg
    torch.cuda.set_device(0)
    which = args.suite.split(",") if args.suite != "all" else list(SUITES)
    fns = SUITE_FNS
    sizes = tuple(int(x) for x in args.sizes.split(",")) if args.sizes else None
    for name in which:
        t0 = time.perf_counter()
        if sizes and name in ("permute", "contraction"):
            r = fns[name](eg, sizes)
        elif name == "batched" and args.items:
            r = fns[name](eg, count=args.items)
        elif name == "gemm":
            mk = sizes or (8192, 1024)
            r = fns[name](eg, m=mk[0], k=mk[1], reps=args.steps)
        else:
            r = fns[name](eg)
        r["suite"] = name
        r["wall_s"] = time.perf_counter() - t0
        print(json.dumps(r), flush=True)


SUITE_FNS = {"fock": suite_fock, "permute": suite_permute, "contraction": suite_contraction, "batched": suite_batched,
             "autograd": suite_autograd, "gemm": suite_gemm}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--o", type=int, default=O_DEF)
    ap.add_argument("--v", type=int, default=V_DEF)
    ap.add_argument("--slices", type=int, default=0)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline sample")
    ap.add_argument("--no-suites", action="store_true",
                    help="skip the other configurations that follow the headline in the same line")
    ap.add_argument("--suite", default=None,
                    help="measure the other configurations instead (all, or a comma list of "
                         "fock,permute,contraction,batched,autograd; gemm: one split-form GEMM of "
                         "--sizes M,K, --steps calls); one JSON line each")
    ap.add_argument("--sizes", default=None, help="extents for the permute / contraction sweeps, e.g. 64,128")
    ap.add_argument("--items", type=int, default=0, help="contractions in the batched suite (default 2048)")
    args = ap.parse_args()
    if args.suite:
        run_suite(args)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        torch.distributed.init_process_group("nccl")
    try:
        run_ours(args, rank, world)
    finally:
        if world > 1:
            import torch
            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
