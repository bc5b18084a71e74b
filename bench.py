#!/usr/bin/env python3
"""Throughput of the HEOM propagation path on GB300: ADO-updates/s.

One ADO-update is one ADO's right-hand side evaluated once with its fused
stage combination (RK4/LSRK4: 4 per step; Dormand-Prince: 7 per attempt,
rejected attempts included).  A bench "step" is one full propagation of the
workload from its initial state to t_final.

Default workload: the 7-site exciton aggregate (n=7, 14 modes, depth 4,
3060 ADOs), Dormand-Prince atol=rtol=1e-8 to 1 ps, seeded synthetic
Hamiltonian.  The chosen form is mixed precision (FP32 bulk products, FP64
state / accumulation / error norm / step control); its final state is
checked against the FP64 path (max |delta rho| <= 1e-6), and the FP64 plain
form is timed beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "exciton7": dict(maker="exciton_7site", solver="rkdp", t_final=1000.0, kw=dict(dt=0.1, atol=1e-8, rtol=1e-8),
                     cpu_sample_t=1000.0),
    "spin_boson": dict(maker="spin_boson", solver="rk4", t_final=10.0, kw=dict(dt=0.005), cpu_sample_t=10.0),
    "aggregate24": dict(maker="aggregate_24site", solver="lsrk4", t_final=1000.0, kw=dict(dt=0.5),
                        cpu_sample_t=1.0),
}
L2_FLUSH_BYTES = 512 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="exciton7")
    ap.add_argument("--form", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip the FP64 comparison run (profiling)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock, throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() in ("active", "1", "yes"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic(workload, form):
    """DRAM bytes per stage launch from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        d = json.load(f)
    return d.get(f"{workload}/{form}")


def cpu_baseline(wl, p, seconds_hint=True):
    """The CPU restatement of the reference path (oracle port) on a bounded sample."""
    import oracle
    cores = os.cpu_count() or 1
    orc = oracle.Oracle("port")
    t_s = wl["cpu_sample_t"]
    t0 = time.perf_counter()
    _, st = orc.solve(p, p.rho0_ground(), [0.0, t_s], solver=wl["solver"], threads=cores, with_stats=True,
                      **wl["kw"])
    el = time.perf_counter() - t0
    rate = st["rhs"] * p.n_hrchy() / el
    return {"value": rate, "unit": "ADO-updates/s", "cores": cores, "kind": "port", "seconds": el,
            "sample": f"{wl['maker']} {wl['solver']} t=0..{t_s} ({st['rhs']} RHS x {p.n_hrchy()} ADOs, "
                      f"{el:.2f} s)"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from libheom_gb300 import configs
    wl = WORKLOADS[args.workload]
    p = getattr(configs, wl["maker"])()
    vals, secs = [], []
    cb = None
    for i in range(max(args.warmup, 0) + args.steps):
        cb = cpu_baseline(wl, p)
        if i >= args.warmup:
            vals.append(cb["value"])
            secs.append(cb["seconds"])
    v = float(np.mean(vals))
    ms = 1000.0 * float(np.mean(secs))
    line = {"impl": "reference", "metric": "ADO-updates/s", "value": v, "unit": "ADO-updates/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128 (f64)",
            "data": "synthetic (seeded)",
            "config": {"workload": args.workload, "n_hrchy": p.n_hrchy(), "n_level": p.n_level,
                       "solver": wl["solver"], "sample": "bounded CPU sample per step"},
            "cpu_baseline": {**cb, "value": v},
            "e2e": {"value": v, "unit": "ADO-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_ours(args):
    import torch

    import libheom_gb300 as lh
    from libheom_gb300 import configs, roofline

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    wl = WORKLOADS[args.workload]
    p = getattr(configs, wl["maker"])()
    nh, n2 = p.n_hrchy(), p.n_level ** 2
    N = nh * n2
    mixed = args.form == "mixed"
    stream = torch.cuda.Stream(device=dev)

    def make(form_prec):
        q = lh.from_params(p, precision=form_prec, stream=stream.cuda_stream)
        return q, lh.qme_solver(q, lh.SOLVERS[wl["solver"]]())

    q, qs = make("mixed" if mixed else "fp64")
    rho0 = torch.from_numpy(p.rho0_ground()).to(dev)
    rho = torch.empty_like(rho0)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    t_list = [0.0, wl["t_final"]]

    def step(solver_obj):
        with torch.cuda.stream(stream):
            rho.copy_(rho0)
        solver_obj.solve_device(rho.data_ptr(), t_list, None, wl["kw"])

    fma_peaks = lh.probe_fma_peaks()
    # accuracy of the chosen form against the FP64 path (parity-tested against the oracle)
    max_err = None
    plain = None
    if mixed and not args.no_plain:
        q64, qs64 = make("fp64")
        step(qs64)
        torch.cuda.synchronize()
        ref_final = rho.clone()
        st64 = qs64.stats()
        step(qs)
        torch.cuda.synchronize()
        max_err = float((rho - ref_final).abs().max().item())
        # plain FP64 form timed once (after its warm-up above)
        with torch.cuda.stream(stream):
            flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step(qs64)
        e1.record(stream)
        torch.cuda.synchronize()
        ms64 = e0.elapsed_time(e1)
        tm64 = qs64.timing()
        avg64 = 1e-3 * tm64["busy_ms"] / max(tm64["kernels"], 1)
        fl64 = roofline.flops_per_element(p) * N / avg64 / 1e12
        plain = {"value": st64["rhs"] * nh / (ms64 / 1e3), "ms_per_step": ms64, "attempts": st64["attempts"],
                 "avg_stage_kernel_us": 1e6 * avg64,
                 "roofline": {"bound": "fp64 pipe", "achieved": fl64, "peak": fma_peaks[0], "unit": "TFLOP/s",
                              "frac": fl64 / fma_peaks[0], "peak_source": "measured (heomgb_probe_fma_peaks)"}}
        del qs64, q64

    for _ in range(args.warmup):
        with torch.cuda.stream(stream):
            flush.zero_()
        step(qs)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    launches0 = lh.launch_count()
    times, rhs, busy, kernels = [], 0, 0.0, 0
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()  # inputs are L2-resident otherwise: flush between steps
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step(qs)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
        st = qs.stats()
        tm = qs.timing()
        rhs += st["rhs"]
        busy += tm["busy_ms"]
        kernels += tm["kernels"]
    launches = lh.launch_count() - launches0
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = sampler.stop()
    total_ms = float(sum(times))
    if world > 1:
        t = torch.tensor([total_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    updates = rhs * nh * world
    value = updates / (total_ms / 1e3)

    # end to end through the public API with host buffers (pinned), copies inside
    rho_h = torch.empty(rho0.shape, dtype=torch.complex128, pin_memory=True)
    e2e_ms = []
    for i in range(max(1, min(3, args.steps))):
        rho_h.copy_(torch.from_numpy(p.rho0_ground()))
        arr = rho_h.numpy()
        t0 = time.perf_counter()
        qs.solve(arr, t_list, None, wl["kw"])
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    e2e_rhs = qs.stats()["rhs"]
    e2e = {"value": e2e_rhs * nh * world / (statistics.median(e2e_ms) / 1e3), "unit": "ADO-updates/s",
           "h2d_bytes_per_step": 16 * N, "d2h_bytes_per_step": 16 * N}

    # roofline of the fused stage kernel
    bpe, launches_per_unit = roofline.bytes_per_element(wl["solver"], mixed)
    alg_bytes_per_launch = bpe * N / launches_per_unit
    avg_launch_s = (busy / 1e3) / max(kernels, 1)
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes_per_launch / avg_launch_s / 1e9
    flops = roofline.flops_per_element(p) * N
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": profile_traffic(args.workload, args.form), "peak_source": peak_kind,
            "kernel": "k_rhs_diag (fused RHS + stage epilogue)",
            "alg_bytes_per_launch": alg_bytes_per_launch, "avg_launch_us": avg_launch_s * 1e6,
            "alg_flops_per_launch": flops,
            "achieved_tflops": flops / avg_launch_s / 1e12,
            "fma_peaks_tflops": {"fp64": fma_peaks[0], "fp32": fma_peaks[1]},
            "note": "state is L2-resident within a propagation; avg launch time includes intra-graph gaps"}
    line = {"metric": "ADO-updates/s", "value": value, "unit": "ADO-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c64 bulk / c128 state" if mixed else "c128 (f64)", "data": "synthetic (seeded)",
            "config": {"workload": args.workload, "n_level": p.n_level, "n_modes": p.n_modes,
                       "max_depth": p.max_depth, "n_hrchy": nh, "solver": wl["solver"], "t_final": wl["t_final"],
                       "kwargs": wl["kw"], "form": args.form, "parallelism": f"replicas x{world}",
                       "l2": "flushed between steps (512 MiB write)"},
            "max_abs_err_vs_fp64": max_err, "plain_fp64": plain,
            "attempts_per_step": rhs // max(1, args.steps) // (7 if wl["solver"] == "rkdp" else 4),
            "gpu_launches": launches, "e2e": e2e, "roofline": roof, "clocks": clocks}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(wl, p)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
