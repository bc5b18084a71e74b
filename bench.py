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
checked against the FP64 path (max |delta rho| <= 1e-6), the FP64 plain form
is timed beside it, and both forms are compared with the CPU oracle's states
on the CPU-baseline sample (for the default workload: the whole propagation
to 1 ps).  Other workloads: --workload spin_boson | batched |
aggregate24 | exciton7_ensemble (16 disorder realisations of the 7-site
aggregate in one batch, RK4 dt = 1 fs).

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
                     cpu_sample_t=1000.0, default_steps=20),
    "spin_boson": dict(maker="spin_boson", solver="rk4", t_final=10.0, kw=dict(dt=0.005), cpu_sample_t=10.0),
    "batched": dict(maker="batched_sweep", solver="rk4", t_final=20.0, kw=dict(dt=0.005), cpu_sample_t=1.0,
                    cpu_sample_instances=24),
    "aggregate24": dict(maker="aggregate_24site", solver="lsrk4", t_final=1000.0, kw=dict(dt=0.5),
                        cpu_sample_t=0.5),
    # 16 disorder realisations of the 7-site aggregate in one batch (RK4: batches take fixed steps)
    "exciton7_ensemble": dict(maker="exciton_7site_ensemble", solver="rk4", t_final=1000.0, kw=dict(dt=1.0),
                              cpu_sample_t=20.0, cpu_sample_instances=1),
}
L2_FLUSH_BYTES = 512 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: 20 for the 7-site workload, whose step is short, else 5)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="exciton7")
    ap.add_argument("--form", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip the FP64 comparison run (profiling)")
    ap.add_argument("--no-secondary", action="store_true",
                    help="skip the bounded 24-site secondary measurement of the default workload")
    ap.add_argument("--t-final", type=float, default=None,
                    help="propagate to this time instead of the workload's (short profiling runs)")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = WORKLOADS[args.workload].get("default_steps", 5)
    return args


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
                                          "--format=csv,noheader,nounits", "-lms", "50"],
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


class Workload:
    """The instances of a workload (one model, or a batch) and their sizes."""

    def __init__(self, name, rank=0):
        from libheom_gb300 import configs
        from libheom_gb300.dist import shard_seed
        self.name = name
        self.wl = WORKLOADS[name]
        maker = getattr(configs, self.wl["maker"])
        # a batched sweep gives every rank its own seeded shard (weak scaling);
        # a single model is replicated
        if self.wl["maker"] == "batched_sweep":
            made = maker(seed=shard_seed(2, rank))
        elif self.wl["maker"] == "exciton_7site_ensemble":
            made = maker(seed=1 + 16 * rank)
        else:
            made = maker()
        self.ps = made if isinstance(made, list) else [made]
        self.batched = len(self.ps) > 1
        self.n_hrchy = sum(p.n_hrchy() for p in self.ps)
        self.N = sum(p.n_hrchy() * p.n_level ** 2 for p in self.ps)
        self.promoted = 0

    def rho0(self):
        return np.concatenate([p.rho0_ground().ravel() for p in self.ps])

    def make(self, precision, stream):
        import libheom_gb300 as lh
        qmes = [lh.from_params(p, precision=precision, stream=stream) for p in self.ps]
        if self.batched:
            # models that the range guard keeps in FP64 form a second
            # sub-batch; group them so each sub-batch is contiguous on the device
            order = sorted(range(len(qmes)), key=lambda i: qmes[i].get_precision()["effective"] == "fp64")
            self.ps = [self.ps[i] for i in order]
            qmes = [qmes[i] for i in order]
            self.promoted = sum(q.get_precision()["effective"] == "fp64" for q in qmes) if precision == "mixed" \
                else self.promoted
        solver = lh.SOLVERS[self.wl["solver"]]()
        qs = lh.batch_solver(qmes, solver) if self.batched else lh.qme_solver(qmes[0], solver)
        return qmes, qs

    def errors(self, got, ref):
        """Accuracy of `got` against the FP64 result `ref` (flat concatenated states).

        rho0: max |delta rho_0| (system density matrix) over the instances whose
        FP64 rho_0 stays physical (|rho_0| <= 1 + 1e-3; some seeded batch
        instances diverge under the reference's algorithm itself); all_ados_rel:
        max over those instances of max |delta rho| / max |rho| taken over all
        of an instance's ADOs."""
        off = 0
        e0, ea, stable = 0.0, 0.0, 0
        for p in self.ps:
            n2 = p.n_level ** 2
            size = p.n_hrchy() * n2
            r, g = ref[off:off + size], got[off:off + size]
            off += size
            if not np.all(np.isfinite(r)) or np.abs(r[:n2]).max() > 1.0 + 1e-3:
                continue
            stable += 1
            e0 = max(e0, float(np.abs(g[:n2] - r[:n2]).max()))
            ea = max(ea, float(np.abs(g - r).max() / (np.abs(r).max() + 1e-300)))
        return {"rho0": e0, "all_ados_rel": ea, "instances_checked": stable, "instances": len(self.ps)}

    def flops_per_launch(self):
        from libheom_gb300 import roofline
        return sum(roofline.flops_per_element(p) * p.n_hrchy() * p.n_level ** 2 for p in self.ps)

    def describe(self):
        if not self.batched:
            p = self.ps[0]
            return {"n_level": p.n_level, "n_modes": p.n_modes, "max_depth": p.max_depth, "n_hrchy": p.n_hrchy()}
        counts = [p.n_hrchy() for p in self.ps]
        return {"instances": len(self.ps), "n_level": sorted({p.n_level for p in self.ps}),
                "max_depth": [min(p.max_depth for p in self.ps), max(p.max_depth for p in self.ps)],
                "n_hrchy_total": self.n_hrchy, "n_hrchy_per_instance": [min(counts), max(counts)],
                "kept_fp64_by_range_guard": self.promoted}


def cpu_baseline(w: Workload, keep_states: bool = False):
    """The CPU restatement of the reference path (oracle port) on a bounded sample.

    keep_states: also return the oracle's final states of the sampled
    instances (key "_final", removed before printing), the reference the
    engine's own results are compared with at the sample's horizon."""
    import oracle
    cores = os.cpu_count() or 1
    orc = oracle.Oracle("port")
    wl = w.wl
    t_s = wl["cpu_sample_t"]
    ps = w.ps[:wl.get("cpu_sample_instances", 1)] if w.batched else w.ps
    rhs_upd = 0
    finals = []
    t0 = time.perf_counter()
    for p in ps:
        rho_t, st = orc.solve(p, p.rho0_ground(), [0.0, t_s], solver=wl["solver"], threads=cores, with_stats=True,
                              **wl["kw"])
        rhs_upd += st["rhs"] * p.n_hrchy()
        if keep_states:
            finals.append(rho_t[-1])
    el = time.perf_counter() - t0
    out = {"value": rhs_upd / el, "unit": "ADO-updates/s", "cores": cores, "kind": "port", "seconds": el,
           "sample": f"{w.name}: {len(ps)} instance(s), {wl['solver']} t=0..{t_s}, {rhs_upd} ADO-updates, "
                     f"{el:.2f} s"}
    if keep_states:
        out["_final"] = (ps, t_s, finals)
    return out


def oracle_errors(w: Workload, sample, precision: str):
    """Error of the engine's `precision` form against the oracle's states of
    the CPU sample (same instances, same horizon), through the host API.

    rho0: max |delta rho_0|; all_ados_rel: max |delta rho| / max |rho| over all
    of an instance's ADOs; both over the instances whose oracle rho_0 stays
    physical (|rho_0| <= 1 + 1e-3)."""
    import libheom_gb300 as lh
    ps, t_s, finals = sample
    qmes = [lh.from_params(p, precision=precision) for p in ps]
    solver = lh.SOLVERS[w.wl["solver"]]()
    qs = lh.batch_solver(qmes, solver) if len(ps) > 1 else lh.qme_solver(qmes[0], solver)
    rho = np.concatenate([p.rho0_ground().ravel() for p in ps])
    qs.solve(rho, [0.0, t_s], None, w.wl["kw"])
    off = qs.offsets() if len(ps) > 1 else [0, rho.size]
    e0, ea, checked = 0.0, 0.0, 0
    for i, (p, ref) in enumerate(zip(ps, finals)):
        got = rho[off[i]:off[i + 1]].reshape(ref.shape)
        if not np.all(np.isfinite(ref)) or np.abs(ref[0]).max() > 1.0 + 1e-3:
            continue
        checked += 1
        e0 = max(e0, float(np.abs(got[0] - ref[0]).max()))
        ea = max(ea, float(np.abs(got - ref).max() / (np.abs(ref).max() + 1e-300)))
    qs.close()
    return {"rho0": e0, "all_ados_rel": ea, "instances_checked": checked, "instances": len(ps), "t": t_s}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    w = Workload(args.workload)
    vals, secs = [], []
    cb = None
    for i in range(max(args.warmup, 0) + args.steps):
        cb = cpu_baseline(w)
        if i >= args.warmup:
            vals.append(cb["value"])
            secs.append(cb["seconds"])
    v = float(np.mean(vals))
    line = {"impl": "reference", "metric": "ADO-updates/s", "value": v, "unit": "ADO-updates/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * float(np.mean(secs)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128 (f64)",
            "data": "synthetic (seeded)",
            "config": {"workload": args.workload, "solver": w.wl["solver"], **w.describe(),
                       "sample": "bounded CPU sample per step"},
            "cpu_baseline": {**cb, "value": v},
            "e2e": {"value": v, "unit": "ADO-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def secondary_aggregate24(stream, fma_peaks, steps=3):
    """The 24-site aggregate (n=24, K=48, depth 3, 20825 ADOs), LSRK4 dt = 0.5 fs,
    on a bounded sample of its 2000-step run: 100 steps (t = 0..50 fs) per solve,
    both forms, the state resident in HBM, L2 flushed between solves.  Reports
    ADO-updates/s, the stage kernel's time per launch and its HBM roofline."""
    import torch

    import libheom_gb300 as lh
    from libheom_gb300 import configs, roofline
    p = configs.aggregate_24site()
    N = p.n_hrchy() * p.n_level ** 2
    rho0 = torch.from_numpy(p.rho0_ground().ravel()).cuda()
    rho = torch.empty_like(rho0)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    peak, peak_kind = measured_peaks()
    out = {"workload": "aggregate24 (n=24, K=48, depth 3, 20825 ADOs), lsrk4 dt=0.5",
           "sample": "100 steps (t = 0..50 fs) of the 2000-step run per solve", "solves_timed": steps}
    for form in ("mixed", "fp64"):
        qs = lh.qme_solver(lh.from_params(p, precision=form, stream=stream.cuda_stream), lh.lsrk4())
        t_list = [0.0, 50.0]

        def solve():
            with torch.cuda.stream(stream):
                rho.copy_(rho0)
            qs.solve_device(rho.data_ptr(), t_list, None, {"dt": 0.5})

        solve()  # warm-up (graph capture)
        ms, busy, rhs = [], 0.0, 0
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            solve()
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
            busy += qs.timing()["busy_ms"]
            rhs += qs.stats()["rhs"]
        upd = qs.stats()["ado_updates"]
        avg_s = 1e-3 * busy / max(rhs, 1)
        bpe, per_unit = roofline.bytes_per_element("lsrk4", form == "mixed")
        alg = bpe * N / per_unit
        tune = qs.tuning()
        entry = {"value": upd / (statistics.median(ms) / 1e3), "unit": "ADO-updates/s",
                 "ms_per_solve": statistics.median(ms), "avg_stage_kernel_us": 1e6 * avg_s,
                 "kernel": "k_rhs_sites" if tune.get("sites") else "k_rhs_diag", "tuning": tune}
        if form == "mixed":
            entry["roofline"] = {"bound": "hbm", "achieved": alg / avg_s / 1e9, "peak": peak, "unit": "GB/s",
                                 "frac": alg / avg_s / 1e9 / peak, "peak_source": peak_kind,
                                 "alg_bytes_per_launch": alg, "traffic": profile_traffic("aggregate24", "mixed")}
        else:
            fl = roofline.flops_per_element(p) * N / avg_s / 1e12
            entry["roofline"] = {"bound": "fp64 pipe", "achieved": fl, "peak": fma_peaks[0], "unit": "TFLOP/s",
                                 "frac": fl / fma_peaks[0], "peak_source": "measured (heomgb_probe_fma_peaks)"}
        out[form] = entry
        qs.close()
    out["mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    return out


def north_star_exciton7(stream, plain_ms, chosen_ms, steps=3):
    """The 7-site workload to t_final = 1 ps (Dormand-Prince, atol = rtol = 1e-8)
    in four forms: plain FP64 depth 4 (the drop-in), mixed depth 4 (the chosen
    form), and depth 3 with plain truncation and with the learned closure
    (mixed; the closure trained here by the library's kernels on 8 seeded
    depth-6 trajectories, about 20 s).  Each form's error is max over t = 0,
    100, ..., 1000 fs of max |delta rho_0| against the depth-6 FP64 solve of
    the same aggregate (3060 vs 38760 ADOs), its time the median of `steps`
    device solves."""
    import torch

    import libheom_gb300 as lh
    from libheom_gb300 import configs
    from libheom_gb300 import terminator as T
    kw = dict(dt=0.1, atol=1e-8, rtol=1e-8)
    t_out = [100.0 * i for i in range(11)]

    def rho0_traj(p, precision, mlp=None):
        q = lh.from_params(p, precision=precision)
        if mlp is not None:
            T.attach(q, mlp)
        qs = lh.qme_solver(q, lh.rkdp())
        rho = p.rho0_ground()
        out = []
        qs.solve(rho, t_out, lambda t: out.append(rho[0].copy()), dict(kw))
        return np.array(out), qs, q

    def timed(qs, p):
        r0 = torch.from_numpy(p.rho0_ground().ravel()).cuda()
        r = torch.empty_like(r0)
        ms = []
        for i in range(steps + 1):
            with torch.cuda.stream(stream):
                r.copy_(r0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            qs.solve_device(r.data_ptr(), [0.0, 1000.0], None, dict(kw))
            e1.record(stream)
            torch.cuda.synchronize()
            if i > 0:
                ms.append(e0.elapsed_time(e1))
        return statistics.median(ms)

    t0 = time.perf_counter()
    rng = np.random.default_rng(31)
    deep = [T.sample_exciton7(rng, 6)[0] for _ in range(8)]
    X, Tt, _ = T.make_dataset(deep, 3, list(np.arange(20.0, 200.01, 20.0)), dt=1.0)
    din, dout = T.dims(deep[0])
    mlp = T.MLP(din, 256, dout, seed=3)
    mlp.set_loss(1, dout // 2)
    T.train(mlp, X, Tt, epochs=8, batch=4096, lr=1e-3, cosine=True)
    train_s = time.perf_counter() - t0
    ref, _, _ = rho0_traj(configs.exciton_7site(depth=6), "fp64")
    out = {"workload": "exciton7, rkdp atol=rtol=1e-8 to 1 ps", "reference": "depth-6 FP64 solve (38760 ADOs)",
           "error": "max over t = 0..1000 fs (every 100 fs) of max |delta rho_0| vs the reference",
           "closure_training_s": train_s, "closure_training": "8 depth-6 trajectories, 8 epochs"}
    forms = {}
    for name, depth, prec, use in (("plain_fp64_depth4", 4, "fp64", False), ("mixed_depth4", 4, "mixed", False),
                                   ("mixed_depth3_truncated", 3, "mixed", False),
                                   ("mixed_depth3_closure", 3, "mixed", True)):
        p = configs.exciton_7site(depth=depth)
        traj, qs, _ = rho0_traj(p, prec, mlp if use else None)
        ms = plain_ms if name == "plain_fp64_depth4" else (chosen_ms if name == "mixed_depth4" else timed(qs, p))
        forms[name] = {"ms_to_t_final": ms, "err_vs_depth6": float(np.abs(traj - ref).max()),
                       "n_hrchy": p.n_hrchy()}
    for f in forms.values():
        f["speedup_vs_plain_fp64"] = plain_ms / f["ms_to_t_final"]
    out["forms"] = forms
    return out


def run_ours(args):
    import torch

    import libheom_gb300 as lh
    from libheom_gb300 import roofline

    from libheom_gb300.dist import job_throughput
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    w = Workload(args.workload, rank)
    wl = w.wl
    N = w.N
    mixed = args.form == "mixed"
    stream = torch.cuda.Stream(device=dev)
    qmes, qs = w.make("mixed" if mixed else "fp64", stream.cuda_stream)
    rho0 = torch.from_numpy(w.rho0()).to(dev)
    rho = torch.empty_like(rho0)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    if args.t_final is not None:
        wl["t_final"] = args.t_final
    t_list = [0.0, wl["t_final"]]
    per_rhs = 7 if wl["solver"] == "rkdp" else 4

    def step(solver_obj):
        with torch.cuda.stream(stream):
            rho.copy_(rho0)
        solver_obj.solve_device(rho.data_ptr(), t_list, None, wl["kw"])

    fma_peaks = lh.probe_fma_peaks()
    # accuracy of the chosen form against the FP64 path (parity-tested against the oracle)
    max_err = None
    plain = None
    if mixed and not args.no_plain:
        q64, qs64 = w.make("fp64", stream.cuda_stream)
        step(qs64)
        torch.cuda.synchronize()
        ref_final = rho.clone()
        st64 = qs64.stats()
        step(qs)
        torch.cuda.synchronize()
        max_err = w.errors(rho.cpu().numpy(), ref_final.cpu().numpy())
        # plain FP64 form: timed over repeats (after its warm-up above), median reported
        n_rep = max(5, min(args.steps, 20)) if args.workload == "exciton7" else max(3, min(args.steps, 5))
        ms64s, busy64, rhs64 = [], 0.0, 0
        for _ in range(n_rep):
            with torch.cuda.stream(stream):
                flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step(qs64)
            e1.record(stream)
            torch.cuda.synchronize()
            ms64s.append(e0.elapsed_time(e1))
            busy64 += qs64.timing()["busy_ms"]
            rhs64 += qs64.stats()["rhs"]
        ms64 = statistics.median(ms64s)
        avg64 = 1e-3 * busy64 / max(rhs64, 1)  # per stage evaluated (an interval launch runs many)
        fl64 = w.flops_per_launch() / avg64 / 1e12
        plain = {"value": st64["ado_updates"] / (ms64 / 1e3), "ms_per_step": ms64,
                 "ms_per_step_min_max": [min(ms64s), max(ms64s)], "repeats": n_rep,
                 "attempts": st64["attempts"], "avg_stage_kernel_us": 1e6 * avg64, "tuning": qs64.tuning(),
                 "roofline": {"bound": "fp64 pipe", "achieved": fl64, "peak": fma_peaks[0], "unit": "TFLOP/s",
                              "frac": fl64 / fma_peaks[0], "peak_source": "measured (heomgb_probe_fma_peaks)"}}
        qs64.close()
        del qs64, q64

    def alg_bytes_of(tm, st):
        """Algorithmic bytes of the stage kernels of one solve (per sub-batch
        precision), counted over the stage launches that did work (right-hand
        sides evaluated); launches of a captured graph replayed after the
        interval ended return at once and move no data."""
        parts = tm.get("parts") or [dict(tm, precision="mixed" if mixed else "fp64", elements=N, rhs=st["rhs"])]
        tot = 0.0
        for part in parts:
            bpe, per_unit = roofline.bytes_per_element(wl["solver"], part["precision"] == "mixed")
            tot += bpe * part["elements"] / per_unit * part["rhs"]
        return tot

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
    times, rhs, upd, busy, kernels, alg_bytes = [], 0, 0, 0.0, 0, 0.0
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()  # the state would stay L2-resident otherwise: flush between steps
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step(qs)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
        st = qs.stats()
        tm = qs.timing()
        rhs += st["rhs"]
        upd += st["ado_updates"]
        busy += tm["busy_ms"]
        kernels += tm["kernels"]
        alg_bytes += alg_bytes_of(tm, st)
    launches = lh.launch_count() - launches0
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = sampler.stop()
    # units of all ranks over the slowest rank's time (no collective touches the state)
    value, total_s = job_throughput(upd, float(sum(times)) / 1e3)
    total_ms = 1e3 * total_s

    # end to end through the public API with host buffers (pinned), copies inside
    rho_h = torch.empty(rho0.shape, dtype=torch.complex128, pin_memory=True)
    e2e_ms = []
    for _ in range(max(1, min(3, args.steps))):
        rho_h.copy_(torch.from_numpy(w.rho0()))
        arr = rho_h.numpy()
        t0 = time.perf_counter()
        qs.solve(arr, t_list, None, wl["kw"])
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    e2e_upd = qs.stats()["ado_updates"]
    e2e = {"value": e2e_upd * world / (statistics.median(e2e_ms) / 1e3), "unit": "ADO-updates/s",
           "h2d_bytes_per_step": 16 * N, "d2h_bytes_per_step": 16 * N}

    # roofline of the fused stage kernel
    # per working launch: busy time / right-hand sides evaluated
    alg_bytes_per_launch = alg_bytes / max(rhs, 1)
    avg_launch_s = (busy / 1e3) / max(rhs, 1)
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes_per_launch / avg_launch_s / 1e9
    flops = w.flops_per_launch()
    tuning = qs.tuning()
    part_tunings = tuning.get("parts", [tuning]) if isinstance(tuning, dict) else []
    resident = any(t.get("resident", False) for t in part_tunings)
    local = any(t.get("local", False) for t in part_tunings)
    if resident:
        kernel = {"rkdp": "k_dp_resident", "rk4": "k_rk4_resident", "lsrk4": "k_ls_resident"}[wl["solver"]] + (
            " (one cooperative launch per output interval: fused RHS and stage epilogues"
            + (", error norm and step control" if wl["solver"] == "rkdp" else "") + "; state in shared memory)")
    elif local:
        kernel = ("k_fixed_local (one launch per output interval; every instance inside one CTA with its stage "
                  "inputs in shared memory, no grid-wide synchronisation)"
                  + ("" if all(t.get("local", False) for t in part_tunings) else "; k_rhs_diag for the other part"))
    else:
        kernel = ("k_rhs_sites (site-local baths: fused RHS + stage epilogue)"
                  if any(t.get("sites", False) for t in part_tunings) else "k_rhs_diag (fused RHS + stage epilogue)")
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": profile_traffic(args.workload, args.form), "peak_source": peak_kind,
            "kernel": kernel,
            "alg_bytes_per_launch": alg_bytes_per_launch, "avg_launch_us": avg_launch_s * 1e6,
            "alg_flops_per_launch": flops, "achieved_tflops": flops / avg_launch_s / 1e12,
            "fma_peaks_tflops": {"fp64": fma_peaks[0], "fp32": fma_peaks[1]},
            "note": ("per stage: CUDA-event time of the resident launches / stages evaluated (grid barriers "
                     "included); bytes per stage are the algorithmic bytes of one stage over the whole state, "
                     "most of which stay in shared memory and L2") if resident
            else ("per stage: CUDA-event time of the interval launches (the longest sub-batch; sub-batches run "
                  "concurrently) / stages evaluated; bytes per stage are the algorithmic bytes of one stage over "
                  "the whole state, which stay in shared memory and L2") if local
            else ("avg launch time = CUDA-event time of the graph replays / stages evaluated (one stage "
                  "over the whole state; intra-graph gaps and the no-op launches replayed after an interval "
                  "ends are included in the time, not in the count)")}
    line = {"metric": "ADO-updates/s", "value": value, "unit": "ADO-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c64 bulk / c128 state" if mixed else "c128 (f64)", "data": "synthetic (seeded)",
            "config": {"workload": args.workload, **w.describe(), "solver": wl["solver"], "t_final": wl["t_final"],
                       "kwargs": wl["kw"], "form": args.form, "parallelism": f"replicas x{world}",
                       "l2": "flushed between steps (512 MiB write)"},
            "max_abs_err_vs_fp64": max_err, "plain_fp64": plain, "tuning": tuning,
            "attempts_per_step": rhs // max(1, args.steps) // per_rhs,
            "gpu_launches": launches, "e2e": e2e, "roofline": roof, "clocks": clocks}
    if rank == 0 and world == 1 and args.workload == "exciton7" and not args.no_secondary:
        line["secondary"] = {"aggregate24": secondary_aggregate24(stream, fma_peaks)}
        if plain is not None:
            line["secondary"]["north_star_exciton7"] = north_star_exciton7(stream, plain["ms_per_step"],
                                                                           total_ms / args.steps)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb = cpu_baseline(w, keep_states=True)
        sample = cb.pop("_final")
        line["cpu_baseline"] = cb
        # both forms against the oracle on the CPU sample (same instances, same horizon)
        line["max_abs_err_vs_oracle"] = {"chosen": oracle_errors(w, sample, args.form)}
        if mixed and not args.no_plain:
            line["max_abs_err_vs_oracle"]["plain_fp64"] = oracle_errors(w, sample, "fp64")
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
