#!/usr/bin/env python3
"""TDVP steps/s of the one-site projector-splitting sweep on one GB300.

Workload (default ``--config c3``): thermofield spin-boson, beta=10, 2x512 = 1024 bath
modes, ohmic alpha=0.2, wc=2, eps=0.5, Delta=1, local dimension 16, bond dimension
chi=64 (2049 tree nodes, 2.2 GB of complex128 node tensors), dt=0.02, Krylov
dimension 16.  Inputs are generated from formulas (no dataset); the start state is
spin up x bath vacuum with std::mt19937(0) unoccupied SPFs.

A "step" is one full symmetric sweep (forward + backward half sweep) over the tree.
The first-step sub-stepping of the reference integrator is replaced in the timed
runs by ``prepare`` (environments + gauge passes) followed by warm-up steps, so every
timed step does the same work.

Arms:
  (default)          the CUDA library (mixed precision when available, else FP64)
  --impl reference   the reference algorithm on the host cores: the reference cannot
                     be built (its linalg/utils submodules are absent), so the CPU
                     restatement in oracle/ stands in, on a bounded sample per step.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "TDVP steps/s at χ=64, 1024 modes: mixed vs FP64 GPU at max|Δ⟨σz⟩|≤1e-6"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c3")
    ap.add_argument("--instances", type=int, default=32, help="instances of the batched form (--config c4)")
    ap.add_argument("--precision", default="auto", choices=["auto", "fp64", "mixed"])
    ap.add_argument("--krylov-stop", default="residual", choices=["full", "residual"],
                    help="how Krylov sub-steps end: on the residual estimate for the remaining interval (the "
                         "reference's rule, default) or after the full Krylov space")
    ap.add_argument("--fp64-steps", type=int, default=3,
                    help="timed steps of the FP64 comparison arm (after the same warm-up steps)")
    ap.add_argument("--no-breakdown", action="store_true")
    ap.add_argument("--drift", type=int, default=0, help="steps of the mixed vs FP64 drift run (no timing)")
    ap.add_argument("--fd", type=int, default=0, help="adjoint form (--config c5): gradient components checked "
                    "against central differences")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-compare", action="store_true")
    ap.add_argument("--override-n", type=int, default=None,
                    help="physical bath modes of a smaller tree of the same shape (profiling runs)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


class Dist:
    """Barrier and max-reduction across replicas (gloo, host memory only)."""

    def __init__(self, world):
        self.world = world
        self.pg = None
        if world > 1:
            import torch.distributed as td
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


class Clocks:
    """nvidia-smi samples (200 ms) during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device)], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return json.load(open(p)), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def traffic_from_profiles(kernel_tag: str):
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    d = json.load(open(p))
    e = d.get(kernel_tag)
    return None if e is None else e.get("dram_bytes_per_launch")


class Nvtx:
    """NVTX range around the timed region (lets ncu capture exactly the timed step)."""

    def __init__(self):
        try:
            import torch.cuda.nvtx as nv
            self.nv = nv
        except Exception:
            self.nv = None

    def push(self, name):
        if self.nv:
            self.nv.range_push(name)

    def pop(self):
        if self.nv:
            self.nv.range_pop()


def upper_node(topo):
    """A node with the largest tensor: the dominant contraction happens there."""
    sizes = [topo.node_size(i) for i in range(topo.nnodes)]
    return int(np.argmax(sizes))


# ---------------------------------------------------------------- CPU reference
def cpu_sample(cfg_name: str, threads: int, krylov_stop: int = 1):
    """Oracle sweep of a tree with the same node shapes and operators as the workload,
    extrapolated to the workload's node counts by per-node-shape times (the full 2049-node
    sweep takes about a quarter of an hour on the host cores).  Returns (steps_per_s,
    description, wall seconds of the sampled sweep)."""
    from oracle.oracle import Oracle
    from ttns_lib_gb300 import spin_boson as sb
    full, cfg = sb.build_config(cfg_name)
    n_small = 4 if cfg.get("beta") is not None else 8   # 8 bath modes: every node shape present
    small, _ = sb.build_config(cfg_name, N=n_small)
    orc = Oracle(small.topology, small.sop, krylov_dim=cfg["krylov_dim"], threads=threads)
    if krylov_stop:
        orc.set_krylov_stop(1)
    orc.set_state(sb.initial_state_numpy(small.topology, seed=0, psi0=np.array([1.0, 0.0])))
    orc.prepare()
    orc.sweep(cfg["dt"])          # move off the exactly rank-deficient start
    orc.reset_node_times()
    t0 = time.perf_counter()
    orc.sweep(cfg["dt"])
    wall = time.perf_counter() - t0
    per = orc.node_times()

    def shape_key(topo, i):
        return (topo.node_shape(i), topo.is_leaf(i), len(topo.children[i]))

    by_shape = {}
    for i in range(small.topology.nnodes):
        by_shape.setdefault(shape_key(small.topology, i), []).append(per[i])
    est = 0.0
    for i in range(full.topology.nnodes):
        k = shape_key(full.topology, i)
        if k not in by_shape:
            raise RuntimeError(f"sample tree lacks node shape {k}")
        est += float(np.mean(by_shape[k]))
    desc = (f"extrapolated: one oracle sweep of a {small.topology.nnodes}-node tree with the workload's node "
            f"shapes and operators ({wall:.1f} s of sweep), per-node-shape times summed over the "
            f"{full.topology.nnodes} nodes of the workload; Krylov stop rule {'residual' if krylov_stop else 'full'}")
    return 1.0 / est, desc, wall


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    if args.config == "c4":
        print(json.dumps({"impl": "reference", "unavailable": "the batched form has no reference implementation "
                          "(the reference steps one instance per integrator); its baseline is the one-after-another "
                          "leg of the same bench line"}), flush=True)
        return 0
    threads = os.cpu_count() or 1
    vals = []
    desc = ""
    stop = 1 if args.krylov_stop == "residual" else 0
    for k in range(args.warmup + args.steps):
        v, desc, _ = cpu_sample(args.config, threads, stop)
        if k >= args.warmup:
            vals.append(v)
    value = float(np.mean(vals))
    from ttns_lib_gb300 import spin_boson as sb
    _, cfg = sb.build_config(args.config)
    line = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 / value, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c128", "data": "synthetic (formula-generated spin-boson bath)",
        "impl": "reference",
        "config": dict(workload_config(args.config, cfg, "fp64 (CPU)"), krylov_stop=args.krylov_stop),
        "cpu_baseline": {"value": value, "unit": "steps/s", "cores": threads, "kind": "port", "sample": desc,
                         "extrapolated": True},
        "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "reference not buildable here (linalg/utils submodules absent); CPU restatement in oracle/ timed",
    }
    print(json.dumps(line), flush=True)
    return 0


def workload_config(name, cfg, precision, over=None):
    from ttns_lib_gb300 import spin_boson as sb
    m, _ = sb.build_config(name, **(over or {}))
    modes = len(m.omega)
    return {
        "workload": f"spin-boson ({'thermofield beta=' + str(cfg['beta']) if cfg.get('beta') else 'T=0'}), "
                    f"{modes} bath modes, chi={cfg['chi']}, d={cfg['d']}, dt={cfg['dt']}, krylov_dim={cfg['krylov_dim']}",
        "config": name, "modes": modes, "chi": cfg["chi"], "local_dim": cfg["d"], "dt": cfg["dt"],
        "krylov_dim": cfg["krylov_dim"], "nodes": m.topology.nnodes, "precision": precision,
        "state_bytes": m.topology.state_size() * 16,
        "l2": ("inputs larger than L2: the node tensors (state) exceed the 129 MB L2"
               if m.topology.state_size() * 16 > 129e6 else "state smaller than L2 (profiling-size tree)"),
    }


# ---------------------------------------------------------------- our arm
def run_ours(args):
    from ttns_lib_gb300 import api
    from ttns_lib_gb300 import spin_boson as sb
    rank, world, local = dist_env()
    dist = Dist(world)
    device = local
    over = {} if args.override_n is None else {"N": args.override_n}
    m, cfg = sb.build_config(args.config, **over)
    topo = m.topology
    psi0 = np.array([1.0, 0.0])

    def make(precision):
        A = api.httensor(topo, device=device)
        A.init_product(psi0, seed=0)
        it = api.fixed_step_projector_splitting_integrator(A, m.sop, krylov_dim=cfg["krylov_dim"],
                                                           krylov_tolerance=1e-12, precision=precision)
        if args.krylov_stop == "residual":
            it.set_krylov_stop(1)
        it.dt = cfg["dt"]
        it.prepare(A)
        return A, it

    prec_name = "fp64"
    if args.precision in ("auto", "mixed"):
        try:
            A, tdvp = make(api.PREC_MIXED)
            prec_name = "mixed"
        except api.TTNError as e:
            if args.precision == "mixed":
                raise
            A, tdvp = make(api.PREC_FP64)
            mixed_unavailable = str(e)
    else:
        A, tdvp = make(api.PREC_FP64)

    # roofline of the dominant kernel: the persistent Krylov exponential on the largest
    # node (it runs every H_eff contraction of the node update)
    node = upper_node(topo)
    nv = Nvtx()
    nv.push("ttn_roofline")
    k_ms, k_fl = tdvp.bench_node_op(A, node, 1, 5)
    nv.pop()
    achieved = k_fl / (k_ms * 1e-3) / 1e12
    peaks, src = measured_peaks()
    if prec_name == "fp64":
        peak = api.fp64_peak_tflops(device)
        roof = {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "traffic": traffic_from_profiles("expm_fp64"),
                "kernel": f"k_expm_coop: Krylov exponential of a {topo.node_shape(node)[0]}x{topo.node_shape(node)[1]} node",
                "peak_source": "FP64 FMA throughput measured in-run (MEASURED_PEAKS.json has no FP64 figure)",
                "ms_per_launch": k_ms, "flops_per_launch": k_fl}
    else:
        peak = peaks["bf16_tflops"]
        roof = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "traffic": traffic_from_profiles("expm_mixed"),
                "kernel": f"Krylov exponential of a {topo.node_shape(node)[0]}x{topo.node_shape(node)[1]} node",
                "peak_source": f"bf16 dense, {src} (MEASURED_PEAKS.json)",
                "ms_per_launch": k_ms, "flops_per_launch": k_fl}

    # Timed steps.  Each step is run the way a drop-in caller that keeps the node tensors
    # on the host runs it: the whole state goes up from pinned host memory, one sweep runs
    # through the C-ABI, the state comes back down and <sz> is read.  `value` is the device
    # time of the sweeps alone (CUDA events on the integrator's stream, the state already
    # resident when each starts); `e2e` is the host wall clock of the same loop, copies
    # included.
    sz_trace = []
    for _ in range(args.warmup):
        tdvp(A, m.sop, -1j)
        sz_trace.append(tdvp.mel()(sb.SZ, 0, A).real)
    host = api.PinnedBuffer(topo.state_size())
    A.download_to(host)
    tdvp.synchronize()
    dist.barrier()
    clocks = Clocks(device)
    l0 = api.launch_count()
    f0 = tdvp.flops()
    io0 = tdvp.io_bytes()
    nvtx = Nvtx()
    clocks.start()
    nvtx.push("ttn_timed")
    ms = 0.0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        A.upload_from(host)
        tdvp.timer_start()
        tdvp(A, m.sop, -1j)
        ms += tdvp.timer_stop()
        A.download_to(host)
        sz_trace.append(tdvp.mel()(sb.SZ, 0, A).real)
    e2e_s = time.perf_counter() - t0
    nvtx.pop()
    clk = clocks.stop()
    launches = api.launch_count() - l0
    flops_step = (tdvp.flops() - f0) / args.steps
    io1 = tdvp.io_bytes()
    dist.barrier()
    ms_max = dist.max(ms)
    e2e = dist.max(e2e_s)
    value = world * args.steps / (ms_max / 1e3)
    h2d = host.nbytes + (io1[0] - io0[0]) // args.steps
    d2h = host.nbytes + (io1[1] - io0[1]) // args.steps
    del host

    # Where a step's time goes: one more step (after the timed ones, not counted) with the
    # synchronising per-operation breakdown on, by operation and node size.
    breakdown = None
    if not args.no_breakdown:
        tdvp.set_profiling(True)
        t0 = time.perf_counter()
        tdvp(A, m.sop, -1j)
        wall_prof = time.perf_counter() - t0
        prof = tdvp.profile()
        tdvp.set_profiling(False)
        breakdown = {"wall_s": wall_prof, "note": "one extra step with a stream synchronisation after every "
                     "operation; seconds and calls per operation[node-size class]",
                     "ops": {k: {"s": round(v[0], 4), "calls": v[1]} for k, v in
                             sorted(prof.items(), key=lambda kv: -kv[1][0])}}

    # The FP64 path from the same start state: the same warm-up steps, then a bounded
    # number of timed steps; its step rate and the largest |<sz>(mixed) - <sz>(FP64)| over
    # the steps both ran.
    fp64 = None
    if prec_name == "mixed" and not args.no_fp64_compare:
        k64 = max(1, min(args.steps, args.fp64_steps))
        A64, t64 = make(api.PREC_FP64)
        sz64 = []
        for _ in range(args.warmup):
            t64(A64, m.sop, -1j)
            sz64.append(t64.mel()(sb.SZ, 0, A64).real)
        t64.synchronize()
        dist.barrier()
        ms64 = 0.0
        for _ in range(k64):
            t64.timer_start()
            t64(A64, m.sop, -1j)
            ms64 += t64.timer_stop()
            sz64.append(t64.mel()(sb.SZ, 0, A64).real)
        ms64 = dist.max(ms64)
        dsz = max(abs(a - b) for a, b in zip(sz_trace, sz64))
        v64 = world * k64 / (ms64 / 1e3)
        fp64 = {"value": v64, "unit": "steps/s", "ms_per_step": ms64 / k64, "timed_steps": k64,
                "mixed_over_fp64": value / v64, "max_abs_dsz": dsz, "dsz_bound": 1e-6,
                "within_bound": bool(dsz <= 1e-6), "compared_points": len(sz64),
                "compared": "<sz> after each warm-up step and each timed FP64 step, same start state, "
                            "same Krylov stop rule"}
        del A64, t64

    line = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "c128" if prec_name == "fp64" else
                 "c128 state and Krylov; rank-64 contractions on tensor cores from exact bf16 integer slices",
        "data": "synthetic (formula-generated spin-boson bath; std::mt19937 unoccupied SPFs)",
        "config": dict(workload_config(args.config, cfg, prec_name, over), krylov_stop=args.krylov_stop),
        "roofline": roof,
        "e2e": {"value": world * args.steps / e2e, "unit": "steps/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "clocks": clk,
        "breakdown": breakdown,
        "algorithmic_tflop_per_step": flops_step / 1e12,
        "sz_last": sz_trace[-1] if sz_trace else None,
        "parallelism": "replicas only (the sweep is a sequential chain over the tree)",
    }
    if prec_name == "fp64" and args.precision == "auto":
        line["mixed"] = {"available": False, "reason": mixed_unavailable}
    if fp64 is not None:
        line["fp64"] = fp64
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, desc, _ = cpu_sample(args.config, threads, 1 if args.krylov_stop == "residual" else 0)
        line["cpu_baseline"] = {"value": v, "unit": "steps/s", "cores": threads, "kind": "port", "sample": desc,
                                "extrapolated": True}
    if rank == 0:
        print(json.dumps(line), flush=True)
    dist.close()
    return 0


# ---------------------------------------------------------------- subspace expansion (c2)
def run_expansion(args):
    """The adaptive-bond form at scale: thermofield beta = 1, 2 x 256 bath modes, d = 16,
    bonds starting at 2 and growing up to chi = 32 by subspace expansion (spawning
    threshold 1e-8), FP64, dt = 0.02, Krylov dimension 16.  A step is one expanding sweep;
    the timed steps follow the expanding preparation and the warm-up steps."""
    from ttns_lib_gb300 import api
    from ttns_lib_gb300 import spin_boson as sb
    rank, world, local = dist_env()
    dist = Dist(world)
    over = {} if args.override_n is None else {"N": args.override_n}
    full, cfg = sb.build_config("c2", **over)
    start, _ = sb.build_config("c2", chi=2, **over)
    topo = start.topology
    cap = full.topology.hrank
    A = api.httensor(topo, device=local)
    A.init_product(np.array([1.0, 0.0]), seed=0)
    it = api.subspace_expansion_projector_splitting_integrator(A, start.sop, cap, krylov_dim=cfg["krylov_dim"],
                                                             krylov_tolerance=1e-12, spawning_threshold=1e-8)
    if args.krylov_stop == "residual":
        it.set_krylov_stop(1)
    it.dt = cfg["dt"]
    t0 = time.perf_counter()
    it.prepare(A)
    prep_s = time.perf_counter() - t0
    sz = []
    for _ in range(args.warmup):
        it(A, start.sop, -1j)
        sz.append(it.mel()(sb.SZ, 0, A).real)
    it.synchronize()
    dist.barrier()
    clocks = Clocks(local)
    l0 = api.launch_count()
    clocks.start()
    ms = 0.0
    ranks = []
    for _ in range(args.steps):
        it.timer_start()
        it(A, start.sop, -1j)
        ms += it.timer_stop()
        sz.append(it.mel()(sb.SZ, 0, A).real)
        ranks.append(int(A.hrank().max()))
    clk = clocks.stop()
    launches = api.launch_count() - l0
    ms_max = dist.max(ms)
    value = world * args.steps / (ms_max / 1e3)
    one, two = it.expansion_counts()
    line = {
        "metric": "TDVP steps/s with subspace expansion (chi <= 32, 2x256 thermofield modes)", "value": value,
        "unit": "steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c128", "data": "synthetic (formula-generated spin-boson bath; std::mt19937 unoccupied SPFs)",
        "impl": "expansion",
        "config": {"workload": f"spin-boson (thermofield beta=1.0), {len(full.omega)} bath modes, chi<=32, d=16, "
                               f"dt=0.02, krylov_dim=16, spawning threshold 1e-8",
                   "config": "c2", "nodes": topo.nnodes, "start_bond": 2, "capacity_bond": 32,
                   "krylov_stop": args.krylov_stop, "precision": "fp64"},
        "prepare_s": prep_s, "largest_bond_per_timed_step": ranks, "expansions": {"onesite": one, "twosite": two},
        "norm": it.mel()(A), "sz_trace": sz, "gpu_launches": launches, "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    dist.close()
    return 0


# ---------------------------------------------------------------- mixed vs FP64 drift
def run_drift(args):
    """|<sz>(mixed) - <sz>(FP64)| step by step over --drift steps of the headline workload's
    model (use --override-n for a smaller tree with the same node shapes): both integrators
    start from the same product state, take the same steps with the same Krylov stop rule,
    and the largest difference so far is reported at powers of two and at the end."""
    from ttns_lib_gb300 import api
    from ttns_lib_gb300 import spin_boson as sb
    over = {} if args.override_n is None else {"N": args.override_n}
    m, cfg = sb.build_config(args.config, **over)
    arms = {}
    for name, prec in (("mixed", api.PREC_MIXED), ("fp64", api.PREC_FP64)):
        A = api.httensor(m.topology, device=0)
        A.init_product(np.array([1.0, 0.0]), seed=0)
        it = api.fixed_step_projector_splitting_integrator(A, m.sop, krylov_dim=cfg["krylov_dim"],
                                                          krylov_tolerance=1e-12, precision=prec)
        if args.krylov_stop == "residual":
            it.set_krylov_stop(1)
        it.dt = cfg["dt"]
        arms[name] = (A, it)
    worst, marks, first_above = 0.0, {}, None
    t0 = time.perf_counter()
    for k in range(1, args.drift + 1):
        sz = {}
        for name, (A, it) in arms.items():
            it(A, m.sop, -1j)
            sz[name] = it.mel()(sb.SZ, 0, A).real
        worst = max(worst, abs(sz["mixed"] - sz["fp64"]))
        if first_above is None and worst > 1e-6:
            first_above = k
        if (k & (k - 1)) == 0 or k == args.drift:
            marks[k] = worst
    line = {"metric": "max |<sz>(mixed) - <sz>(FP64)| over the first k steps", "impl": "drift",
            "config": dict(workload_config(args.config, cfg, "mixed and fp64", over), krylov_stop=args.krylov_stop),
            "steps": args.drift, "max_abs_dsz_by_step": marks, "first_step_above_1e-6": first_above,
            "wall_s": time.perf_counter() - t0}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------- adjoint form (c5)
def generic_isometric_state(topo, seed):
    """Random state with every non-root node an isometry (all bonds populated): gradients
    through the QR gauge moves need invertible R factors, which a product state lacks."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(topo.nnodes):
        d, r = topo.node_shape(i)
        a = rng.normal(size=(d, r)) + 1j * rng.normal(size=(d, r))
        out.append(np.linalg.qr(a)[0] if i else a / np.linalg.norm(a))
    return out


def run_adjoint(args):
    """The adjoint form at its configuration's shapes: zero-temperature spin-boson, N = 128
    modes (alpha = 0.4, wc = 5), d = 12, chi = 24, dt = 0.05, J = sum_t w_t <sz>(t) with
    w_t ~ U[0, 1] (seeded), the gradient with respect to eps, Delta and all 128 c_k by the
    device adjoint sweep with a checkpoint every 20 steps, over --steps time steps from a
    seeded generic state.  The FP64 forward path over the same steps is timed beside it, and
    --fd n checks n gradient components against central differences (h = 1e-6) of the
    plain FP64 path."""
    from ttns_lib_gb300 import api
    from ttns_lib_gb300 import spin_boson as sb
    rank, world, local = dist_env()
    m, cfg = sb.build_config("c5")
    topo = m.topology
    nsteps = args.steps
    st = generic_isometric_state(topo, seed=5)
    wt = np.random.default_rng(17).uniform(size=nsteps)
    theta = np.concatenate([[m.eps, m.delta], m.coupling])
    evaluate = api.spin_boson_adjoint(m.omega, cfg["d"], cfg["chi"], st, cfg["dt"], wt, krylov_dim=cfg["krylov_dim"],
                                      krylov_tolerance=1e-12, checkpoint_every=20, device=local)

    def plain_J(th):
        mm = sb.build_from_modes(m.omega, th[2:], cfg["d"], cfg["chi"], float(th[0]), float(th[1]))
        A = api.httensor(topo, device=local)
        A.set(st)
        it = api.fixed_step_projector_splitting_integrator(A, mm.sop, krylov_dim=cfg["krylov_dim"],
                                                          krylov_tolerance=1e-12)
        it.dt = cfg["dt"]
        J = 0.0
        for k in range(nsteps):
            it(A, mm.sop, -1j)
            J += wt[k] * it.mel()(sb.SZ, 0, A).real
        it.synchronize()
        return J

    for _ in range(max(0, args.warmup)):
        plain_J(theta)
    t0 = time.perf_counter()
    J0 = plain_J(theta)
    fwd_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    J, grad = evaluate(theta)
    adj_s = time.perf_counter() - t0
    fd = {}
    if args.fd > 0:
        h = 1e-6
        idx = [0, 1] + [2 + int(k) for k in np.linspace(0, len(m.coupling) - 1, max(0, args.fd - 2)).astype(int)]
        for i in idx[:args.fd]:
            e = np.zeros_like(theta)
            e[i] = h
            fd[int(i)] = (plain_J(theta + e) - plain_J(theta - e)) / (2 * h)
    names = ["eps", "delta"] + [f"c_{k}" for k in range(len(m.coupling))]
    check = {names[i]: {"adjoint": float(grad[i]), "fd": v, "rel": abs(grad[i] - v) / max(abs(v), 1e-300)}
             for i, v in fd.items()}
    line = {
        "metric": "adjoint gradient of a time-integrated <sz> (eps, Delta, 128 c_k), seconds per TDVP step",
        "value": adj_s / nsteps, "unit": "s/step", "n_gpus": 1, "steps": nsteps, "warmup": args.warmup,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "c128", "impl": "adjoint",
        "data": "synthetic (formula-generated bath; seeded generic start state and weights)",
        "config": {"workload": "spin-boson (T=0), 128 bath modes, chi=24, d=12, dt=0.05, krylov_dim=12, "
                               "checkpoint every 20 steps", "config": "c5", "nodes": topo.nnodes,
                   "steps_of_config": 400},
        "J": J, "J_plain_path": J0, "forward_s_per_step": fwd_s / nsteps, "adjoint_over_forward": adj_s / fwd_s,
        "gradient_norm": float(np.linalg.norm(grad)), "fd_check": check,
        "max_rel_fd": max((c["rel"] for c in check.values()), default=None),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------- batched form (c4)
def batched_specs(count: int, seed: int = 0):
    """Instances of the batched workload: alpha ~ U[0.05, 1], omega_c ~ U[1, 10],
    eps ~ U[-1, 1], Delta = 1, N in {32, 64, 128, 256}, d in {8, 16}, chi in
    {8, 16, 24, 32}, dt = 0.05 (numpy's seeded generator)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        out.append(dict(N=int(rng.choice([32, 64, 128, 256])), alpha=float(rng.uniform(0.05, 1.0)),
                        wc=float(rng.uniform(1.0, 10.0)), d=int(rng.choice([8, 16])),
                        chi=int(rng.choice([8, 16, 24, 32])), eps=float(rng.uniform(-1.0, 1.0)), delta=1.0))
    return out


def run_batched(args):
    """Per-instance throughput of independent instances: one after another (one host
    thread) against ttn_batch_step (all host threads, one stream per instance)."""
    from ttns_lib_gb300 import api
    from ttns_lib_gb300 import spin_boson as sb
    rank, world, local = dist_env()
    count = args.instances
    specs = batched_specs(count, seed=rank)

    def make_all():
        inst = []
        for sp in specs:
            m = sb.build(sp["N"], sp["alpha"], sp["wc"], sp["d"], sp["chi"], sp["eps"], sp["delta"], None)
            A = api.httensor(m.topology, device=local)
            A.init_product(np.array([1.0, 0.0]), seed=0)
            it = api.fixed_step_projector_splitting_integrator(A, m.sop, krylov_dim=12, krylov_tolerance=1e-12)
            it.dt = 0.05
            it.prepare(A)
            inst.append((m, A, it))
        return inst

    seq, bat = make_all(), make_all()
    for _ in range(args.warmup):
        for m, A, it in seq:
            it(A, m.sop, -1j)
        api.batch_step([x[2] for x in bat], [x[1] for x in bat], -1j)
    for x in seq + bat:
        x[2].synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for m, A, it in seq:
            it(A, m.sop, -1j)
    t_seq = time.perf_counter() - t0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        api.batch_step([x[2] for x in bat], [x[1] for x in bat], -1j)
    t_bat = time.perf_counter() - t0
    dsz = max(abs(a[2].mel()(sb.SZ, 0, a[1]) - b[2].mel()(sb.SZ, 0, b[1])) for a, b in zip(seq, bat))
    v_seq = count * args.steps / t_seq
    v_bat = count * args.steps / t_bat
    line = {
        "metric": "instance-steps/s of independent spin-boson instances, batched vs one after another",
        "value": world * v_bat, "unit": "instance-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_bat / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128", "impl": "batched",
        "data": "synthetic (formula-generated baths; instance parameters from a seeded generator)",
        "config": {"workload": f"{count} independent instances, N in {{32..256}}, d in {{8,16}}, chi in {{8..32}}",
                   "config": "c4", "instances": count, "krylov_dim": 12, "dt": 0.05,
                   "timing": "host wall clock around whole steps (each step ends with a device sync)"},
        "sequential": {"value": v_seq, "unit": "instance-steps/s"},
        "batched_over_sequential": v_bat / v_seq,
        "max_abs_dsz_batched_vs_sequential": float(abs(dsz)),
        "host_threads": os.cpu_count(),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.config == "c4":
        return run_batched(args)
    if args.config == "c2":
        return run_expansion(args)
    if args.config == "c5":
        return run_adjoint(args)
    if args.drift > 0:
        return run_drift(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
