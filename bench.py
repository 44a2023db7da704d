#!/usr/bin/env python
"""Throughput of FFEA's per-timestep blob update on GB300.

Metric: node-steps/s (linear nodes advanced one timestep per second) with
every CG solve run to relative residual 1e-6 (confirmed by an FP64 true
residual), for the learned two-level preconditioner (the headline `value`)
and for plain Jacobi-PCG (`plain`), measured in the same run, with their
ratios in `learned_vs_plain`.

Workload (default): a 64^3-cell grid split into 6 tetrahedra per cell and
cut to a 40 nm-radius sphere (146,737 linear nodes, 823,968 elements,
1,135,891 nodes with the edge midpoints), node positions jittered by
N(0, 0.05 cell) from a seed; density 1.5e3 kg/m^3, shear/bulk modulus
3.7e8/1.1e9 Pa, shear/bulk viscosity 1e-3 Pa s, kT at 300 K, dt 1e-14 s,
thermal noise on, Stokes drag on, CG_nomass solver to epsilon 1e-6, FP32
element forces and SpMV with double-float / FP64 reductions.
Synthetic, seeded inputs stand in for a real protein mesh.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--workload sphere40|sphere61|replicas256|ensemble64|heldout|...]
                  [--precond learned|two-level|jacobi] [--no-plain] [--autotune]

Other workloads: sphere61 (98^3-cell sphere, ~515k nodes), replicas256 (256
replicas of the 20 nm sphere), ensemble64 (64 uneven blobs), heldout (the
learned preconditioner's held-out family, 10-50 nm).  Each line carries the
roofline of k_cg and of every step kernel (kernel_roofline).

N > 1 runs under torchrun, one process per GPU and no exchange while
stepping (weak scaling).  A single-blob workload runs one replica per GPU
with its own RNG stream (a single blob does not shard).  A multi-blob
workload runs N replicas of its blobs, packed over the GPUs by estimated
bytes per step (ffea_gb300.partition).
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from ffea_gb300.workloads import WORKLOADS, replica_seed  # noqa: E402

METRIC = "node-steps/s at CG rel-res 1e-6"
PRECISION_MIXED_DESC = ("FP32 element forces, matrix and SpMV; CG dot products as FP32 warp sums combined in "
                        "double-float (TwoSum) across warps and segments; FP32 CG coefficients; FP64 positions, "
                        "rhs and the FP64 true residual that confirms every solve")
PRECONDS = {"jacobi": 0, "two-level": 1, "learned": 2}
L2_BYTES = 129 * 1024 * 1024


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="sphere40")
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--e2e-steps", type=int, default=None)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=20.0, help="CPU work budget of the cpu_baseline sample")
    ap.add_argument("--precond", choices=sorted(PRECONDS), default="learned",
                    help="preconditioner of the headline arm (plain Jacobi-PCG is measured beside it)")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain Jacobi-PCG and two-level arms")
    ap.add_argument("--no-memory-resident", action="store_true",
                    help="skip the in-process memory-resident solve measurement (sphere61) of the default run")
    ap.add_argument("--parity-steps", type=int, default=5,
                    help="steps of the parity leg on the measured single-blob workload (0: no parity leg)")
    ap.add_argument("--autotune", action="store_true",
                    help="pick each arm's launch shape with ffea_gb300.autotune on this batch first")
    return ap.parse_args()


def build_specs(workload: str, rank: int, precision: str):
    """The blobs of one rank's replica of the workload."""
    from ffea_gb300.workloads import build_specs as specs_of
    return specs_of(workload, rank, precision)


def config_of(args, specs, world_size):
    specs = specs if isinstance(specs, (list, tuple)) else [specs]
    return {
        "workload": f"{args.workload}: {WORKLOADS[args.workload]['desc']}",
        "blobs": len(specs),
        "linear_nodes": int(sum(s.mesh.num_linear for s in specs)),
        "elements": int(sum(s.mesh.num_elements for s in specs)),
        "total_nodes": int(sum(s.mesh.num_nodes for s in specs)),
        "solver": "CG_nomass, epsilon 1e-6, convergence confirmed by an FP64 true residual",
        "precision": PRECISION_MIXED_DESC if args.precision == "mixed" else "FP64",
        "noise": "on (MRG32k3a, RngStream-exact)",
        "replicas": world_size,
        "l2": "L2 flushed (256 MiB write) between timed steps",
    }


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm_, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm_)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------- roofline
def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def cg_iteration_bytes(num_linear: int, num_edges: int) -> int:
    """Algorithmic bytes of one Jacobi-PCG iteration in the minimum-traffic
    model (FP32 values, int32 indices): SpMV over the block-sparse matrix with
    B = N + 2 edges 3x3 blocks (36 B values + 4 B column each, 4 B row pointer
    and 12 + 12 B for the input and output vectors per row), the solution /
    residual update (48 N + 24 N) and the direction update (36 N + 12 N):
    40 B + 148 N."""
    B = num_linear + 2 * num_edges
    return 40 * B + 148 * num_linear


def step_kernel_bytes(num_linear: int, num_elements: int, num_edges: int, num_total: int) -> dict:
    """Algorithmic bytes per launch of the per-step kernels in the same model:
    element forces 12 N + 168 E (positions, connectivity, rest state,
    material and sign in; nodal forces, scaled gradients and sign out);
    the draws 4 (7 E + 3 N) (one FP32 value written per draw generated: the
    elements' and those of the nodes with a Stokes drag, here the corner
    nodes); the viscosity assembly 40 E + 64 E + 36 B (element coefficients
    and source indices in, block values out); the node gather 64 E + 16 N.
    The update (48 N) runs at the end of the solve kernel."""
    N, E, B = num_linear, num_elements, num_linear + 2 * num_edges
    return {"noise": 4 * (7 * E + 3 * N), "elements": 12 * N + 168 * E,
            "assemble": 40 * E + 64 * E + 36 * B, "nodes": 64 * E + 16 * N}


def ncu_summary_value(key, kernel="k_cg", workload="sphere40"):
    """A `key: value` figure from the committed ncu summary of a kernel, if present."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.md")
    try:
        with open(path) as fh:
            m = re.search(re.escape(key) + r":\s*([0-9.eE+]+)", fh.read())
        return float(m.group(1)) if m else None
    except OSError:
        return None


def memory_resident_roofline(args, peak):
    """The solve where HBM is the bound: one blob of 514,965 corner nodes
    (98^3-cell, 61.25 nm sphere) runs the memory-resident solve (more CG
    segments than SMs; the matrix, about 300 MB, does not fit in L2).
    Learned two-level preconditioner, steps timed per kernel over one
    coarse-refresh cycle.  frac: the algorithmic bytes (40 B + 148 N per
    iteration, 48 N for the update) over the solve's time; dram_frac: the
    DRAM bytes per iteration of the committed ncu capture of this kernel on
    this workload over the same time."""
    from ffea_gb300 import learned
    from ffea_gb300.workloads import build_specs as specs_of
    from ffea_gb300.world import World
    specs = specs_of("sphere61", 0, args.precision)
    with World(specs, graph=True, true_residual=True, preconditioner=PRECONDS["learned"]) as w:
        if w.preconditioner() == PRECONDS["learned"]:
            learned.apply(w, learned.load())
        w.run(3)
        nl, _, nedges = w.sizes()
        n = int(os.environ.get("FFEA_GPU_COARSE_REFRESH", "10"))
        loops0 = w.cg_loop_count()
        w.set_timing(True)
        w.run(n)
        cg_ms = float(w.phase_times()[3]) / n
        w.set_timing(False)
        iters = (w.cg_loop_count() - loops0) / n
    alg = iters * cg_iteration_bytes(nl, nedges) + 48 * nl
    gbs = alg / (cg_ms / 1e3) / 1e9
    out = {"workload": f"sphere61: {WORKLOADS['sphere61']['desc']} ({nl:,} corner nodes)",
           "kernel": "k_cg (memory-resident)", "us": round(cg_ms * 1e3, 1), "cg_iters": iters,
           "us_per_iteration": round(cg_ms * 1e3 / max(iters, 1e-9), 2),
           "algorithmic_bytes": int(alg), "achieved_gbs": round(gbs, 1), "frac": round(gbs / peak, 4)}
    dram_it = ncu_summary_value("dram_bytes_per_iteration", workload="sphere61")
    if dram_it:
        dgbs = dram_it * iters / (cg_ms / 1e3) / 1e9
        out.update({"dram_bytes_per_iteration": dram_it, "dram_gbs": round(dgbs, 1),
                    "dram_frac": round(dgbs / peak, 4),
                    "dram_source": "profiles/k_cg_sphere61.md (one ncu capture of this kernel on this workload)"})
    return out


def ncu_traffic(kernel="k_cg", workload="sphere40"):
    """Per-launch DRAM bytes from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.md")
    try:
        with open(path) as fh:
            m = re.search(r"dram_bytes_per_launch:\s*([0-9.eE+]+)", fh.read())
        return float(m.group(1)) if m else None
    except OSError:
        return None


# ---------------------------------------------------------------- CPU baseline
def unlimited_stack() -> str:
    """`ulimit -s unlimited` for this process, as FFEA's run instructions ask
    (its CG copies vectors into stack arrays); returns what was set."""
    import resource
    try:
        _, hard = resource.getrlimit(resource.RLIMIT_STACK)
        resource.setrlimit(resource.RLIMIT_STACK, (hard, hard))
        return "unlimited" if hard == resource.RLIM_INFINITY else f"{hard} B"
    except (ValueError, OSError):
        return "unchanged"


def cpu_baseline(specs, budget_s: float, min_steps: int = 3):
    """FFEA's algorithm (the oracle built with FFEA's release flags) on all
    host cores, a bounded sample: whole timesteps of the workload's blobs in
    order (OpenMP within each blob, FFEA_PARALLEL_WITHIN_BLOB) until the
    budget is spent and at least `min_steps` steps ran; node-steps/s from the
    median step time."""
    from oracle import oracle as O
    O.build(ref=False)
    stack = unlimited_stack()
    specs = specs if isinstance(specs, (list, tuple)) else [specs]
    threads = os.cpu_count() or 1
    rates, total, k, blobs_used = [], 0.0, 0, set()
    blob, blob_i = None, -1
    while (total < budget_s or k < min_steps) and k < 1000:
        i = k % len(specs)
        if i != blob_i:
            blob, blob_i = O.blob_from_spec(specs[i], num_threads=threads, impl="fast"), i
        t = time.perf_counter()
        if blob.step(1) != 0:
            raise RuntimeError("oracle step failed in the CPU baseline")
        dt = time.perf_counter() - t
        rates.append(specs[i].mesh.num_linear / dt)
        total += dt
        blobs_used.add(i)
        k += 1
    v = statistics.median(rates)
    what = ("the full workload" if len(specs) == 1 else
            f"{len(blobs_used)} of the workload's {len(specs)} blobs, one step each")
    return {"value": v, "unit": "node-steps/s", "cores": threads, "kind": "port",
            "sample": f"{k} timestep(s) of {what} after set-up, {total:.1f} s; median of the per-step rates; "
                      f"oracle built with {O.FAST_FLAGS}; OpenMP {threads} threads, per-thread RNG streams as "
                      f"FFEA_PARALLEL_WITHIN_BLOB; stack limit {stack}",
            "steps": k, "seconds": total}


# ---------------------------------------------------------------- arms
def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x: float, world: int, device="cuda") -> float:
    """The slowest rank's time: the whole job is done when the last replica is."""
    if world <= 1:
        return float(x)
    import torch
    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x: float, world: int, device="cuda") -> float:
    """The whole job's total of a per-rank count (host-side, after the timed region)."""
    if world <= 1:
        return float(x)
    import torch
    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.SUM)
    return float(t.item())


def aggregate_throughput(nodes_per_replica: int, steps: int, world: int, seconds: float) -> float:
    """Whole-job node-steps/s: every replica advances all its linear nodes each step."""
    return nodes_per_replica * steps * world / seconds


def run_reference(args):
    """The reference's algorithm (the oracle built with FFEA's release flags,
    FP64, OpenMP over all host cores) on this workload: set-up outside the
    timed region, `warmup` untimed steps, then `steps` timed steps.  A step
    is one timestep of one blob of the workload (the blobs of a batch in
    turn), the bounded sample of the whole job's step; the value comes from
    the median step."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O
    O.build(ref=False)
    stack = unlimited_stack()
    specs = build_specs(args.workload, 0, args.precision)
    specs = specs if isinstance(specs, (list, tuple)) else [specs]
    threads = os.cpu_count() or 1
    blobs = {}

    def one_step(k):
        i = k % len(specs)
        t = time.perf_counter()
        if blobs[i].step(1) != 0:
            raise RuntimeError("oracle step failed in the reference arm")
        return time.perf_counter() - t, specs[i].mesh.num_linear

    for i in sorted({k % len(specs) for k in range(args.warmup + args.steps)}):  # set-up, untimed
        blobs[i] = O.blob_from_spec(specs[i], num_threads=threads, impl="fast")
    for k in range(args.warmup):
        one_step(k)
    total, rates = 0.0, []
    for k in range(args.warmup, args.warmup + args.steps):
        dt, n = one_step(k)
        total += dt
        rates.append(n / dt)
    value = statistics.median(rates)
    what = ("the full workload" if len(specs) == 1 else
            f"one blob of the workload's {len(specs)} (in turn)")
    line = {
        "metric": METRIC, "value": value, "unit": "node-steps/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_of(args, specs if len(specs) > 1 else specs[0], 1), "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "node-steps/s", "cores": threads, "kind": "port",
                         "sample": f"each step: one timestep of {what}, after {args.warmup} untimed step(s); "
                                   f"{args.steps} timed steps took {total:.1f} s; value from the median step; "
                                   f"oracle built with {O.FAST_FLAGS}; OpenMP {threads} threads, per-thread RNG "
                                   f"streams as FFEA_PARALLEL_WITHIN_BLOB; stack limit {stack}"},
        "e2e": {"value": value, "unit": "node-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    line["config"]["l2"] = "n/a (CPU)"
    line["config"]["precision"] = "FP64 (the reference algorithm on the host cores)"
    print(json.dumps(line), flush=True)


def measure_arm(args, specs, precond: str, world: int, local: int):
    """One arm on this rank: warm-up, K timed steps (device events on the
    handle's stream, L2 flushed between steps), the end-to-end loop through
    the C ABI with host buffers, and a profile pass with per-phase events."""
    import torch
    from ffea_gb300 import learned
    from ffea_gb300.world import World, kernel_launches

    N = sum(s_.mesh.num_linear for s_ in specs)
    tuned = None
    if args.autotune:
        from ffea_gb300 import autotune
        space = [{"FFEA_GPU_CG_SMEM_SLOTS": sl, "FFEA_GPU_CG_MAX_CTAS": ct, "FFEA_GPU_COARSE_REFRESH": rf}
                 for sl in (0, 2, 64) for ct in (torch.cuda.get_device_properties(local).multi_processor_count,
                                                 (3 * torch.cuda.get_device_properties(local).multi_processor_count) // 4)
                 for rf in ((10, 25) if precond != "jacobi" else (10,))]
        tuned = autotune.tune(specs, PRECONDS[precond], space=space, cache=None,
                              weights=learned.load() if precond == "learned" else None)
        with autotune.applied(tuned["config"]):
            w = World(list(specs), graph=True, true_residual=True, preconditioner=PRECONDS[precond])
    else:
        w = World(list(specs), graph=True, true_residual=True, preconditioner=PRECONDS[precond])
    if precond == "learned" and w.preconditioner() == PRECONDS["learned"]:
        learned.apply(w, learned.load())
    nl, ne, nedges = w.sizes()
    stream = torch.cuda.ExternalStream(w.stream())
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    w.run(max(args.warmup, 3))
    K = args.steps
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    loops0 = w.cg_loop_count()
    launches0 = kernel_launches()
    sampler = ClockSampler(local)
    sampler.start()
    barrier()
    torch.cuda.synchronize()
    for k in range(K):
        starts[k].record(stream)
        w.run_async(1)
        ends[k].record(stream)
        with torch.cuda.stream(stream):
            flush.fill_(float(k))
    w.synchronize()
    torch.cuda.synchronize()
    barrier()
    clocks = sampler.stop()
    total_ms = float(sum(s_.elapsed_time(e_) for s_, e_ in zip(starts, ends)))
    loops = w.cg_loop_count() - loops0
    launches = kernel_launches() - launches0
    total_ms = max_over_ranks(total_ms, world)
    N_job = sum_over_ranks(N, world)  # every rank's linear nodes (replicas or ensemble shards)
    value = N_job * K / (total_ms / 1e3)

    # end to end through the C ABI with the caller's pinned host buffers (all
    # N_t nodes in the reference's order), per step: set_nodes of the step's
    # inputs (H2D), the step, get_nodes of positions, velocities and forces
    # (D2H).  The inputs are the positions, plus the velocities for the mass
    # solvers: a CG_nomass step does not read velocities (FFEA's NoMass
    # forces never use node.vel, src/Blob.cpp:3853-3905, and euler_integrate
    # overwrites it with the solution, :3937-3969).
    from ffea_gb300 import params as Pm
    blobs = [w.blob(i) for i in range(len(specs))]
    Nt = sum(s_.mesh.num_nodes for s_ in specs)
    reads_vel = [s_.params.solver != Pm.SOLVER_NOMASS for s_ in specs]
    # pinned (page-locked) host arrays, as a caller that streams state would hold
    bufs = [tuple(torch.empty((s_.mesh.num_nodes, 3), dtype=torch.float64, pin_memory=True).numpy()
                  for _ in range(3)) for s_ in specs]
    for b_, buf in zip(blobs, bufs):
        b_.get_nodes(out=buf)
    Ke = args.e2e_steps or max(3, K // 2)
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(Ke):
        for b_, buf, rv in zip(blobs, bufs, reads_vel):
            b_.set_nodes(buf[0], buf[1] if rv else None)
        w.run(1)
        for b_, buf in zip(blobs, bufs):
            b_.get_nodes(out=buf)
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    h2d = sum((2 if rv else 1) * 3 * 8 * s_.mesh.num_nodes for s_, rv in zip(specs, reads_vel))
    e2e = {"value": N_job * Ke / e2e_s, "unit": "node-steps/s",
           "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": 3 * 3 * 8 * Nt, "steps": Ke,
           "copies": "H2D: positions (+ velocities for mass solvers); D2H: positions, velocities, forces"}

    # profile pass: direct launches with CUDA events around each phase of a
    # step, over one whole coarse-refresh cycle (the refresh runs on every
    # tenth step, so its per-step share is its cost over ten steps)
    prof_steps = int(os.environ.get("FFEA_GPU_COARSE_REFRESH", "10"))
    loops_p0 = w.cg_loop_count()
    w.set_timing(True)
    w.run(prof_steps)
    phases = w.phase_times() / prof_steps
    kernel_ms = {k: v / prof_steps for k, v in w.kernel_times().items()}
    w.set_timing(False)
    iters_p = (w.cg_loop_count() - loops_p0) / prof_steps
    pc_used = {v: k for k, v in PRECONDS.items()}[w.preconditioner()]
    w.close()
    cg_ms = float(phases[3])
    return {
        "value": value, "ms_per_step": total_ms / K, "e2e": e2e, "gpu_launches": int(launches),
        "cg_iters_per_step": loops / K, "clocks": clocks, "preconditioner": pc_used,
        "phase_ms_per_step": {"elements": float(phases[0]), "assemble": float(phases[1]),
                              "nodes": float(phases[2]), "cg": cg_ms},  # cg: the solve and the Euler update
        "cg_us_per_iteration": 1e3 * cg_ms / max(iters_p, 1), "cg_iters_profiled": iters_p,
        "sizes": (nl, ne, nedges), "autotune": tuned, "kernel_ms": kernel_ms,
        "total_nodes": sum(s_.mesh.num_nodes for s_ in specs),
    }


def run_gb300(args):
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from ffea_gb300 import partition, workloads
    shard = None
    if world > 1 and workloads.blob_count(args.workload) > 1:
        # an ensemble shards: `world` replicas of the workload's blobs, packed
        # over the ranks by estimated bytes per step (no exchange while stepping)
        plan, loads = partition.ensemble_plan(workloads.blob_radii(args.workload), world)
        specs = workloads.build_items(args.workload, plan[rank], args.precision)
        shard = {"method": "greedy size-balanced bin packing by estimated HBM bytes per step "
                           "(ffea_gb300.partition)", "replicas": world,
                 "blobs_total": sum(len(b) for b in plan), "blobs_per_rank": [len(b) for b in plan],
                 "load_imbalance": max(loads) / (sum(loads) / len(loads))}
    else:
        specs = build_specs(args.workload, rank, args.precision)
    main_arm = measure_arm(args, specs, args.precond, world, local)
    plain = two_level = None
    if main_arm["preconditioner"] != "jacobi" and not args.no_plain:
        plain = measure_arm(args, specs, "jacobi", world, local)
    if main_arm["preconditioner"] == "learned" and not args.no_plain:
        # the same coarse space with every smoother weight 1: what the network adds
        two_level = measure_arm(args, specs, "two-level", world, local)
    if rank != 0:
        return
    nl, ne, nedges = main_arm["sizes"]
    # roofline of the dominant kernel (k_cg): the algorithmic bytes of its
    # iterations over its measured duration
    iters_p = main_arm["cg_iters_profiled"]
    cg_ms = main_arm["phase_ms_per_step"]["cg"]
    alg = int(iters_p * cg_iteration_bytes(nl, nedges)) + 48 * nl  # the iterations, then the Euler update
    peak, peak_kind = measured_peak()
    achieved = alg / (cg_ms / 1e3) / 1e9
    roofline = {"bound": "hbm", "kernel": "k_cg", "achieved": round(achieved, 1), "peak": peak,
                "peak_source": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 4),
                "traffic": ncu_traffic(workload=args.workload), "algorithmic_bytes_per_launch": alg,
                "avg_launch_us": round(cg_ms * 1e3, 1), "cg_iters_per_launch": iters_p,
                "bytes_per_iteration": cg_iteration_bytes(nl, nedges)}
    # every other kernel of the step against the same peak: algorithmic bytes
    # over its event-timed duration in the profile pass (direct launches)
    kernels = {}
    for name, b in step_kernel_bytes(nl, ne, nedges, main_arm["total_nodes"]).items():
        ms = main_arm["kernel_ms"].get(name, 0.0)
        if ms > 0:
            gbs = b / (ms / 1e3) / 1e9
            kernels[name] = {"us": round(ms * 1e3, 1), "algorithmic_bytes": b, "achieved_gbs": round(gbs, 1),
                             "frac": round(gbs / peak, 4)}
    kernels["cg"] = {"us": round(cg_ms * 1e3, 1), "algorithmic_bytes": alg, "achieved_gbs": round(achieved, 1),
                     "frac": round(achieved / peak, 4)}
    if main_arm["kernel_ms"].get("coarse", 0.0) > 0:
        kernels["coarse"] = {"us": round(main_arm["kernel_ms"]["coarse"] * 1e3, 1),
                             "note": "coarse-space refresh (assembly of A_c, one Newton-Schulz update), every "
                                     "tenth step: its time over a ten-step cycle, per step"}
    line = {
        "metric": METRIC, "value": main_arm["value"], "unit": "node-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": main_arm["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64" if args.precision == "mixed" else "f64", "data": "synthetic",
        "config": config_of(args, specs, world), "e2e": main_arm["e2e"], "gpu_launches": main_arm["gpu_launches"],
        "preconditioner": main_arm["preconditioner"], "cg_iters_per_step": main_arm["cg_iters_per_step"],
        "roofline": roofline, "clocks": main_arm["clocks"], "phase_ms_per_step": main_arm["phase_ms_per_step"],
        "cg_us_per_iteration": main_arm["cg_us_per_iteration"], "kernel_roofline": kernels,
    }
    if main_arm["autotune"]:
        line["autotune"] = main_arm["autotune"]
    if shard is not None:
        line["config"]["sharding"] = shard
    line["config"]["edges"] = int(nedges)
    line["config"]["solver"] = (f"CG_nomass, {main_arm['preconditioner']} preconditioner, epsilon 1e-6, "
                                "convergence confirmed by an FP64 true residual")
    arm_keys = ("value", "ms_per_step", "cg_iters_per_step", "cg_us_per_iteration", "e2e", "clocks", "preconditioner")

    def ratio(a, b):
        return {"node_steps_ratio": a["value"] / b["value"], "e2e_ratio": a["e2e"]["value"] / b["e2e"]["value"],
                "iteration_ratio": b["cg_iters_per_step"] / max(a["cg_iters_per_step"], 1e-9)}
    if plain is not None:
        line["plain"] = {k: plain[k] for k in arm_keys}
        line["learned_vs_plain"] = ratio(main_arm, plain)
    if two_level is not None:
        line["two_level"] = {k: two_level[k] for k in arm_keys}
        line["learned_vs_two_level"] = ratio(main_arm, two_level)
        if plain is not None:
            line["two_level_vs_plain"] = ratio(two_level, plain)
    if world == 1 and args.workload == "sphere40" and not args.no_memory_resident:
        kernels["cg_memory_resident"] = memory_resident_roofline(args, peak)
    if world == 1 and not args.no_cpu_baseline:
        base = cpu_baseline(specs, args.cpu_seconds)
        line["cpu_baseline"] = {k: base[k] for k in ("value", "unit", "cores", "kind", "sample")}
    if world == 1 and args.parity_steps > 0:
        line["parity"] = parity_report(args.precond, args.workload if args.workload.startswith("sphere") else "sphere40",
                                       args.parity_steps)
    print(json.dumps(line), flush=True)


def parity_report(precond: str, workload: str = "sphere40", steps: int = 5, small_steps: int = 20):
    """Per-step force (rhs) and velocity error of the measured path against
    an FP64 oracle run (FFEA's algorithm restated), the worst relative
    2-norm difference over the first steps: `steps` steps on the measured
    single-blob workload (the oracle single-stream on all host cores, the
    same draws as one thread) and `small_steps` on the 10 nm sphere.  Both
    sides solve to epsilon 1e-12 (the mixed path down to its FP32 floor)."""
    from ffea_gb300 import learned
    from ffea_gb300.workloads import build_specs as specs_of
    from ffea_gb300.world import World
    from oracle import oracle as O
    O.build(ref=False)
    threads = os.cpu_count() or 1
    out = {"precision": "mixed (the measured path) vs the FP64 oracle", "preconditioner": precond, "bar": 1e-5,
           "epsilon": "1e-12 on both sides", "oracle_threads": threads}
    for key, wl, n in (("", workload, steps), ("small_", "sphere10", small_steps)):
        spec = specs_of(wl, 0, "mixed", epsilon=1e-12)[0]
        ref = O.blob_from_spec(spec, parallel=threads)
        worst_v = worst_f = 0.0
        rng_exact = True
        t0 = time.perf_counter()
        with World([spec], preconditioner=PRECONDS[precond]) as w:
            if precond == "learned" and w.preconditioner() == PRECONDS["learned"]:
                learned.apply(w, learned.load())
            b = w.blob(0)
            for _ in range(n):
                w.run(1)
                if ref.step(1) != 0:
                    raise RuntimeError("oracle step failed in the parity report")
                _, vel, _ = b.get_nodes()
                _, rvel, _ = ref.nodes()
                worst_v = max(worst_v, float(np.linalg.norm(vel - rvel) / np.linalg.norm(rvel)))
                rf = ref.rhs()
                worst_f = max(worst_f, float(np.linalg.norm(b.rhs() - rf) / np.linalg.norm(rf)))
                rng_exact = rng_exact and bool(np.array_equal(b.rng_state(), ref.rng_state()))
        out[key + "workload"] = f"{wl}: {WORKLOADS[wl]['desc']} ({spec.mesh.num_linear:,} linear nodes)"
        out[key + "steps"] = n
        out[key + "max_rel_err_velocity"] = worst_v
        out[key + "max_rel_err_force"] = worst_f
        out[key + "rng_state_bit_exact"] = rng_exact
        out[key + "seconds"] = round(time.perf_counter() - t0, 1)
    return out


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
