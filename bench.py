#!/usr/bin/env python3
"""Throughput of the GB300 implicit cloth step, in vertex-steps/s.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload grid1025|batch4096]
    python bench.py --impl reference ...     # the reference's CPU step on the host cores

A step is ComputeForces + IntegrateImplicit (forces, Jacobians, assembly, PCG to the
configured tolerance, update) over every cloth of the workload.

Workloads (synthetic, seeded):
  grid1025   one 1025 x 1025 cloth (1,050,625 vertices, 6,295,552 springs including the
             reference's duplicate bend springs), 4.0 x 4.0 square, Ks 50.75/50.75/50.95,
             Kd -0.25, mass 1, gravity (0,-0.00981,0), dt 1/60, top corners pinned,
             N(0,(1e-3 spacing)^2) position jitter, CG <= 200 iterations to 1e-5.
  batch4096  4096 cloths, side uniform in [8,128], per-type Ks log-uniform [10,500],
             Kd uniform [-0.5,-0.05], same jitter, CG <= 200 iterations to 1e-5.
  coupled1025      grid1025 in the COUPLED Jacobian mode (Baraff-Witkin block-sparse
                   system, block-Jacobi PCG to 1e-5, at most 200 iterations).
  stepphysics1025  grid1025 plus EllipsoidCollision and ApplyProvotDynamicInverse after
                   every step (the reference's whole StepPhysics).

The timed region replays the step's CUDA graph K times on the solver's stream with
inputs resident in HBM; the per-step working set (grid1025: ~0.75 GB) exceeds the 129 MB
L2, so no explicit flush is done.  Multi-GPU runs are replicas (one workload per rank,
no collective on the data path): weak scaling.
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
from dataclasses import dataclass
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

DT = 1.0 / 60.0
METRIC = "vertex-steps/s"


# ---- workloads ------------------------------------------------------------------------
#
# A workload is a list of cloth specifications plus the initial state.  The GPU arm turns
# the specifications into the library's descriptors; the reference arm builds the same
# lattices with the oracle's own builder (bit-identical to the library's, a CPU test checks
# it), so its process never loads the GPU library.

@dataclass
class ClothSpec:
    n_vertices: int
    springs: np.ndarray
    pinned: np.ndarray
    cg_max_iter: int = 200
    cg_tol: float = 1e-5
    coupled: bool = False  # the COUPLED Jacobian mode (no counterpart in the reference)
    passes: bool = False  # EllipsoidCollision and ApplyProvotDynamicInverse after each step


def _grid_builder(impl: str):
    if impl == "reference":
        import oracle

        return oracle.grid_cloth
    from opencloth_gb300 import grid_cloth

    return grid_cloth


def grid1025(seed: int, impl: str = "ours"):
    cols = 1025
    X, sp = _grid_builder(impl)(cols, cols, ks=(50.75, 50.75, 50.95), kd=(-0.25, -0.25, -0.25), jitter=1e-3,
                                seed=seed)
    spec = ClothSpec(n_vertices=cols * cols, springs=sp, pinned=np.array([0, cols - 1], np.int32))
    return [spec], [(cols, cols)], X, np.zeros_like(X)


def batch4096(seed: int, impl: str = "ours", count: int = 4096):
    rng = np.random.default_rng(seed)
    sides = rng.integers(8, 129, count)
    build = _grid_builder(impl)
    specs, shapes, Xs = [], [], []
    for k, n in enumerate(sides):
        n = int(n)
        ks = np.exp(rng.uniform(np.log(10.0), np.log(500.0), 3))
        kd = rng.uniform(-0.5, -0.05, 3)
        X, sp = build(n, n, ks=tuple(ks), kd=tuple(kd), jitter=1e-3, seed=seed * 100003 + k)
        specs.append(ClothSpec(n_vertices=n * n, springs=sp, pinned=np.array([0, n - 1], np.int32)))
        shapes.append((n, n))
        Xs.append(X)
    X = np.concatenate(Xs)
    return specs, shapes, X, np.zeros_like(X)


def coupled1025(seed: int, impl: str = "ours"):
    """grid1025 in the COUPLED Jacobian mode (Baraff-Witkin block-sparse system)."""
    specs, shapes, X, V = grid1025(seed, impl)
    specs[0].coupled = True
    return specs, shapes, X, V


def stepphysics1025(seed: int, impl: str = "ours"):
    """grid1025 with the rest of StepPhysics: the reference's ellipsoid and Provot pass."""
    specs, shapes, X, V = grid1025(seed, impl)
    specs[0].passes = True
    return specs, shapes, X, V


WORKLOADS = {"grid1025": grid1025, "batch4096": batch4096, "coupled1025": coupled1025,
             "stepphysics1025": stepphysics1025}
# The reference arm steps the reference's implicit step alone (ComputeForces +
# IntegrateImplicit); the COUPLED mode has no counterpart there.
REFERENCE_WORKLOADS = ("grid1025", "batch4096")


def to_descs(specs):
    """The library's descriptors for a workload's cloth specifications."""
    from opencloth_gb300 import JAC_COUPLED, PASS_ELLIPSOID, PASS_PROVOT, ClothDesc, reference_ellipsoid

    out = []
    for c in specs:
        d = ClothDesc(n_vertices=c.n_vertices, springs=c.springs, pinned=c.pinned, cg_max_iter=c.cg_max_iter,
                      cg_tol=c.cg_tol)
        if c.coupled:
            d.jacobian_mode = JAC_COUPLED
        if c.passes:
            d.passes = PASS_ELLIPSOID | PASS_PROVOT
            d.ellipsoid, d.ellipsoid_inv = reference_ellipsoid()
        out.append(d)
    return out


def workload_config(name: str, specs, world: int) -> dict:
    """The ``config`` object of a workload's JSON line (the same for both arms)."""
    return {"workload": name, "vertices": int(sum(c.n_vertices for c in specs)),
            "springs": int(sum(len(c.springs) for c in specs)), "instances": len(specs), "dt": DT,
            "cg_max_iter": 200, "cg_tol": 1e-5, "parallelism": f"replicas x{world}",
            "l2": "per-step working set larger than the 129 MB L2; no flush"}


def algorithmic_bytes(kernel: str, n_vertices: int, n_springs: int, first_dir: bool = False) -> int:
    """Bytes a launch must move over n_vertices iterating vertices, each array element
    counted once (device layout: X/V float4 with mass / pin flag in w, 16-byte incidence
    records, FP32 planes).  The library applies the same model per instance and reports
    it from oc_profile_steps; this copy documents it and sizes ncu captures."""
    N, S = n_vertices, n_springs
    if kernel == "k_assemble":
        # X, V 32 + rowptr 4 + own spring ends/params 24 + warm start 12 + A 24 + r 12 + d 12
        # per vertex, plus two 16-byte incidence records per spring.
        return 120 * N + 32 * S
    if kernel == "k_assemble_grid":
        # k_assemble without the incidence records and the row pointer (the neighbours come
        # from the lattice's stencil); rest lengths that vary add the row pointer and 4 B
        # per incidence.
        return 116 * N
    if kernel == "k_cg_dir":
        return (36 if first_dir else 60) * N  # A 24 + d 12 (+ r 12, d write 12)
    if kernel == "k_cg_update":
        return 84 * N  # A 24 + d 12 + x 12 + r 12, write x 12 + r 12
    if kernel == "k_cg_persist":
        # one step's CG passes and the update in one launch: 36 + 60 (it - 1) B for the
        # directions, 84 it B for the updates, 76 B for the closing update; use
        # first_dir=True for one iteration.
        return (36 + 84 + 76) * N if first_dir else (60 + 84) * N
    if kernel == "k_integrate":
        return 76 * N  # X, V 32 + dV 12 in, X, V 32 out
    if kernel == "k_provot":
        return 53 * N + 32 * S  # X 16, V 32, pin flag 1, rowptr 4; two records per spring
    if kernel == "k_cpl_assemble":
        # X, V 32, rowptr 4, warm start 12, P^-1 24, m' 4, r, z, d 36 per vertex; per
        # spring two records in and two 20-byte blocks out.
        return 112 * N + 72 * S
    if kernel == "k_cpl_dir":
        # pin flag 1, z 16 (+ d 16; 16-byte records), m' 4, rowptr 4, q 12 per vertex; per
        # spring the other vertex and the block at both ends.
        return (37 if first_dir else 53) * N + 48 * S
    if kernel == "k_cpl_update":
        return (132 if first_dir else 148) * N  # z, (d), x, r, q, P^-1 in; x, r, d, z out
    raise KeyError(kernel)


# ---- clocks -----------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx.append(float(f[2]))
                except ValueError:
                    continue
                for name, v in zip(names, f[5:9]):
                    if v.lower() == "active":
                        reasons.add(name)
        finally:
            os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---- CPU side (oracle) ------------------------------------------------------------------

def _cpu_worker(args):
    """One process: the oracle port on a list of cloths for a number of steps."""
    import oracle

    items, steps, use_ref = args
    vsteps, secs = 0, 0.0
    for springs, cols, rows, X, i_max, eps in items:
        n = cols * rows
        if use_ref:
            cl = oracle.Cloth(n, springs, num_x=cols - 1, i_max=i_max, eps=eps)
            _, s = oracle.ref_run(cl, cols - 1, rows - 1, X, np.zeros_like(X), snaps=(steps,), timed=True)
        else:
            cl = oracle.Cloth(n, springs, pinned=[0, cols - 1], i_max=i_max, eps=eps)
            t0 = time.perf_counter()
            oracle.port_step(cl, X, np.zeros_like(X), n_steps=steps, filter_pinned=True)
            s = time.perf_counter() - t0
        vsteps += n * steps
        secs += s
    return vsteps, secs


def cpu_throughput(workload: str, descs, shapes, X, budget_s: float, processes: int):
    """The reference step (or its port) on a bounded sample of the same workload
    (``descs``: the cloth specifications).  Returns (vertex-steps/s, cores, kind, sample
    description)."""
    import oracle

    oracle.build(reference=True)
    use_ref = oracle.ref_available()
    kind = "reference" if use_ref else "port"
    offs = np.cumsum([0] + [d.n_vertices for d in descs])
    items = [(d.springs, c, r, X[offs[k]:offs[k + 1]], d.cg_max_iter, d.cg_tol)
             for k, (d, (c, r)) in enumerate(zip(descs, shapes))]
    if len(items) == 1:
        # One cloth: the reference is serial.  Time single steps until the budget is spent.
        t0, steps, vs, secs = time.perf_counter(), 0, 0, 0.0
        Xc = items[0][3]
        while True:
            v, s = _cpu_worker(([items[0][:3] + (Xc,) + items[0][4:]], 1, use_ref))
            vs, secs, steps = vs + v, secs + s, steps + 1
            if time.perf_counter() - t0 >= budget_s:
                break
        c, r = shapes[0]
        return vs / secs, 1, kind, f"{steps} step(s) of the full {c}x{r} cloth from its initial state, 1 thread"
    # Batch: a size-spanning subset of cloths, one process per core, 3 steps each.
    order = np.argsort([it[1] * it[2] for it in items])
    pick = order[np.linspace(0, len(order) - 1, min(len(order), 8 * processes)).astype(int)]
    chunks = [[items[i] for i in pick[j::processes]] for j in range(processes)]
    import multiprocessing as mp

    steps = 3
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(processes) as pool:
        res = pool.map(_cpu_worker, [(c, steps, use_ref) for c in chunks if c])
    wall = time.perf_counter() - t0
    vs = sum(r[0] for r in res)
    return vs / wall, processes, kind, (f"{len(pick)} cloths spanning the size range x {steps} steps, "
                                        f"{processes} processes (one per core)")


# ---- arms -------------------------------------------------------------------------------

def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(v: float, world: int, device: str = "cuda") -> float:
    """The maximum of v over the ranks (the timed region's length is the slowest rank's);
    device "cpu" for a gloo group."""
    if world == 1:
        return v
    import torch

    t = torch.tensor([v], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def aggregate_value(vertices_per_rank: int, steps: int, world: int, ms: float) -> float:
    """Whole-job vertex-steps/s: every rank's vertices times the steps, over the slowest
    rank's time (weak scaling: each rank steps its own replica)."""
    return vertices_per_rank * steps * world / (ms / 1e3)


def run_reference(args) -> None:
    """The reference's CPU step (the reference build where it exists, else the oracle's
    restatement of it) on the GPU arm's workload and config; rank 0 only.  The process
    builds its inputs with the oracle and never loads the GPU library."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    name = "grid1025" if args.workload == "all" else args.workload
    if name not in REFERENCE_WORKLOADS:
        print(json.dumps({"impl": "reference", "unavailable": f"{name} has no counterpart in the reference"}),
              flush=True)
        return
    specs, shapes, X, _ = WORKLOADS[name](args.seed, impl="reference")
    nv = sum(c.n_vertices for c in specs)
    procs = max(1, os.cpu_count() or 1)
    budget = min(120.0, 2.0 * max(args.steps, 1))
    value, cores, kind, sample = cpu_throughput(name, specs, shapes, X, budget, procs)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * nv / value, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(name, specs, world),
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": cores, "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _traffic(kernel: str, workload: str):
    """ncu's DRAM bytes per launch of the kernel on the workload, from its summary in
    profiles/ (None when no capture exists)."""
    tpath = ROOT / "profiles" / f"{kernel}_{workload}.traffic.json"
    return json.loads(tpath.read_text()).get("dram_bytes_per_launch") if tpath.exists() else None


def _dominant_roofline(prof: dict, peak: float, workload: str) -> dict:
    """Roofline of the kernel with the largest share of the step: its algorithmic bytes
    (reported by the library for the instances still iterating) over its CUDA-event
    durations, summed over the profiled launches."""
    dom = max(prof, key=lambda k: prof[k]["ms_total"])
    n = max(prof[dom]["launches"], 1)
    secs = prof[dom]["ms_total"] / 1e3
    achieved = prof[dom]["bytes"] / secs / 1e9
    traffic = _traffic(dom, workload)
    return {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": traffic, "algorithmic_bytes_per_launch": prof[dom]["bytes"] / n,
            "avg_launch_us": 1e6 * secs / n}


def _cg_roofline(prof: dict, peak: float) -> dict:
    """The SpMV-bound CG kernels the step actually launched (persistent, block-resident,
    direction/update or the COUPLED pair), their algorithmic bytes over their summed
    CUDA-event durations."""
    cg = ["k_cg_persist", "k_resident", "k_cg_dir", "k_cg_update", "k_cpl_dir", "k_cpl_update"]
    pair = [k for k in cg if k in prof and prof[k]["launches"] > 0]
    if not pair:
        return None
    byts = sum(prof[k]["bytes"] for k in pair)
    secs = sum(prof[k]["ms_total"] for k in pair) / 1e3
    achieved = byts / secs / 1e9 if secs > 0 else 0.0
    return {"bound": "hbm", "kernels": pair, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak}


def measure(name: str, args, steps: int, rank: int, world: int, local: int, plain_steps: int) -> dict:
    """Time one workload on this rank; returns the figures rank 0 reports."""
    import torch

    from opencloth_gb300 import ClothSolver

    specs, shapes, X0, V0 = WORKLOADS[name](args.seed + 7919 * rank)
    descs = to_descs(specs)
    nv = sum(d.n_vertices for d in descs)
    ns = sum(len(d.springs) for d in descs)
    stream = torch.cuda.Stream()
    solver = ClothSolver(descs, device=local, stream=stream.cuda_stream)
    solver.set_state(X0, V0)
    # The library's autotuner picks the launch configuration on this workload and state
    # (untimed set-up; the state is left as it was).
    t0 = time.perf_counter()
    tuned, tuned_ms = solver.autotune(DT, cache_path=tune_cache_path())
    tune_s = time.perf_counter() - t0
    solver.step(DT, args.warmup)
    solver.synchronize()
    l0 = solver.launch_count()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def slowest(v: float) -> float:
        return max_over_ranks(v, world)

    barrier()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        ev0.record(stream)
        solver.step(DT, steps)
        ev1.record(stream)
        ev1.synchronize()
    barrier()
    ms = slowest(ev0.elapsed_time(ev1))
    launches = solver.launch_count() - l0
    iters, rr, flags = solver.stats()
    value = aggregate_value(nv, steps, world, ms)

    prof = solver.profile(DT, 3)
    peaks_path = ROOT / "MEASURED_PEAKS.json"
    peak = float(json.loads(peaks_path.read_text())["hbm_gbs"]) if peaks_path.exists() else 6800.0
    roof = _dominant_roofline(prof, peak, name)
    roof["peak_source"] = "measured" if peaks_path.exists() else "fallback"
    cg_roof = _cg_roofline(prof, peak)
    if cg_roof is not None and cg_roof["kernels"] == ["k_resident"]:
        # The resident kernel keeps the CG on chip, so its HBM figure counts only the state
        # it loads and stores.  Beside it: the CG's algorithmic bytes in the streamed
        # layout (first direction 36 B, 60 B per later direction pass, 84 B per update
        # pass, 76 B for the update, per vertex) over the resident kernel's time.
        it_p, _, _ = solver.stats()
        nv_k = np.array([d.n_vertices for d in descs], np.float64)
        itk = it_p.astype(np.float64)
        per_step = float(np.sum(nv_k * np.where(itk > 0, 36 + 60 * (itk - 1) + 84 * itk + 76, 76)))
        secs = prof["k_resident"]["ms_total"] / 1e3
        eq = 3 * per_step / secs / 1e9 if secs > 0 else 0.0
        # Not an HBM figure: the iterations run in shared memory and registers, so this is the
        # kernel's on-chip throughput and carries no fraction of the HBM peak.
        cg_roof["on_chip"] = {"streamed_layout_bytes_per_s": eq * 1e9, "bytes_per_step": per_step,
                              "note": "the CG's algorithmic bytes in the streamed layout over k_resident's time; "
                                      "its HBM use is the 'achieved' figure above"}

    # End to end through the public API with host buffers: each step copies pinned
    # host X, V in, runs the step and reads X, V back (oc_step_host: StepPhysics on host
    # arrays, one wait per step).
    e2e_steps = max(5, min(steps, 50 if nv < 4_000_000 else 10))
    Xh = torch.empty((nv, 3), dtype=torch.float32, pin_memory=True).numpy()
    Vh = torch.empty((nv, 3), dtype=torch.float32, pin_memory=True).numpy()
    solver.get_state_into(Xh, Vh, None)
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        solver.step_host(Xh, Vh, DT, 1)
    e2e_s = slowest(time.perf_counter() - t0)
    e2e = {"value": aggregate_value(nv, e2e_steps, world, 1e3 * e2e_s), "unit": METRIC, "h2d_bytes_per_step": 24 * nv,
           "d2h_bytes_per_step": 24 * nv, "steps": e2e_steps}
    # The same with pageable host arrays (plain numpy), as a caller passing its own
    # std::vector storage would (the copies then go through the driver's staging).
    Xp, Vp = np.array(Xh), np.array(Vh)
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        solver.step_host(Xp, Vp, DT, 1)
    e2e_p = slowest(time.perf_counter() - t0)
    e2e_pageable = {"value": aggregate_value(nv, e2e_steps, world, 1e3 * e2e_p), "unit": METRIC,
                    "h2d_bytes_per_step": 24 * nv, "d2h_bytes_per_step": 24 * nv, "steps": e2e_steps}
    solver.close()

    # The plain GPU step on the same inputs: the same kernels, one launch sequence per
    # cloth, the CG loop driven from the host.
    plain_gpu = None
    if plain_steps > 0:
        plain = ClothSolver(descs, device=local, stream=stream.cuda_stream, executor="plain")
        plain.set_state(X0, V0)
        plain.step(DT, 1)
        plain.synchronize()
        barrier()
        ev0.record(stream)
        plain.step(DT, plain_steps)
        ev1.record(stream)
        ev1.synchronize()
        pms = slowest(ev0.elapsed_time(ev1))
        plain_value = aggregate_value(nv, plain_steps, world, pms)
        plain.close()
        plain_gpu = {"value": plain_value, "unit": METRIC, "ms_per_step": pms / plain_steps, "steps": plain_steps,
                     "speedup": value / plain_value}

    return {
        "name": name, "specs": specs, "descs": descs, "shapes": shapes, "X0": X0, "nv": nv, "ns": ns, "value": value,
        "ms_per_step": ms / steps, "steps": steps, "launches": launches, "clocks": clocks.summary(),
        "cg": {"iters_last_step_max": int(iters.max()), "iters_last_step_mean": float(iters.mean()),
               "rel_residual_max": float(rr.max()), "flags_any": int(np.bitwise_or.reduce(flags))},
        "roofline": roof, "cg_roofline": cg_roof, "e2e": e2e, "e2e_pageable": e2e_pageable,
        "kernels": {k: {"avg_us": 1e3 * v["ms_total"] / max(v["launches"], 1), "launches": v["launches"]}
                    for k, v in prof.items()},
        "plain_gpu": plain_gpu,
        "launch_config": {"chosen": tuned, "tuner_ms_per_step": tuned_ms, "tuning_s": tune_s},
    }


def tune_cache_path() -> str:
    """The autotuner's cache file: OC_TUNE_CACHE, else ~/.cache/opencloth_gb300/tune.txt."""
    p = os.environ.get("OC_TUNE_CACHE")
    if p:
        return p
    d = Path.home() / ".cache" / "opencloth_gb300"
    d.mkdir(parents=True, exist_ok=True)
    return str(d / "tune.txt")


def measure_adjoint(name: str, seed: int, local: int) -> dict:
    """Forward, taped forward and reverse pass times of one gradient evaluation: the
    reverse pass with the gradients left on the device (backward_ms) and with all of them
    copied to host arrays (backward_e2e_ms); both upload dL/dX_T from a host array."""
    import torch

    from opencloth_gb300 import ClothSolver

    from opencloth_gb300.profile_adjoint import adjoint_workload

    descs, X0, ks_target, steps, every = adjoint_workload(name, seed)
    nv = len(X0)
    budget = 40 << 30
    # The single cloth barely moves (about 1e-3 in 200 steps from rest): its taped forward
    # runs in the displacement mode, which resolves the small loss residual; the batch of
    # 512 cloths (more than one cooperative launch takes) tapes positions.
    displacement = len(descs) == 1
    with ClothSolver(descs, device=local) as s:
        s.set_tape_mode(displacement)
        ks0 = np.concatenate([d.springs["ks"] for d in descs])
        s.set_spring_params(ks=ks_target)
        s.set_state(X0, np.zeros_like(X0), np.zeros_like(X0))
        s.step(DT, steps)
        target, _, _ = s.get_state()
        s.set_spring_params(ks=ks0)

        def reset():
            s.set_state(X0, np.zeros_like(X0), np.zeros_like(X0))
            s.synchronize()

        reset()
        t0 = time.perf_counter()
        s.step(DT, steps)
        s.synchronize()
        fwd = time.perf_counter() - t0
        offs = s.offsets

        def loss_grad():
            if displacement:
                X = X0.astype(np.float64) + s.tape_displacement().astype(np.float64)
            else:
                X, _, _ = s.get_state()
            gX = np.empty_like(X)
            for k in range(len(descs)):
                sl = slice(offs[k], offs[k + 1])
                gX[sl] = 2.0 * (X[sl] - target[sl]) / (offs[k + 1] - offs[k])
            return gX

        # One untimed gradient evaluation first (the tape's buffers and the adjoint
        # solve's graph are built on first use), as the forward has its warm-up steps.
        reset()
        s.tape_forward(DT, steps, every, budget)
        s.tape_backward(loss_grad())
        reset()
        t0 = time.perf_counter()
        s.tape_forward(DT, steps, every, budget)
        tape = time.perf_counter() - t0
        gX = loss_grad()
        t0 = time.perf_counter()
        g = s.tape_backward(gX)
        bwd_e2e = time.perf_counter() - t0
        every_used, tape_bytes = s.tape_info()
        kind, intervals = s.tape_layout()
        # The same reverse pass with the gradients left on the device (every gradient is
        # still computed; only the copies to host arrays are left out).
        reset()
        s.tape_forward(DT, steps, every, budget)
        gX = loss_grad()
        t0 = time.perf_counter()
        s.tape_backward(gX, want=())
        bwd = time.perf_counter() - t0
    torch.cuda.synchronize()
    per_interval = {int(e): int((intervals == e).sum()) for e in np.unique(intervals)}
    return {"vertices": nv, "instances": len(descs), "steps": steps, "checkpoint_every": every_used,
            "tape_mode": "displacement" if displacement else "positions", "tape": kind,
            "cloths_per_interval": per_interval, "budget_bytes": budget, "tape_bytes": tape_bytes, "forward_ms": 1e3 * fwd, "taped_forward_ms": 1e3 * tape,
            "backward_ms": 1e3 * bwd, "backward_to_forward": bwd / fwd, "gradient_to_forward": (tape + bwd) / fwd,
            "backward_e2e_ms": 1e3 * bwd_e2e, "gradient_to_forward_e2e": (tape + bwd_e2e) / fwd,
            "gradients_per_s": len(descs) / (tape + bwd_e2e),
            "grad_norm_ks": float(np.linalg.norm(g["dKs"])), "finite": bool(np.isfinite(g["dKs"]).all())}


def fem_workload(name: str, seed: int):
    """The FEM demo's CG on systems the demo's assembly builds at rest (opencloth_gb300.fem,
    restating FEM:240-405, 659-831) with random velocities N(0, 0.1^2), i_max 20:
      fem160x48x48   one mesh of 160 x 48 x 48 cubes (386,561 block rows, 4.9M blocks)
      fem_batch4096  4096 bodies of the demo's own 10 x 3 x 3 mesh (176 rows each)."""
    from opencloth_gb300.fem import fem_system

    rng = np.random.default_rng(seed)
    if name == "fem160x48x48":
        n = 161 * 49 * 49
        g = fem_system(160, 48, 48, V=rng.normal(0.0, 0.1, (n, 3)))
        return [g]
    base = fem_system(10, 3, 3)
    out = []
    mass_b = None
    for _ in range(4096):
        V = rng.normal(0.0, 0.1, base["V"].shape)
        V[base["fixed"] == 1] = 0.0
        if mass_b is None:  # b = b0 + V m: recover m from one assembly with unit velocity
            ones = fem_system(10, 3, 3, V=np.ones_like(base["V"]))
            mass_b = (ones["b"].astype(np.float64) - base["b"])[:, :1]
        d = dict(base)
        with np.errstate(invalid="ignore"):
            d["b"] = (base["b"] + V * mass_b).astype(np.float32)
        d["V"] = V.astype(np.float32)
        out.append(d)
    return out


def measure_fem(name: str, seed: int, local: int, solves: int) -> dict:
    """The batched block-sparse CG: solves/s and block-row iterations/s on the device,
    end to end through the C ABI with host buffers, the SpMV roofline and the oracle's
    restatement (bit-exact to the reference's CG) on the host cores."""
    import torch

    import oracle
    from opencloth_gb300.fem import BsrSolver

    systems = fem_workload(name, seed)
    rows = sum(len(g["row_ptr"]) - 1 for g in systems)
    iters = systems[0]["i_max"]
    blocks = np.concatenate([g["blocks"] for g in systems])
    b = np.concatenate([g["b"] for g in systems])
    V0 = np.concatenate([g["V"] for g in systems])
    stream = torch.cuda.Stream()
    s = BsrSolver(systems, device=local, stream=stream.cuda_stream)
    s.set_system(blocks, b, V0)
    for _ in range(3):
        s.solve()
    s.synchronize()
    l0 = s.launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        ev0.record(stream)
        for _ in range(solves):
            s.solve()
        ev1.record(stream)
        ev1.synchronize()
    ms = ev0.elapsed_time(ev1) / solves
    launches = s.launch_count() - l0
    prof = s.profile(2)
    peaks_path = ROOT / "MEASURED_PEAKS.json"
    peak = float(json.loads(peaks_path.read_text())["hbm_gbs"]) if peaks_path.exists() else 6800.0
    # The dominant kernel: the streamed matrix-vector pass, or the resident CG when every
    # system runs on chip (the demo's 176-row bodies).
    kname = max(("k_bsr_spmv", "k_bsr_resident"), key=lambda k: prof.get(k, {"ms_total": 0.0})["ms_total"])
    dom = prof[kname]
    achieved = dom["bytes"] / (dom["ms_total"] / 1e3) / 1e9 if dom["ms_total"] > 0 else 0.0
    roof = {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "algorithmic_bytes_per_launch": dom["bytes"] / max(dom["launches"], 1),
            "avg_launch_us": 1e3 * dom["ms_total"] / max(dom["launches"], 1),
            "traffic": _traffic(kname, name),
            "peak_source": "measured" if peaks_path.exists() else "fallback"}
    if kname == "k_bsr_resident":
        # The iterations run in shared memory, so the HBM figure counts the blocks and rows
        # read once and the solution written.  Beside it: the solve's algorithmic bytes in
        # the streamed layout (pack 72 B/block + 8 B/row, init 40 B/block + 61 B/row, per
        # iteration 40 B/block + 162 B/row) over the resident kernel's time.
        nnzb_r = float(len(blocks))
        per_solve = 72 * nnzb_r + 8 * rows + 40 * nnzb_r + 61 * rows + iters * (40 * nnzb_r + 162 * rows)
        secs = dom["ms_total"] / 1e3 / max(dom["launches"], 1)
        eq = per_solve / secs / 1e9 if secs > 0 else 0.0
        # Not an HBM figure (the iterations run in shared memory): on-chip throughput only.
        roof["on_chip"] = {"streamed_layout_bytes_per_s": eq * 1e9, "bytes_per_solve": per_solve,
                           "note": "the solve's algorithmic bytes in the streamed layout over k_bsr_resident's "
                                   "time; its HBM use is the 'achieved' figure above"}
    # End to end: host blocks, b and V in, solve, V out, every solve.
    e2e_n = max(3, min(solves, 10))
    Vh = np.empty_like(V0)
    t0 = time.perf_counter()
    for _ in range(e2e_n):
        s.set_system(blocks, b, V0)
        s.solve()
        Vh[:], _ = s.solution()
    e2e_s = (time.perf_counter() - t0) / e2e_n
    s.close()
    # CPU: the restatement of ConjugateGradientSolver on a bounded sample, one core.
    sample = systems if name == "fem160x48x48" else systems[:256]
    t0 = time.perf_counter()
    for g in sample:
        oracle.bsr_cg(oracle.BsrSystem(g["row_ptr"], g["col"], g["blocks"], g["b"], g["V"], g["fixed"], g["i_max"]))
    cpu_s = time.perf_counter() - t0
    cpu_rows = sum(len(g["row_ptr"]) - 1 for g in sample)
    nnzb = len(blocks)
    return {
        "workload": name, "systems": len(systems), "block_rows": rows, "blocks": nnzb, "iterations": iters,
        "metric": "block-row-iterations/s", "value": rows * iters / (ms / 1e3), "ms_per_solve": ms,
        "solves_per_s": 1e3 / ms, "solves": solves, "gpu_launches": int(launches), "clocks": clocks.summary(),
        "e2e": {"value": rows * iters / e2e_s, "unit": "block-row-iterations/s",
                "h2d_bytes_per_solve": int(blocks.nbytes + b.nbytes + V0.nbytes), "d2h_bytes_per_solve": int(2 * V0.nbytes)},  # V and the residual
        "roofline": roof,
        "kernels": {k: {"avg_us": 1e3 * v["ms_total"] / max(v["launches"], 1), "launches": v["launches"]}
                    for k, v in prof.items()},
        "cpu_baseline": {"value": cpu_rows * iters / cpu_s, "unit": "block-row-iterations/s", "cores": 1,
                         "kind": "port", "sample": f"{len(sample)} of {len(systems)} systems, one solve each"},
    }


def run_ours(args) -> None:
    import torch

    from opencloth_gb300.build import build

    rank, world, local = dist_env()
    build()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    names = (["grid1025", "batch4096", "coupled1025", "stepphysics1025"] if args.workload == "all"
             else [args.workload])
    plain_steps = {"grid1025": 20, "batch4096": 2, "coupled1025": 3, "stepphysics1025": 0}
    results = []
    for name in names:
        steps = args.steps if name == names[0] else max(10, args.steps // 20)
        results.append(measure(name, args, steps, rank, world, local, plain_steps[name]))
    if rank == 0:
        r = results[0]
        cpu_v, cores, kind, sample = cpu_throughput(r["name"], r["specs"], r["shapes"], r["X0"], 12.0,
                                                    max(1, os.cpu_count() or 1))
        line = {
            "metric": METRIC, "value": r["value"], "unit": METRIC, "n_gpus": world, "steps": r["steps"],
            "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(r["name"], r["specs"], world),
            "cg": r["cg"], "gpu_launches": int(r["launches"]), "clocks": r["clocks"], "e2e": r["e2e"],
            "e2e_pageable": r["e2e_pageable"],
            "roofline": r["roofline"], "cg_roofline": r["cg_roofline"], "kernels": r["kernels"],
            "plain_gpu": r["plain_gpu"], "launch_config": r["launch_config"],
            "cpu_baseline": {"value": cpu_v, "unit": METRIC, "cores": cores, "kind": kind, "sample": sample},
        }
        if args.workload == "all":
            line["adjoint"] = {n: measure_adjoint(n, args.seed, local) for n in ("grid257", "batch512")}
            line["fem_cg"] = {n: measure_fem(n, args.seed, local, 20) for n in ("fem160x48x48", "fem_batch4096")}
        for b in results[1:]:
            line[b["name"]] = {
                "value": b["value"], "unit": METRIC, "ms_per_step": b["ms_per_step"], "steps": b["steps"],
                "vertices": b["nv"], "springs": b["ns"], "instances": len(b["descs"]), "cg": b["cg"],
                "gpu_launches": int(b["launches"]), "clocks": b["clocks"], "e2e": b["e2e"],
                "e2e_pageable": b["e2e_pageable"],
                "roofline": b["roofline"], "cg_roofline": b["cg_roofline"], "kernels": b["kernels"],
                "plain_gpu": b["plain_gpu"], "launch_config": b["launch_config"],
            }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + ["all"], default="all",
                    help="all: the 1M-vertex cloth (headline value), the 4096-cloth batch, the 1M-vertex "
                         "cloth in the COUPLED mode and with the StepPhysics passes")
    ap.add_argument("--seed", type=int, default=20261203)
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
