"""Run a few implicit steps of a synthetic workload, for profilers and launch-shape sweeps.

    python -m opencloth_gb300.profile_step --cols 1025 --steps 3 [--vpt 4] [--instances 1] [--coupled] [--passes]

Prints one JSON line: graph-replayed ms/step (CUDA events on the solver's stream) and
the per-kernel average durations of an un-graphed pass.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import JAC_COUPLED, JAC_REFERENCE, PASS_ELLIPSOID, PASS_PROVOT, ClothDesc, ClothSolver, grid_cloth
from .cloth import reference_ellipsoid


def workload(cols: int, instances: int, seed: int, random_sides: bool, coupled: bool = False, passes: bool = False):
    rng = np.random.default_rng(seed)
    descs, Xs = [], []
    for k in range(instances):
        n = int(rng.integers(8, 129)) if random_sides else cols
        ks = np.exp(rng.uniform(np.log(10.0), np.log(500.0), 3)) if random_sides else (50.75, 50.75, 50.95)
        kd = rng.uniform(-0.5, -0.05, 3) if random_sides else (-0.25, -0.25, -0.25)
        X, sp = grid_cloth(n, n, ks=tuple(ks), kd=tuple(kd), jitter=1e-3, seed=seed + k)
        E, Einv = reference_ellipsoid() if passes else (None, None)
        descs.append(ClothDesc(n_vertices=n * n, springs=sp, pinned=np.array([0, n - 1], np.int32),
                               cg_max_iter=200, cg_tol=1e-5, jacobian_mode=JAC_COUPLED if coupled else JAC_REFERENCE,
                               passes=(PASS_ELLIPSOID | PASS_PROVOT) if passes else 0, ellipsoid=E,
                               ellipsoid_inv=Einv))
        Xs.append(X)
    return descs, np.concatenate(Xs)


def main() -> None:
    import torch

    ap = argparse.ArgumentParser()
    ap.add_argument("--cols", type=int, default=1025)
    ap.add_argument("--instances", type=int, default=1)
    ap.add_argument("--random-sides", action="store_true", help="sides uniform in [8,128], random Ks/Kd")
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--vpt", type=int, default=0)
    ap.add_argument("--executor", default="auto")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--no-profile", action="store_true")
    ap.add_argument("--no-graph", action="store_true", help="launch kernels directly (CG loop driven from the host)")
    ap.add_argument("--own-stream", action="store_true", help="let the library create its stream")
    ap.add_argument("--coupled", action="store_true", help="COUPLED Jacobian mode")
    ap.add_argument("--passes", action="store_true", help="ellipsoid collision and Provot pass after each step")
    a = ap.parse_args()
    t0 = time.perf_counter()
    descs, X = workload(a.cols, a.instances, a.seed, a.random_sides, a.coupled, a.passes)
    stream = torch.cuda.Stream()
    s = ClothSolver(descs, stream=None if a.own_stream else stream.cuda_stream, vertices_per_thread=a.vpt,
                    executor=a.executor, use_graph=not a.no_graph)
    s.set_state(X, np.zeros_like(X))
    setup = time.perf_counter() - t0
    s.step(1.0 / 60.0, a.warmup)
    s.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    w0 = time.perf_counter()
    e0.record(stream)
    s.step(1.0 / 60.0, a.steps)
    s.synchronize()
    e1.record(stream)
    e1.synchronize()
    wall_ms = 1e3 * (time.perf_counter() - w0) / max(a.steps, 1)
    ms = e0.elapsed_time(e1) / max(a.steps, 1)
    if a.own_stream:
        ms = wall_ms
    it, rr, fl = s.stats()
    out = {"vertices": s.n_vertices, "springs": s.n_springs, "instances": s.n_instances, "vpt": a.vpt,
           "executor": a.executor, "graph": not a.no_graph, "ms_per_step": ms, "wall_ms_per_step": wall_ms, "vertex_steps_per_s": s.n_vertices / (ms / 1e3),
           "iters_max": int(it.max()), "residual_max": float(rr.max()), "flags": int(np.bitwise_or.reduce(fl)),
           "setup_s": setup}
    if not a.no_profile:
        prof = s.profile(1.0 / 60.0, 2)
        out["kernels_us"] = {k: 1e3 * v["ms_total"] / max(v["launches"], 1) for k, v in prof.items()}
    print(json.dumps(out), flush=True)
    s.close()


if __name__ == "__main__":
    main()
