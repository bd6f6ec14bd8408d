"""Run a taped forward and its reverse pass on the differentiable workloads, for
profilers and timing sweeps.

    python -m opencloth_gb300.profile_adjoint [--workload batch512] [--instances N]
        [--steps T] [--every K] [--budget-gb B] [--repeat R]

Prints one JSON line: the plain forward, the taped forward and the reverse pass (wall
time around each call, the reverse pass with the gradients left on the device), the
tape's kind and bytes, and the last reverse step's adjoint CG iterations.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

DT = 1.0 / 60.0


def adjoint_workload(name: str, seed: int):
    """The differentiable configurations: one 257 x 257 cloth (200 steps, checkpoint every
    20) and 512 cloths with sides uniform in [16,256] (100 steps, the default interval).
    Returns (descs, X0, per-spring target Ks, steps, interval); the target Ks carry
    log-normal(0, 0.1^2) factors on the cloths' own."""
    from . import ClothDesc, grid_cloth

    rng = np.random.default_rng(seed)
    if name == "grid257":
        sides, steps, every = [257], 200, 20
    else:
        sides, steps, every = list(rng.integers(16, 257, 512)), 100, 0
    descs, Xs, ks_t = [], [], []
    for k, n in enumerate(sides):
        n = int(n)
        if name == "grid257":
            ks, kd = (50.75, 50.75, 50.95), (-0.25, -0.25, -0.25)
        else:
            ks, kd = tuple(np.exp(rng.uniform(np.log(10.0), np.log(500.0), 3))), tuple(rng.uniform(-0.5, -0.05, 3))
        X, sp = grid_cloth(n, n, ks=ks, kd=kd, jitter=1e-3, seed=seed * 7 + k)
        descs.append(ClothDesc(n_vertices=n * n, springs=sp, pinned=np.array([0, n - 1], np.int32),
                               cg_max_iter=200, cg_tol=1e-5))
        Xs.append(X)
        ks_t.append((sp["ks"] * np.exp(rng.normal(0.0, 0.1, len(sp)))).astype(np.float32))
    return descs, np.concatenate(Xs), np.concatenate(ks_t), steps, every


def main() -> None:
    from . import ClothSolver

    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="batch512", choices=("batch512", "grid257"))
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--instances", type=int, default=0, help="the first N cloths only (0: all)")
    ap.add_argument("--steps", type=int, default=0, help="0: the workload's own")
    ap.add_argument("--every", type=int, default=-1, help="-1: the workload's own")
    ap.add_argument("--budget-gb", type=float, default=40.0)
    ap.add_argument("--repeat", type=int, default=1)
    a = ap.parse_args()
    descs, X0, _, steps, every = adjoint_workload(a.workload, a.seed)
    if a.instances:
        descs = descs[:a.instances]
        X0 = X0[:sum(d.n_vertices for d in descs)]
    steps = a.steps or steps
    every = every if a.every < 0 else a.every
    budget = int(a.budget_gb * (1 << 30))
    gX = np.full_like(X0, 1e-6)
    out = {"vertices": len(X0), "instances": len(descs), "steps": steps}
    with ClothSolver(descs) as s:
        def reset():
            s.set_state(X0, np.zeros_like(X0), np.zeros_like(X0))
            s.synchronize()

        for _ in range(a.repeat):
            reset()
            t0 = time.perf_counter()
            s.step(DT, steps)
            s.synchronize()
            out["forward_ms"] = 1e3 * (time.perf_counter() - t0)
            reset()
            t0 = time.perf_counter()
            s.tape_forward(DT, steps, every, budget)
            s.synchronize()
            out["taped_forward_ms"] = 1e3 * (time.perf_counter() - t0)
            t0 = time.perf_counter()
            s.tape_backward(gX, want=())
            out["backward_ms"] = 1e3 * (time.perf_counter() - t0)
        kind, ev = s.tape_layout()
        it, _, _ = s.stats()
        out.update({"tape": kind, "intervals": sorted(set(ev.tolist())), "tape_bytes": s.tape_info()[1],
                    "adjoint_cg_iters_max": int(it.max())})
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
