"""Gradient check of the 257 x 257 differentiable configuration against FP64 central
differences (the oracle run in FP64 with a tight CG tolerance).

    python tests/gradcheck_config.py [--directions 32] [--procs N] [--steps 200]

Configuration: 257 x 257 cloth (Ks 50.75/50.75/50.95, Kd -0.25, jitter 1e-3), 200 steps,
checkpoint every 20; target = final positions of a run whose per-spring Ks carry
log-normal(0, 0.1^2) factors; loss = mean squared distance to the target; gradients with
respect to per-spring Ks and Kd, the initial velocities and a constant per-vertex external
force, compared along random joint directions (eps 1e-4 relative).

Prints one JSON line with the relative error of the directional-derivative vector
||ad - fd|| / ||fd||, the per-direction errors, and the two figures that bound what an
FP32 forward can reach: the loss residual X_T - target and the FP32 error of X_T.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(Path(__file__).resolve().parent))

DT = 1.0 / 60.0
REL_EPS = 1e-4


def build_case(cols: int, steps: int, seed: int):
    from opencloth_gb300 import grid_cloth

    X, sp = grid_cloth(cols, cols, ks=(50.75, 50.75, 50.95), kd=(-0.25, -0.25, -0.25), jitter=1e-3, seed=seed)
    rng = np.random.default_rng(seed)
    sp_t = sp.copy()
    sp_t["ks"] = (sp["ks"] * np.exp(rng.normal(0.0, 0.1, len(sp)))).astype(np.float32)
    return X, sp, sp_t, np.array([0, cols - 1], np.int32)


def fp64_final(springs, X, V0, ext, pins, steps):
    import oracle

    cl = oracle.Cloth(len(X), springs, pinned=pins, i_max=2000, eps=1e-10, ext_force=ext)
    Xo, _, _, _, _ = oracle.port_step(cl, X, V0, n_steps=steps, fp64=True, dot_fp64=True, filter_pinned=True)
    return Xo


def _loss_job(args):
    springs, X, V0, ext, pins, steps, target = args
    Xo = fp64_final(springs, X, V0, ext, pins, steps)
    return float(np.mean(np.sum((Xo - target) ** 2, axis=1)))


def perturb(sp, V0, ext, u, sign):
    s = sp.copy()
    for name in ("ks", "kd"):
        s[name] = (sp[name].astype(np.float64) * (1 + sign * REL_EPS * u[name])).astype(np.float32)
    sc_v = REL_EPS * max(np.abs(V0).max(), 1e-3)
    sc_e = REL_EPS * max(np.abs(ext).max(), 1e-3)
    v = (V0.astype(np.float64) + sign * sc_v * u["V0"]).astype(np.float32)
    e = (ext.astype(np.float64) + sign * sc_e * u["ext"]).astype(np.float32)
    return s, v, e


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--cols", type=int, default=257)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--every", type=int, default=20)
    ap.add_argument("--directions", type=int, default=32)
    ap.add_argument("--procs", type=int, default=max(1, os.cpu_count() or 1))
    ap.add_argument("--seed", type=int, default=20261204)
    a = ap.parse_args()
    import oracle

    oracle.build(reference=False)
    X, sp, sp_t, pins = build_case(a.cols, a.steps, a.seed)
    V0 = np.zeros_like(X)
    ext = np.zeros_like(X)
    pool = mp.get_context("spawn").Pool(a.procs)  # before any GPU work
    target = fp64_final(sp_t, X, V0, ext, pins, a.steps)
    X64 = fp64_final(sp, X, V0, ext, pins, a.steps)

    from opencloth_gb300 import ClothDesc, ClothSolver

    desc = ClothDesc(n_vertices=len(X), springs=sp, pinned=pins, cg_max_iter=500, cg_tol=1e-6)
    with ClothSolver(desc) as s:
        s.set_ext_force(ext)
        s.set_state(X, V0, np.zeros_like(X))
        t0 = time.perf_counter()
        s.tape_forward(DT, a.steps, a.every)
        XT, _, _ = s.get_state()
        gX = 2.0 * (XT.astype(np.float64) - target) / len(X)
        g = s.tape_backward(gX)
        t_grad = time.perf_counter() - t0

    rng = np.random.default_rng(a.seed + 1)
    dirs, jobs = [], []
    for _ in range(a.directions):
        u = {"ks": rng.normal(size=len(sp)), "kd": rng.normal(size=len(sp)), "V0": rng.normal(size=X.shape),
             "ext": rng.normal(size=X.shape)}
        sp_p, v_p, e_p = perturb(sp, V0, ext, u, +1)
        sp_m, v_m, e_m = perturb(sp, V0, ext, u, -1)
        d = {"ks": sp_p["ks"].astype(np.float64) - sp_m["ks"], "kd": sp_p["kd"].astype(np.float64) - sp_m["kd"],
             "V0": v_p.astype(np.float64) - v_m, "ext": e_p.astype(np.float64) - e_m}
        dirs.append(d)
        jobs += [(sp_p, X, v_p, e_p, pins, a.steps, target), (sp_m, X, v_m, e_m, pins, a.steps, target)]
    t0 = time.perf_counter()
    losses = pool.map(_loss_job, jobs)
    t_fd = time.perf_counter() - t0
    pool.close()
    fd = np.array([losses[2 * k] - losses[2 * k + 1] for k in range(a.directions)])
    key = {"ks": "dKs", "kd": "dKd", "V0": "dV0", "ext": "dext"}
    ad = np.array([sum(float(np.sum(g[key[n]].astype(np.float64).reshape(d[n].shape) * d[n])) for n in key)
                   for d in dirs])
    per = np.abs(ad - fd) / np.maximum(np.abs(fd), 1e-300)
    out = {
        "config": f"{a.cols}x{a.cols} cloth, {a.steps} steps, checkpoint every {a.every}",
        "directions": a.directions, "rel_eps": REL_EPS,
        "rel_err_vector": float(np.linalg.norm(ad - fd) / np.linalg.norm(fd)),
        "rel_err_per_direction_median": float(np.median(per)), "rel_err_per_direction_max": float(per.max()),
        "loss_residual_rms": float(np.sqrt(np.mean((X64 - target) ** 2))),
        "fp32_final_state_err_rms": float(np.sqrt(np.mean((XT - X64) ** 2))),
        "gpu_gradient_s": t_grad, "fd_s": t_fd, "fd_procs": a.procs,
    }
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
