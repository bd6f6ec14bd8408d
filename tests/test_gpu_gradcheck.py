"""Gradient check of the differentiable single-cloth configuration against FP64 central
differences (the oracle stepped in FP64 with a tight CG tolerance).

Configuration: 257 x 257 cloth (Ks 50.75/50.75/50.95, Kd -0.25, jitter 1e-3 of the
spacing), V0 = 0, 200 steps, checkpoint every 20; target = final positions of an FP64 run
whose per-spring Ks carry log-normal(0, 0.1^2) factors; loss = mean squared distance to
the target; gradients with respect to per-spring Ks and Kd, the initial velocities and a
constant per-vertex external force, compared along 32 random joint directions (eps 1e-4
relative).  The bar: the relative error of the vector of directional derivatives,
||ad - fd|| / ||fd||, at most 1e-3.

The cloth moves at most 1e-3 in 200 steps from rest and the loss residual is about 1.7e-6
rms, below what FP32 positions near 5 resolve (about 4e-7 of rounding per coordinate), so
the taped forward runs in the displacement mode (start positions plus an FP32
displacement, elongations from FP64-rounded start constants) and the residual is formed in
FP64 from the returned displacement.

Also a command line for the full measurement (the figures in profiles/):

    python tests/test_gpu_gradcheck.py [--directions 32] [--procs N] [--steps 200] [--positions]
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
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(Path(__file__).resolve().parent))

DT = 1.0 / 60.0
REL_EPS = 1e-4
TOL = 1e-3


def build_case(cols: int, seed: int):
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


def gradcheck(cols=257, steps=200, every=20, directions=32, procs=None, seed=20261204, displacement=True):
    """The figures of one check (see the module docstring)."""
    import oracle

    oracle.build(reference=False)
    procs = procs or max(1, min(32, os.cpu_count() or 1))
    X, sp, sp_t, pins = build_case(cols, seed)
    V0 = np.zeros_like(X)
    ext = np.zeros_like(X)
    rng = np.random.default_rng(seed + 1)
    dirs, jobs = [], []
    for _ in range(directions):
        u = {"ks": rng.normal(size=len(sp)), "kd": rng.normal(size=len(sp)), "V0": rng.normal(size=X.shape),
             "ext": rng.normal(size=X.shape)}
        sp_p, v_p, e_p = perturb(sp, V0, ext, u, +1)
        sp_m, v_m, e_m = perturb(sp, V0, ext, u, -1)
        dirs.append({"ks": sp_p["ks"].astype(np.float64) - sp_m["ks"], "kd": sp_p["kd"].astype(np.float64) - sp_m["kd"],
                     "V0": v_p.astype(np.float64) - v_m, "ext": e_p.astype(np.float64) - e_m})
        jobs.append((sp_p, v_p, e_p))
        jobs.append((sp_m, v_m, e_m))
    with mp.get_context("spawn").Pool(procs) as pool:
        tgt = pool.apply_async(fp64_final, (sp_t, X, V0, ext, pins, steps))
        ref = pool.apply_async(fp64_final, (sp, X, V0, ext, pins, steps))
        target = tgt.get()
        t0 = time.perf_counter()
        pending = pool.map_async(_loss_job, [(s_, X, v_, e_, pins, steps, target) for s_, v_, e_ in jobs])

        from opencloth_gb300 import ClothDesc, ClothSolver

        desc = ClothDesc(n_vertices=len(X), springs=sp, pinned=pins, cg_max_iter=500, cg_tol=1e-6)
        with ClothSolver(desc) as s:
            s.set_tape_mode(displacement)
            s.set_ext_force(ext)
            s.set_state(X, V0, np.zeros_like(X))
            t_g = time.perf_counter()
            s.tape_forward(DT, steps, every)
            if displacement:
                XT = X.astype(np.float64) + s.tape_displacement().astype(np.float64)
            else:
                XT = s.get_state()[0].astype(np.float64)
            gX = 2.0 * (XT - target) / len(X)
            g = s.tape_backward(gX)
            t_grad = time.perf_counter() - t_g
        losses = pending.get()
        t_fd = time.perf_counter() - t0
        X64 = ref.get()
    fd = np.array([losses[2 * k] - losses[2 * k + 1] for k in range(directions)])
    key = {"ks": "dKs", "kd": "dKd", "V0": "dV0", "ext": "dext"}
    ad = np.array([sum(float(np.sum(g[key[n]].astype(np.float64).reshape(d[n].shape) * d[n])) for n in key)
                   for d in dirs])
    per = np.abs(ad - fd) / np.maximum(np.abs(fd), 1e-300)
    return {
        "config": f"{cols}x{cols} cloth, {steps} steps, checkpoint every {every}",
        "tape_mode": "displacement" if displacement else "positions",
        "directions": directions, "rel_eps": REL_EPS,
        "rel_err_vector": float(np.linalg.norm(ad - fd) / np.linalg.norm(fd)),
        "rel_err_per_direction_median": float(np.median(per)), "rel_err_per_direction_max": float(per.max()),
        "loss_residual_rms": float(np.sqrt(np.mean((X64 - target) ** 2))),
        "final_state_err_rms": float(np.sqrt(np.mean((XT - X64) ** 2))),
        "gpu_gradient_s": t_grad, "fd_s": t_fd, "fd_procs": procs,
    }


@pytest.mark.gpu
def test_config4_gradients_match_fp64_central_differences():
    out = gradcheck()
    print(json.dumps(out))
    assert out["final_state_err_rms"] <= 1e-3 * out["loss_residual_rms"], out
    assert out["rel_err_vector"] <= TOL, out


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--cols", type=int, default=257)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--every", type=int, default=20)
    ap.add_argument("--directions", type=int, default=32)
    ap.add_argument("--procs", type=int, default=0)
    ap.add_argument("--seed", type=int, default=20261204)
    ap.add_argument("--positions", action="store_true", help="tape in FP32 positions (the step itself)")
    a = ap.parse_args()
    out = gradcheck(a.cols, a.steps, a.every, a.directions, a.procs or None, a.seed, not a.positions)
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
