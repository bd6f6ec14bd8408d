"""Shared inputs for the adjoint tests: a seeded cloth with per-spring Ks/Kd, initial
velocity and external force, a target from a run with perturbed stiffness, and the FP64
reference loss (oracle port with a tight CG tolerance)."""
from __future__ import annotations

import numpy as np

import oracle
from opencloth_gb300 import grid_cloth

DT = 1.0 / 60.0


def make_case(cols=10, rows=8, steps=12, seed=0, ks_range=(10.0, 100.0), v_sigma=0.02):
    rng = np.random.default_rng(seed)
    X, sp = grid_cloth(cols, rows, jitter=0.02, seed=seed + 1)
    sp["ks"] = np.exp(rng.uniform(np.log(ks_range[0]), np.log(ks_range[1]), len(sp))).astype(np.float32)
    sp["kd"] = rng.uniform(-0.5, -0.05, len(sp)).astype(np.float32)
    V0 = rng.normal(0, v_sigma, X.shape).astype(np.float32)
    V0[[0, cols - 1]] = 0.0
    ext = rng.normal(0, 0.005, X.shape).astype(np.float32)
    pins = np.array([0, cols - 1], np.int32)
    # Target: the final positions of a run whose Ks carry log-normal(0, 0.1^2) factors.
    sp_t = sp.copy()
    sp_t["ks"] = (sp["ks"] * np.exp(rng.normal(0.0, 0.1, len(sp)))).astype(np.float32)
    target, _ = fp64_final(sp_t, X, V0, ext, pins, steps)
    return dict(cols=cols, rows=rows, steps=steps, X=X, springs=sp, V0=V0, ext=ext, pins=pins, target=target,
                rng=rng)


def fp64_final(springs, X, V0, ext, pins, steps, eps=1e-10):
    cl = oracle.Cloth(len(X), springs, pinned=pins, i_max=1000, eps=eps, ext_force=ext)
    Xo, Vo, _, _, _ = oracle.port_step(cl, X, V0, n_steps=steps, fp64=True, dot_fp64=True, filter_pinned=True)
    return Xo, Vo


def loss_fp64(case, springs=None, V0=None, ext=None):
    sp = case["springs"] if springs is None else springs
    Xo, _ = fp64_final(sp, case["X"], case["V0"] if V0 is None else V0, case["ext"] if ext is None else ext,
                       case["pins"], case["steps"])
    return float(np.mean(np.sum((Xo - case["target"]) ** 2, axis=1)))


def fd_direction(case, name, u, rel_eps=1e-4):
    """FP64 central difference of the loss along u for parameter `name` (ks, kd, V0,
    ext); returns (difference, the exact float32 perturbation applied)."""
    if name in ("ks", "kd"):
        base = case["springs"][name].astype(np.float64)
        spp, spm = case["springs"].copy(), case["springs"].copy()
        spp[name] = (base * (1 + rel_eps * u)).astype(np.float32)
        spm[name] = (base * (1 - rel_eps * u)).astype(np.float32)
        d = spp[name].astype(np.float64) - spm[name].astype(np.float64)
        return loss_fp64(case, springs=spp) - loss_fp64(case, springs=spm), d
    base = case[name].astype(np.float64)
    scale = rel_eps * max(np.abs(base).max(), 1e-3)
    p = (base + scale * u).astype(np.float32)
    m = (base - scale * u).astype(np.float32)
    d = p.astype(np.float64) - m.astype(np.float64)
    kw = {name: p}
    lp = loss_fp64(case, **kw)
    kw = {name: m}
    return lp - loss_fp64(case, **kw), d


def fd_joint(case, u, rel_eps=1e-4):
    """FP64 central difference along a joint direction u = (ks, kd, V0, ext); returns
    (difference, the exact float32 perturbations applied, keyed like u)."""
    sp_p, sp_m = case["springs"].copy(), case["springs"].copy()
    d = {}
    for name in ("ks", "kd"):
        base = case["springs"][name].astype(np.float64)
        sp_p[name] = (base * (1 + rel_eps * u[name])).astype(np.float32)
        sp_m[name] = (base * (1 - rel_eps * u[name])).astype(np.float32)
        d[name] = sp_p[name].astype(np.float64) - sp_m[name].astype(np.float64)
    vals = {}
    for name in ("V0", "ext"):
        base = case[name].astype(np.float64)
        scale = rel_eps * max(np.abs(base).max(), 1e-3)
        p = (base + scale * u[name]).astype(np.float32)
        m = (base - scale * u[name]).astype(np.float32)
        d[name] = p.astype(np.float64) - m.astype(np.float64)
        vals[name] = (p, m)
    lp = loss_fp64(case, springs=sp_p, V0=vals["V0"][0], ext=vals["ext"][0])
    lm = loss_fp64(case, springs=sp_m, V0=vals["V0"][1], ext=vals["ext"][1])
    return lp - lm, d
