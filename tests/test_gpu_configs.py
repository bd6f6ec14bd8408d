"""The benchmark configurations at their own size and length against the oracle.

* The 1M-vertex cloth (1025 x 1025, Ks 50.75/50.75/50.95, Kd -0.25, jitter 1e-3 of the
  spacing, CG up to 200 iterations to 1e-5), 600 steps, against the FP64 method: the
  restatement in FP64 (bit-identical to the reference built in FP64) stepped on this
  container, kept as a seeded 4096-vertex sample with full-array norms
  (tests/golden/grid1025_fp64.npz, made by make_grid1025_fp64.py).  Bounds: positions
  within 1e-4 relative (max-norm over max-norm), and within 1e-3 of the motion (the
  max-norm error over the largest displacement from the initial positions).
* A seeded 64-cloth subset of the 4096-cloth batch that spans its sizes (sides 8 ... 128,
  per-type Ks log-uniform in [10, 500], Kd uniform in [-0.5, -0.05]), 300 steps in one
  handle (the resident executor), each cloth against the FP32 restatement run with the
  GPU's arithmetic (FP64 dots, pin filter) and against the FP64 restatement.  Bounds per
  cloth: within 1e-5 relative and 1e-3 of the motion of the FP32 restatement; within
  1e-4 relative of the FP64 one.
"""
import multiprocessing as mp
import zlib

import numpy as np
import pytest

from cases import GOLDEN, rel, rel_disp
from opencloth_gb300 import ClothDesc, ClothSolver, grid_cloth

pytestmark = pytest.mark.gpu
DT = 1.0 / 60.0

TOL_FP64_X = 1e-4
TOL_FP64_MOTION = 1e-3
TOL_PORT_X, TOL_PORT_MOTION = 1e-5, 1e-3


def test_grid1025_600_steps_against_fp64():
    g = np.load(GOLDEN / "grid1025_fp64.npz")
    cols = int(g["cols"])
    X0, sp = grid_cloth(cols, cols, ks=(50.75, 50.75, 50.95), kd=(-0.25, -0.25, -0.25), jitter=1e-3,
                        seed=int(g["seed"]))
    assert zlib.crc32(X0.tobytes()) == int(g["x0_crc32"]), "not the input the fixture was made from"
    desc = ClothDesc(n_vertices=cols * cols, springs=sp, pinned=np.array([0, cols - 1], np.int32), cg_max_iter=200,
                     cg_tol=1e-5)
    idx = g["idx"]
    X0d = X0.astype(np.float64)
    with ClothSolver(desc) as s:
        s.set_state(X0, np.zeros_like(X0), np.zeros_like(X0))
        s.step(DT, 1)
        X1, V1, _ = s.get_state()
        s.step(DT, int(g["steps"]) - 1)
        XT, VT, _ = s.get_state()
        _, rr, fl = s.stats()
    assert fl[0] == 0 and rr[0] <= 1e-5
    # Positions, relative to the full array's norm.
    assert np.abs(XT[idx] - g["X600"]).max() / float(g["X600_inf"]) <= TOL_FP64_X
    assert np.abs(X1[idx] - g["X1"]).max() / float(g["X600_inf"]) <= TOL_FP64_X
    # The motion after 600 steps (the first step's displacement, about 5e-8, is below
    # the FP32 resolution of positions near 5).
    motion = np.abs(XT[idx] - g["X600"]).max() / float(g["disp600_inf"])
    assert motion <= TOL_FP64_MOTION, motion
    assert np.abs(np.abs(XT - X0d).max() - float(g["disp600_inf"])) <= TOL_FP64_MOTION * float(g["disp600_inf"])
    assert np.abs(VT[idx] - g["V600"]).max() / float(g["V600_inf"]) <= 1e-2


def batch_subset(count: int = 64, seed: int = 20261203, total: int = 4096):
    """Cloths of the 4096-cloth batch (same generator and draws as bench.batch4096): a
    seeded choice of `count` that spans the size range (evenly spaced in size order)."""
    rng = np.random.default_rng(seed)
    sides = rng.integers(8, 129, total)
    order = np.argsort(sides, kind="stable")
    pick = set(order[np.linspace(0, total - 1, count).astype(int)].tolist())
    out = []
    for k, n in enumerate(sides):
        n = int(n)
        ks = np.exp(rng.uniform(np.log(10.0), np.log(500.0), 3))
        kd = rng.uniform(-0.5, -0.05, 3)
        if k in pick:
            X, sp = grid_cloth(n, n, ks=tuple(ks), kd=tuple(kd), jitter=1e-3, seed=seed * 100003 + k)
            out.append((n, X, sp))
    return out


def _port_job(args):
    n, X, sp, steps, fp64 = args
    import oracle as o

    cl = o.Cloth(n * n, sp, pinned=np.array([0, n - 1], np.int32), i_max=200, eps=1e-5)
    Xo, Vo, _, _, _ = o.port_step(cl, X, np.zeros_like(X), n_steps=steps, fp64=fp64, dot_fp64=True,
                                  filter_pinned=True)
    return Xo, Vo


def test_batch_subset_300_steps_against_port():
    steps = 300
    cloths = batch_subset()
    sides = [n for n, _, _ in cloths]
    assert min(sides) <= 9 and max(sides) >= 127
    jobs = [(n, X, sp, steps, fp64) for fp64 in (False, True) for n, X, sp in cloths]
    with mp.get_context("spawn").Pool(min(16, mp.cpu_count())) as pool:
        pending = pool.map_async(_port_job, jobs)
        descs = [ClothDesc(n_vertices=n * n, springs=sp, pinned=np.array([0, n - 1], np.int32), cg_max_iter=200,
                           cg_tol=1e-5) for n, _, sp in cloths]
        X0 = np.concatenate([X for _, X, _ in cloths])
        with ClothSolver(descs) as s:
            s.set_state(X0, np.zeros_like(X0), np.zeros_like(X0))
            s.step(DT, steps)
            XT, VT, _ = s.get_state()
            _, rr, fl = s.stats()
            offs = s.offsets
        ports = pending.get(timeout=900)
    assert not fl.any() and (rr <= 1e-5).all()
    m = len(cloths)
    worst = {"port_x": 0.0, "port_motion": 0.0, "fp64_x": 0.0}
    for k, (n, X, _) in enumerate(cloths):
        sl = slice(offs[k], offs[k + 1])
        Xp, _ = ports[k]
        X64, _ = ports[m + k]
        worst["port_x"] = max(worst["port_x"], rel(XT[sl], Xp))
        worst["port_motion"] = max(worst["port_motion"], rel_disp(XT[sl], Xp, X))
        worst["fp64_x"] = max(worst["fp64_x"], rel(XT[sl], X64))
    assert worst["port_x"] <= TOL_PORT_X, worst
    assert worst["port_motion"] <= TOL_PORT_MOTION, worst
    assert worst["fp64_x"] <= TOL_FP64_X, worst
