"""Shared test inputs: golden fixtures from the reference and seeded cloths."""
from __future__ import annotations

from pathlib import Path

import numpy as np

import oracle
from opencloth_gb300 import SPRING_DTYPE, ClothDesc, grid_cloth

GOLDEN = Path(__file__).resolve().parent / "golden"
GOLDEN_CASES = ("grid21_ref", "random7x5_ref", "clamp9_ref", "stepphysics21_ref")


def golden(name: str) -> dict:
    d = dict(np.load(GOLDEN / f"{name}.npz"))
    d["springs"] = d["springs"].reshape(-1).view(SPRING_DTYPE).copy()
    for k in ("cols", "rows", "i_max"):
        d[k] = int(d[k])
    d["dt"] = float(d["dt"])
    d["eps"] = float(d["eps"])
    d["passes"] = int(d.get("passes", 0))
    return d


def rel(a, b) -> float:
    """max |a - b| / max |b| (b the reference)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def rel_disp(a, b, x0) -> float:
    """max |a - b| / max |b - x0|: the error relative to the motion from x0 (b the
    reference), which a solver that did not move the cloth fails."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b - np.asarray(x0, np.float64)).max(), 1e-30))


def desc_for(g: dict, **kw) -> ClothDesc:
    """Library description of a golden case; pins = the reference's {0, numX}."""
    return ClothDesc(n_vertices=g["cols"] * g["rows"], springs=g["springs"],
                     pinned=np.array([0, g["cols"] - 1], np.int32), gravity=tuple(g["gravity"]),
                     cg_max_iter=g["i_max"], cg_tol=g["eps"], passes=g["passes"], ellipsoid=g["ellipsoid"],
                     ellipsoid_inv=g["ellipsoid_inv"], **kw)


def oracle_for(g: dict, explicit_pins: bool = False) -> oracle.Cloth:
    return oracle.Cloth(g["cols"] * g["rows"], g["springs"], num_x=g["cols"] - 1,
                        pinned=[0, g["cols"] - 1] if explicit_pins else None, gravity=tuple(g["gravity"]),
                        i_max=g["i_max"], eps=g["eps"], passes=g["passes"], ellipsoid=g["ellipsoid"],
                        ellipsoid_inv=g["ellipsoid_inv"], ellipsoid64=g["ellipsoid64"],
                        ellipsoid_inv64=g["ellipsoid_inv64"])


def seeded_cloth(cols: int, rows: int, seed: int, i_max: int = 200, eps: float = 1e-5, jitter: float = 1e-3,
                 random_params: bool = True, velocity: float = 0.0):
    """A jittered grid with per-type log-uniform Ks and uniform Kd (the batch
    configuration's distributions).  Returns (desc, oracle cloth, X, V)."""
    rng = np.random.default_rng(seed)
    if random_params:
        ks = np.exp(rng.uniform(np.log(10.0), np.log(500.0), 3)).astype(np.float32)
        kd = rng.uniform(-0.5, -0.05, 3).astype(np.float32)
    else:
        ks = np.array([50.75, 50.75, 50.95], np.float32)
        kd = np.array([-0.25, -0.25, -0.25], np.float32)
    X, sp = grid_cloth(cols, rows, ks=tuple(ks), kd=tuple(kd), jitter=jitter, seed=seed)
    V = np.zeros_like(X)
    if velocity:
        V = rng.normal(0.0, velocity, X.shape).astype(np.float32)
        V[[0, cols - 1]] = 0.0
    pins = np.array([0, cols - 1], np.int32)
    desc = ClothDesc(n_vertices=cols * rows, springs=sp, pinned=pins, cg_max_iter=i_max, cg_tol=eps)
    ocl = oracle.Cloth(cols * rows, sp, pinned=pins, i_max=i_max, eps=eps)
    return desc, ocl, X, V


FEM_CASES = ("m0", "m30", "m120", "big10")


def fem_golden(tag: str):
    """A system the FEM demo's CG received (tests/golden/fem_cg_ref.npz), with the
    reference CG's FP32 and FP64 results: (system, V32, r32, V64, r64)."""
    d = np.load(GOLDEN / "fem_cg_ref.npz")
    sys_ = oracle.BsrSystem.from_bytes(d[f"{tag}_system"].tobytes())
    return sys_, d[f"{tag}_V32"], d[f"{tag}_r32"], d[f"{tag}_V64"], d[f"{tag}_r64"]
