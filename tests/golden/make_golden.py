"""Generate the golden fixtures in this directory from the reference itself.

Runs the reference's own implicit step and the FEM demo's CG compiled headless
(oracle/build_ref.sh -> oracle/_ref/ref_step_f32/_f64 and fem_step_f32/_f64) on seeded
inputs and stores inputs and outputs as .npz, so hosts without the reference tree (the
GPU host) can check against them.  Needs the reference tree; run from the repository root:

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from opencloth_gb300 import grid_cloth  # noqa: E402

OUT = Path(__file__).resolve().parent


def save_case(name, cols, rows, X, V, dV, springs, dt, i_max, eps, gravity, snaps32, snaps64, passes=0):
    E, Einv = oracle.ref_ellipsoid()
    E64, Einv64 = oracle.ref_ellipsoid(fp64=True)
    cl = oracle.Cloth(cols * rows, springs, num_x=cols - 1, gravity=gravity, i_max=i_max, eps=eps, passes=passes,
                      ellipsoid=E, ellipsoid_inv=Einv, ellipsoid64=E64, ellipsoid_inv64=Einv64)
    r32 = oracle.ref_run(cl, cols - 1, rows - 1, X, V, dV, dt=dt, snaps=snaps32)
    r64 = oracle.ref_run(cl, cols - 1, rows - 1, X, V, dV, dt=dt, snaps=snaps64, fp64=True)
    out = dict(cols=cols, rows=rows, X0=X, V0=V, dV0=dV, springs=springs.view(np.uint8).reshape(len(springs), -1),
               dt=np.float32(dt), i_max=i_max, eps=np.float32(eps), gravity=np.asarray(gravity, np.float32),
               snaps32=np.asarray(snaps32, np.int32), snaps64=np.asarray(snaps64, np.int32), passes=passes,
               ellipsoid=E, ellipsoid_inv=Einv, ellipsoid64=E64, ellipsoid_inv64=Einv64)
    for s in snaps32:
        out[f"X32_{s}"], out[f"V32_{s}"], out[f"dV32_{s}"] = r32[s]
    for s in snaps64:
        out[f"X64_{s}"], out[f"V64_{s}"], out[f"dV64_{s}"] = r64[s]
    np.savez_compressed(OUT / f"{name}.npz", **out)
    print("wrote", name)


def main():
    oracle.build()
    if not oracle.ref_available():
        raise SystemExit("the reference build (oracle/_ref) is not available here")
    g = (0.0, -0.00981, 0.0)

    # 21 x 21 cloth, Ks 50.75/50.75/50.95, Kd -0.25, dt 1/60, i_max 10, EPS 1e-3.
    X, sp = grid_cloth(21, 21, ks=(50.75, 50.75, 50.95), kd=(-0.25, -0.25, -0.25))
    save_case("grid21_ref", 21, 21, X, np.zeros_like(X), np.zeros_like(X), sp, 1.0 / 60.0, 10, 1e-3, g,
              (1, 10, 600), (1, 600))

    # Small irregular case: per-spring Ks/Kd, jitter, non-zero V and warm start off the pins.
    rng = np.random.default_rng(20261203)
    cols, rows = 7, 5
    X, sp = grid_cloth(cols, rows, jitter=0.05, seed=7)
    sp["ks"] = np.exp(rng.uniform(np.log(10.0), np.log(500.0), len(sp))).astype(np.float32)
    sp["kd"] = rng.uniform(-0.5, -0.05, len(sp)).astype(np.float32)
    V = rng.normal(0, 0.05, X.shape).astype(np.float32)
    dV = rng.normal(0, 1e-3, X.shape).astype(np.float32)
    for p in (0, cols - 1):
        V[p] = 0
        dV[p] = 0
    save_case("random7x5_ref", cols, rows, X, V, dV, sp, 1.0 / 60.0, 50, 1e-5, g, (1, 25), (1, 25))

    # Ground clamp: a cloth hanging just above y = 0 under strong gravity.
    cols, rows = 9, 9
    X, sp = grid_cloth(cols, rows, size=1.0, ks=(50.75, 50.75, 50.95), kd=(-0.25, -0.25, -0.25))
    X[:, 1] -= 1.95
    save_case("clamp9_ref", cols, rows, X, np.zeros_like(X), np.zeros_like(X), sp, 1.0 / 60.0, 30, 1e-4,
              (0.0, -9.81, 0.0), (1, 40), (1, 40))

    # The whole StepPhysics (IMP:873-880): the ellipsoid of InitGL sits at y = 2 and cuts
    # the lower rows of the cloth, and soft springs let Provot's correction act.
    cols, rows = 21, 21
    X, sp = grid_cloth(cols, rows, ks=(0.75, 0.75, 0.95), kd=(-0.25, -0.25, -0.25))
    save_case("stepphysics21_ref", cols, rows, X, np.zeros_like(X), np.zeros_like(X), sp, 5.0 / 60.0, 10, 1e-3, g,
              (1, 10, 100), (1,), passes=3)

    # The FEM demo's block-sparse CG (FEM:837-922) on the systems the demo itself builds:
    # its default mesh after 0, 30 and 120 steps and a larger mesh after 10 steps, with
    # the reference CG's FP32 result and the FP64 build's result on the same system.
    fem = {}
    for tag, steps, dims in (("m0", 0, (10, 3, 3)), ("m30", 30, (10, 3, 3)), ("m120", 120, (10, 3, 3)),
                             ("big10", 10, (14, 4, 4))):
        sys_, V32, r32 = oracle.fem_ref_system(steps, dims)
        V64, r64 = oracle.fem_ref_solve(sys_, fp64=True)
        fem[f"{tag}_dims"] = np.array(dims, np.int32)
        fem[f"{tag}_steps"] = np.int32(steps)
        fem[f"{tag}_system"] = np.frombuffer(sys_.to_bytes(), np.uint8)
        fem[f"{tag}_V32"], fem[f"{tag}_r32"] = V32, r32
        fem[f"{tag}_V64"], fem[f"{tag}_r64"] = V64, r64
    np.savez_compressed(OUT / "fem_cg_ref.npz", **fem)
    print("wrote fem_cg_ref")

    # InitGL's own topology for a few grid sizes.
    topo = {}
    for nx, ny in ((20, 20), (2, 2), (5, 9), (9, 3)):
        _, spr = oracle.ref_topology(nx, ny)
        topo[f"p1_{nx}_{ny}"] = spr["p1"]
        topo[f"p2_{nx}_{ny}"] = spr["p2"]
        topo[f"type_{nx}_{ny}"] = spr["type"]
    np.savez_compressed(OUT / "topology_ref.npz", **topo)
    print("wrote topology_ref")


if __name__ == "__main__":
    main()
