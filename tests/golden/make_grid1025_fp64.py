"""Generate grid1025_fp64.npz: the 1M-vertex configuration stepped 600 times by the FP64
restatement of the reference step (oracle/oc_oracle.c, bit-identical to the reference built
in FP64; tests/test_oracle.py pins it).

Configuration: 1025 x 1025 cloth, 4.0 x 4.0, Ks 50.75/50.75/50.95, Kd -0.25, mass 1,
gravity (0, -0.00981, 0), dt 1/60, top corners pinned, N(0, (1e-3 spacing)^2) jitter
(seed 20261203), CG up to 200 iterations to 1e-5 with the pin filter.  The full state is
25 MB per snapshot, so the fixture keeps a seeded sample of 4096 vertices (the corners and
the centre included) after 1 and 600 steps, the full-array infinity norms the tests divide
by, and a CRC-32 of the input positions so a test can check it steps the same input.
Takes about five minutes on one core:

    python tests/golden/make_grid1025_fp64.py
"""
from __future__ import annotations

import sys
import zlib
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402

OUT = Path(__file__).resolve().parent / "grid1025_fp64.npz"
COLS, SEED, STEPS, SAMPLE = 1025, 20261203, 600, 4096


def main() -> None:
    oracle.build(reference=False)
    X0, sp = oracle.grid_cloth(COLS, COLS, ks=(50.75, 50.75, 50.95), kd=(-0.25, -0.25, -0.25), jitter=1e-3, seed=SEED)
    n = len(X0)
    pins = np.array([0, COLS - 1], np.int32)
    cl = oracle.Cloth(n, sp, pinned=pins, i_max=200, eps=1e-5)
    V0 = np.zeros_like(X0)
    X1, V1, dV1, _, _ = oracle.port_step(cl, X0, V0, n_steps=1, fp64=True, filter_pinned=True)
    XT, VT, _, itT, _ = oracle.port_step(cl, X1, V1, dV1, n_steps=STEPS - 1, fp64=True, filter_pinned=True)
    rng = np.random.default_rng(SEED)
    fixed = [0, COLS - 1, n - COLS, n - 1, (COLS // 2) * COLS + COLS // 2]
    idx = np.unique(np.concatenate([fixed, rng.choice(n, SAMPLE - len(fixed), replace=False)])).astype(np.int32)
    X0d = X0.astype(np.float64)
    np.savez_compressed(
        OUT, cols=COLS, seed=SEED, steps=STEPS, idx=idx, x0_crc32=np.uint32(zlib.crc32(X0.tobytes())),
        X1=X1[idx], V1=V1[idx], X600=XT[idx], V600=VT[idx],
        disp1_inf=np.abs(X1 - X0d).max(), disp600_inf=np.abs(XT - X0d).max(), X600_inf=np.abs(XT).max(),
        V1_inf=np.abs(V1).max(), V600_inf=np.abs(VT).max(), iters_last=np.int32(itT[-1]))
    print(f"wrote {OUT.name}: {len(idx)} sampled vertices, max displacement {np.abs(XT - X0d).max():.4g}, "
          f"last step {int(itT[-1])} CG iterations")


if __name__ == "__main__":
    main()
