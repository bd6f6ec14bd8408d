"""Run a few solves of the FEM demo's block-sparse CG, for profilers and launch-shape sweeps.

    python -m opencloth_gb300.profile_fem --dims 160 48 48 --solves 3 [--batch 1] [--no-graph]

Prints one JSON line: ms per solve (CUDA events on the solver's stream) and, unless
--no-profile, the per-kernel average durations of an un-graphed solve.
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from .fem import BsrSolver, fem_system


def main() -> None:
    import torch

    ap = argparse.ArgumentParser()
    ap.add_argument("--dims", type=int, nargs=3, default=[160, 48, 48])
    ap.add_argument("--batch", type=int, default=1, help="copies of the system in one handle")
    ap.add_argument("--solves", type=int, default=3)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--no-profile", action="store_true")
    a = ap.parse_args()
    x, y, z = a.dims
    n = (x + 1) * (y + 1) * (z + 1)
    g = fem_system(x, y, z, V=np.random.default_rng(a.seed).normal(0.0, 0.1, (n, 3)))
    systems = [g] * a.batch
    stream = torch.cuda.Stream()
    s = BsrSolver(systems, stream=stream.cuda_stream, use_graph=not a.no_graph)
    s.set_system(np.concatenate([q["blocks"] for q in systems]), np.concatenate([q["b"] for q in systems]),
                 np.concatenate([q["V"] for q in systems]))
    s.solve()
    s.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(a.solves):
        s.solve()
    e1.record(stream)
    e1.synchronize()
    out = {"rows": s.n_rows, "blocks": s.nnzb, "systems": s.n_systems, "graph": not a.no_graph,
           "ms_per_solve": e0.elapsed_time(e1) / max(a.solves, 1)}
    if not a.no_profile:
        prof = s.profile(1)
        out["kernels_us"] = {k: 1e3 * v["ms_total"] / max(v["launches"], 1) for k, v in prof.items()}
    print(json.dumps(out), flush=True)
    s.close()


if __name__ == "__main__":
    main()
