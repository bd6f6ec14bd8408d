"""The oracle pinned to the reference (CPU only).

The C restatement (oracle/oc_oracle.c) must reproduce the reference's own step bit for
bit: against the golden fixtures made by the reference build (everywhere), and against
the reference build itself on fresh seeded inputs (where the reference tree exists).
"""
import numpy as np
import pytest

import oracle
from cases import GOLDEN, GOLDEN_CASES, golden, oracle_for, rel
from opencloth_gb300 import grid_cloth


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_port_fp32_matches_reference_golden(name):
    g = golden(name)
    cl = oracle_for(g)
    for s in g["snaps32"]:
        X, V, dV, _, _ = oracle.port_step(cl, g["X0"], g["V0"], g["dV0"], dt=g["dt"], n_steps=int(s))
        assert np.array_equal(X, g[f"X32_{s}"]), (name, s)
        assert np.array_equal(V, g[f"V32_{s}"]), (name, s)
        assert np.array_equal(dV, g[f"dV32_{s}"]), (name, s)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_port_fp64_matches_reference_golden(name):
    g = golden(name)
    cl = oracle_for(g)
    for s in g["snaps64"]:
        X, V, dV, _, _ = oracle.port_step(cl, g["X0"], g["V0"], g["dV0"], dt=g["dt"], n_steps=int(s), fp64=True)
        assert np.array_equal(X, g[f"X64_{s}"]), (name, s)
        assert np.array_equal(V, g[f"V64_{s}"]), (name, s)


def test_golden_clamp_case_exercises_the_clamp():
    g = golden("clamp9_ref")
    assert (g["X32_40"][:, 1] == 0.0).sum() > 10


def test_explicit_pins_with_filter_equal_reference_pins():
    """Pins given as a list plus the CG filter reproduce the reference's hard-coded
    pins {0, numX} exactly when the pinned vertices start at rest."""
    g = golden("grid21_ref")
    ref = oracle_for(g)
    ours = oracle_for(g, explicit_pins=True)
    a = oracle.port_step(ref, g["X0"], g["V0"], g["dV0"], dt=g["dt"], n_steps=200)
    b = oracle.port_step(ours, g["X0"], g["V0"], g["dV0"], dt=g["dt"], n_steps=200, filter_pinned=True)
    for x, y in zip(a[:3], b[:3]):
        assert np.array_equal(x, y)


def test_fp64_dot_accumulation_stays_close_to_reference():
    """The GPU's FP64 dot accumulation perturbs the FP32 reference far below the
    parity tolerance (CPU proxy of the GPU arithmetic)."""
    g = golden("grid21_ref")
    cl = oracle_for(g, explicit_pins=True)
    X, V, _, _, _ = oracle.port_step(cl, g["X0"], g["V0"], g["dV0"], dt=g["dt"], n_steps=600, dot_fp64=True,
                                     filter_pinned=True)
    assert rel(X, g["X32_600"]) < 1e-9
    assert rel(V, g["V32_600"]) < 1e-6


def test_topology_golden_matches_grid_builder():
    t = dict(np.load(GOLDEN / "topology_ref.npz"))
    for nx, ny in ((20, 20), (2, 2), (5, 9), (9, 3)):
        _, sp = grid_cloth(nx + 1, ny + 1)
        assert np.array_equal(sp["p1"], t[f"p1_{nx}_{ny}"])
        assert np.array_equal(sp["p2"], t[f"p2_{nx}_{ny}"])
        assert np.array_equal(sp["type"], t[f"type_{nx}_{ny}"])


needs_ref = pytest.mark.skipif(not oracle.ref_available(), reason="reference tree not built here")


@needs_ref
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_port_matches_reference_build_on_seeded_inputs(seed):
    rng = np.random.default_rng(seed)
    cols, rows = int(rng.integers(3, 12)), int(rng.integers(3, 12))
    X, sp = grid_cloth(cols, rows, jitter=0.02, seed=seed)
    sp["ks"] = np.exp(rng.uniform(np.log(10), np.log(500), len(sp))).astype(np.float32)
    sp["kd"] = rng.uniform(-0.5, -0.05, len(sp)).astype(np.float32)
    V = rng.normal(0, 0.02, X.shape).astype(np.float32)
    V[[0, cols - 1]] = 0
    cl = oracle.Cloth(cols * rows, sp, num_x=cols - 1, i_max=int(rng.integers(1, 40)), eps=1e-4)
    ref = oracle.ref_run(cl, cols - 1, rows - 1, X, V, snaps=(1, 7))
    ref64 = oracle.ref_run(cl, cols - 1, rows - 1, X, V, snaps=(7,), fp64=True)
    for s in (1, 7):
        Xp, Vp, dVp, _, _ = oracle.port_step(cl, X, V, n_steps=s)
        assert np.array_equal(Xp, ref[s][0]) and np.array_equal(Vp, ref[s][1]) and np.array_equal(dVp, ref[s][2])
    Xp, Vp, _, _, _ = oracle.port_step(cl, X, V, n_steps=7, fp64=True)
    assert np.array_equal(Xp, ref64[7][0]) and np.array_equal(Vp, ref64[7][1])


@needs_ref
def test_grid_builder_matches_reference_initgl_live():
    for nx, ny in ((3, 7), (12, 4)):
        _, spr = oracle.ref_topology(nx, ny)
        _, sp = grid_cloth(nx + 1, ny + 1)
        assert np.array_equal(sp["p1"], spr["p1"]) and np.array_equal(sp["p2"], spr["p2"])


def test_oracle_grid_builder_matches_topology_golden():
    """The oracle's own lattice builder (used by the benchmark's CPU arms) reproduces
    InitGL's spring order from the reference build."""
    t = dict(np.load(GOLDEN / "topology_ref.npz"))
    for nx, ny in ((20, 20), (2, 2), (5, 9), (9, 3)):
        _, sp = oracle.grid_cloth(nx + 1, ny + 1)
        assert np.array_equal(sp["p1"], t[f"p1_{nx}_{ny}"])
        assert np.array_equal(sp["p2"], t[f"p2_{nx}_{ny}"])
        assert np.array_equal(sp["type"], t[f"type_{nx}_{ny}"])


@pytest.mark.parametrize("cols,rows,jitter,seed", [(21, 21, 0.0, 0), (33, 17, 1e-3, 7), (129, 64, 2e-2, 20261203),
                                                   (8, 8, 1e-3, 123456789)])
def test_oracle_grid_builder_matches_library_builder(cols, rows, jitter, seed):
    """Same arguments, same bits: positions (jitter included), spring records and rest
    lengths, so the benchmark's CPU arms step exactly the GPU arm's inputs."""
    ks, kd = (50.75, 49.5, 50.95), (-0.25, -0.3, -0.2)
    Xo, so = oracle.grid_cloth(cols, rows, ks=ks, kd=kd, jitter=jitter, seed=seed)
    Xl, sl = grid_cloth(cols, rows, ks=ks, kd=kd, jitter=jitter, seed=seed)
    assert np.array_equal(Xo.view(np.uint32), Xl.view(np.uint32))
    assert so.tobytes() == sl.tobytes()
