"""The stencil assembly of grid cloths (k_assemble_grid) against the general incidence
gather (k_assemble): the same expressions in the same order, so the same bits.

Grid cloths of the reference's lattice are detected at create time (oc_describe_instances
reports them); OC_STENCIL=0 at create time keeps every cloth on the incidence gather.
"""
import os

import numpy as np
import pytest

from cases import desc_for, golden
from opencloth_gb300 import ClothDesc, ClothSolver, describe, grid_cloth

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0


def same_bits(a, b) -> bool:
    return np.array_equal(np.asarray(a).view(np.uint32), np.asarray(b).view(np.uint32))


def run(descs, X, V, steps, stencil: bool, dt: float = DT, **kw):
    old = os.environ.get("OC_STENCIL")
    os.environ["OC_STENCIL"] = "1" if stencil else "0"
    try:
        s = ClothSolver(descs, **kw)
    finally:
        if old is None:
            del os.environ["OC_STENCIL"]
        else:
            os.environ["OC_STENCIL"] = old
    with s:
        s.set_state(X, V)
        s.step(dt, steps)
        return s.get_state(), s.stats()


@pytest.mark.parametrize("name", ["grid21_ref", "clamp9_ref", "stepphysics21_ref"])
def test_golden_grids_same_bits(name):
    g = golden(name)
    d = desc_for(g)
    assert describe(d)[0] == (g["cols"], g["rows"])
    a, sa = run(d, g["X0"], g["V0"], 30, True, dt=g["dt"])
    b, sb = run(d, g["X0"], g["V0"], 30, False, dt=g["dt"])
    for x, y in zip(a, b):
        assert same_bits(x, y)
    assert np.array_equal(sa[0], sb[0])


@pytest.mark.parametrize("executor", ["streamed", "resident", "plain"])
def test_mixed_batch_same_bits(executor):
    """Exact-spacing grids (rest lengths in the slots), inexact ones (rest per incidence),
    a non-square grid, and a random-parameter cloth that stays on the incidence gather."""
    rng = np.random.default_rng(4)
    descs, Xs, Vs = [], [], []
    for cols, rows in ((17, 17), (23, 23), (9, 14), (64, 33), (7, 5)):
        X, sp = grid_cloth(cols, rows, ks=(50.75, 40.0, 30.0), kd=(-0.25, -0.2, -0.1), jitter=1e-2,
                           seed=cols * rows)
        if (cols, rows) == (7, 5):
            sp["ks"] = rng.uniform(10.0, 100.0, len(sp)).astype(np.float32)
        V = rng.normal(0.0, 0.02, X.shape).astype(np.float32)
        V[[0, cols - 1]] = 0.0
        descs.append(ClothDesc(n_vertices=cols * rows, springs=sp, pinned=np.array([0, cols - 1], np.int32),
                               cg_max_iter=40, cg_tol=1e-5))
        Xs.append(X)
        Vs.append(V)
    kinds = describe(descs)
    assert kinds[-1] == (0, 0) and all(k != (0, 0) for k in kinds[:-1])
    X, V = np.concatenate(Xs), np.concatenate(Vs)
    a, sa = run(descs, X, V, 8, True, executor=executor)
    b, sb = run(descs, X, V, 8, False, executor=executor)
    for x, y in zip(a, b):
        assert same_bits(x, y)
    assert np.array_equal(sa[0], sb[0])


def test_coupled_grid_unaffected():
    """COUPLED cloths keep their own assembly whatever the topology."""
    from opencloth_gb300 import JAC_COUPLED

    X, sp = grid_cloth(17, 17)
    d = ClothDesc(n_vertices=289, springs=sp, pinned=np.array([0, 16], np.int32), jacobian_mode=JAC_COUPLED,
                  cg_max_iter=100, cg_tol=1e-6)
    a, _ = run(d, X, np.zeros_like(X), 5, True)
    b, _ = run(d, X, np.zeros_like(X), 5, False)
    for x, y in zip(a, b):
        assert same_bits(x, y)


@pytest.mark.parametrize("executor", ["streamed", "resident"])
def test_spring_params_refit_the_stencil(executor):
    """oc_set_spring_params on grid cloths: Ks / Kd scaled per spring type still fit the
    stencil's parameter slots (the slots take the new values); per-spring values move the
    cloth to the incidence gather; the original values move it back.  Each state steps
    exactly (bit for bit) like a handle created with those parameters."""
    rng = np.random.default_rng(8)
    descs, Xs, Vs = [], [], []
    for cols, rows in ((19, 19), (26, 11)):
        X, sp = grid_cloth(cols, rows, ks=(50.75, 40.0, 30.0), kd=(-0.25, -0.2, -0.1), jitter=1e-3,
                           seed=cols + rows)
        V = rng.normal(0.0, 0.02, X.shape).astype(np.float32)
        V[[0, cols - 1]] = 0.0
        descs.append(ClothDesc(n_vertices=cols * rows, springs=sp, pinned=np.array([0, cols - 1], np.int32),
                               cg_max_iter=40, cg_tol=1e-5))
        Xs.append(X)
        Vs.append(V)
    X, V = np.concatenate(Xs), np.concatenate(Vs)
    ks0 = np.concatenate([d.springs["ks"] for d in descs])
    kd0 = np.concatenate([d.springs["kd"] for d in descs])
    scaled = (ks0 * np.float32(1.5)).astype(np.float32)
    per_spring = (ks0 * np.exp(rng.normal(0.0, 0.1, ks0.size))).astype(np.float32)

    def fresh(ks, kd):
        out, o = [], 0
        for d in descs:
            sp = d.springs.copy()
            n = len(sp)
            sp["ks"], sp["kd"] = ks[o:o + n], kd[o:o + n]
            o += n
            out.append(ClothDesc(n_vertices=d.n_vertices, springs=sp, pinned=d.pinned, cg_max_iter=40, cg_tol=1e-5))
        with ClothSolver(out, executor=executor) as s:
            s.set_state(X, V)
            s.step(DT, 6)
            return s.get_state(), [k != (0, 0) for k in describe(out)]

    with ClothSolver(descs, executor=executor) as s:
        for ks, kd, stencil in ((scaled, kd0 * np.float32(0.5), True), (per_spring, kd0, False), (ks0, kd0, True)):
            kd = kd.astype(np.float32)
            s.set_spring_params(ks=ks, kd=kd)
            s.set_state(X, V, np.zeros_like(X))
            s.step(DT, 6)
            got = s.get_state()
            want, kinds = fresh(ks, kd)
            assert all(k == stencil for k in kinds)
            for x, y in zip(got, want):
                assert same_bits(x, y)


def run_env(descs, X, V, steps, env: dict, dt: float = DT, **kw):
    """Create a handle with the given environment switches set (read at create time)."""
    old = {k: os.environ.get(k) for k in env}
    os.environ.update({k: str(v) for k, v in env.items()})
    try:
        s = ClothSolver(descs, **kw)
    finally:
        for k, v in old.items():
            if v is None:
                del os.environ[k]
            else:
                os.environ[k] = v
    with s:
        s.set_state(X, V)
        s.step(dt, steps)
        return s.get_state(), s.stats()


def strip_batch(seed: int):
    """Grid cloths for the strip sweep: exact spacing (rest lengths in the slots) and
    inexact (rest planes), square and not, widths around the strip boundaries (28 owned
    columns per warp), extra pins, per-vertex masses and an external force on one cloth."""
    rng = np.random.default_rng(seed)
    descs, Xs, Vs = [], [], []
    for cols, rows in ((21, 21), (28, 9), (29, 30), (33, 17), (56, 57), (57, 20), (85, 40), (129, 65)):
        X, sp = grid_cloth(cols, rows, ks=tuple(rng.uniform(20, 80, 3)), kd=tuple(rng.uniform(-0.5, -0.05, 3)),
                           jitter=1e-2, seed=cols * 1000 + rows)
        V = rng.normal(0.0, 0.02, X.shape).astype(np.float32)
        pins = np.unique(np.array([0, cols - 1, int(rng.integers(0, cols * rows))], np.int32))
        V[pins] = 0.0
        mass = rng.uniform(0.5, 2.0, cols * rows).astype(np.float32) if cols == 33 else None
        ext = rng.normal(0.0, 1e-3, X.shape).astype(np.float32) if cols == 57 else None
        descs.append(ClothDesc(n_vertices=cols * rows, springs=sp, pinned=pins, mass=mass, ext_force=ext,
                               cg_max_iter=60, cg_tol=1e-6))
        Xs.append(X)
        Vs.append(V)
    return descs, np.concatenate(Xs), np.concatenate(Vs)


@pytest.mark.parametrize("rows_per_band", [0, 1, 2, 5, 16])
@pytest.mark.parametrize("executor", ["streamed", "resident"])
def test_strip_sweep_same_bits_as_stencil(rows_per_band, executor):
    """k_assemble_strip (each spring force once, bands of rows, delta0 summed in the
    sweep's own order) against k_assemble_grid (each spring at both ends): the same F, A
    and b; delta0's two orders agree to about 2^-48 relative, which leaves the float CG
    scalars, and so every step, the same bits here, for any band height."""
    descs, X, V = strip_batch(11)
    env = {"OC_STRIP": 1}
    if rows_per_band:
        env["OC_STRIP_ROWS"] = rows_per_band
    a, sa = run_env(descs, X, V, 12, env, executor=executor)
    b, sb = run_env(descs, X, V, 12, {"OC_STRIP": 0}, executor=executor)
    for x, y in zip(a, b):
        assert same_bits(x, y)
    assert np.array_equal(sa[0], sb[0]) and np.array_equal(sa[2], sb[2])


def test_strip_sweep_exact_spacing_and_passes():
    """Exact grid spacing (rest lengths in the parameter slots) with the StepPhysics passes,
    against the incidence-record gather."""
    from opencloth_gb300 import PASS_ELLIPSOID, PASS_PROVOT, reference_ellipsoid

    E, Einv = reference_ellipsoid()
    X, sp = grid_cloth(65, 33, ks=(50.75, 50.75, 50.95), kd=(-0.25, -0.25, -0.25))
    d = ClothDesc(n_vertices=65 * 33, springs=sp, pinned=np.array([0, 64], np.int32), cg_max_iter=200, cg_tol=1e-5,
                  passes=PASS_ELLIPSOID | PASS_PROVOT, ellipsoid=E, ellipsoid_inv=Einv)
    V = np.zeros_like(X)
    a, sa = run_env(d, X, V, 20, {"OC_STRIP": 1, "OC_STRIP_ROWS": 4})
    b, sb = run_env(d, X, V, 20, {"OC_STENCIL": 0})
    for x, y in zip(a, b):
        assert same_bits(x, y)
    assert np.array_equal(sa[0], sb[0])


def test_strip_sweep_profile_names_its_kernels():
    """Streamed cloths on the strip sweep: the persistent CG forms their delta0 itself, so
    k_assemble_finish does not run; with the WHILE-loop CG (persist 0) it does."""
    descs, X, V = strip_batch(3)
    with ClothSolver(descs, executor="streamed") as s:
        s.set_launch_config(strip=1)
        s.set_state(X, V)
        prof = s.profile(DT, 2)
        assert prof["k_assemble_strip"]["launches"] == 2 and prof["k_cg_persist"]["launches"] == 2
        assert "k_assemble_finish" not in prof
        s.set_launch_config(persist=0)
        s.set_state(X, V)
        prof = s.profile(DT, 2)
        assert prof["k_assemble_strip"]["launches"] == 2 and prof["k_assemble_finish"]["launches"] == 2
