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
