"""GPU interaction and constraint entry points: the reference's vertex picking
(IMP:399-405) and drag (IMP:433-438) on the device state, per-step vertex overrides and
arbitrary pin sets.

Tolerances: picking, dragging and overrides are exact (the same FP32 expressions as
the oracle's restatement); a step after any of them is bit-exact against the port run
with the GPU's arithmetic, as every single step is; a handle whose pins were replaced
steps bit for bit like a handle created with those pins.
"""
import numpy as np
import pytest

import oracle
from opencloth_gb300 import ClothDesc, ClothSolver, OcError, grid_cloth

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0


def cloth(cols=21, rows=17, seed=2, pins=None):
    rng = np.random.default_rng(seed)
    X, sp = grid_cloth(cols, rows, ks=(50.75, 50.75, 50.95), kd=(-0.25, -0.25, -0.25), jitter=0.02, seed=seed)
    V = rng.normal(0.0, 0.02, X.shape).astype(np.float32)
    pins = np.array([0, cols - 1] if pins is None else pins, np.int32)
    V[pins] = 0.0
    desc = ClothDesc(n_vertices=cols * rows, springs=sp, pinned=pins, cg_max_iter=50, cg_tol=1e-5)
    ocl = oracle.Cloth(cols * rows, sp, pinned=pins, i_max=50, eps=1e-5)
    return desc, ocl, X, V


def test_pick_matches_reference_loop():
    desc, _, X, V = cloth()
    rng = np.random.default_rng(0)
    with ClothSolver(desc) as s:
        s.set_state(X, V)
        pts = [X[37] + np.float32(0.03), X[200], X[0] - np.float32(0.5), np.array([9.0, 9.0, 9.0], np.float32)]
        pts += [X[int(i)] + rng.normal(0.0, 0.08, 3).astype(np.float32) for i in rng.integers(0, len(X), 20)]
        for p in pts:
            for r in (0.1, 0.3):
                assert s.pick_vertex(p, r) == oracle.ref_pick(X, p, r), (p, r)
    assert oracle.ref_pick(X, np.array([9.0, 9.0, 9.0]), 0.1) == -1


def test_pick_in_a_batch_is_instance_local():
    a, _, Xa, Va = cloth(9, 9, seed=1)
    b, _, Xb, Vb = cloth(13, 11, seed=2)
    with ClothSolver([a, b]) as s:
        s.set_state(np.concatenate([Xa, Xb]), np.concatenate([Va, Vb]))
        assert s.pick_vertex(Xb[40], 0.01, instance=1) == oracle.ref_pick(Xb, Xb[40], 0.01)
        assert s.pick_vertex(Xa[3], 0.01, instance=0) == oracle.ref_pick(Xa, Xa[3], 0.01)


def test_drag_then_step_matches_port():
    """The reference's frame loop while dragging: OnMouseMove edits X/V, then StepPhysics."""
    desc, ocl, X, V = cloth()
    rng = np.random.default_rng(5)
    sel = 200
    Xo, Vo, dVo = X.copy(), V.copy(), np.zeros_like(X)
    with ClothSolver(desc) as s:
        s.set_state(X, V)
        for frame in range(12):
            delta = rng.normal(0.0, 0.02, 3).astype(np.float32)
            if frame == 5:
                delta[1] = np.float32(-50.0)  # would go below 0: y is kept (IMP:436)
            s.drag_vertex(sel, delta)
            Xo, Vo = oracle.ref_drag(Xo, Vo, sel, delta)
            Xg, Vg, _ = s.get_state()
            assert np.array_equal(Xg, Xo) and np.array_equal(Vg, Vo), frame
            s.step(DT, 1)
            Xo, Vo, dVo, _, _ = oracle.port_step(ocl, Xo, Vo, dVo, dt=DT, n_steps=1, dot_fp64=True,
                                                 filter_pinned=True)
            Xg, Vg, dVg = s.get_state()
            assert np.array_equal(Xg, Xo) and np.array_equal(Vg, Vo) and np.array_equal(dVg, dVo), frame


def test_set_vertices_overrides_positions_and_velocities():
    desc, ocl, X, V = cloth()
    idx = np.array([5, 77, 300], np.int64)
    newX = X[idx] + np.float32(0.1)
    newV = np.full((3, 3), 0.25, np.float32)
    with ClothSolver(desc) as s:
        s.set_state(X, V)
        s.set_vertices(idx, X=newX)
        s.set_vertices(idx[:2], V=newV[:2])
        Xg, Vg, _ = s.get_state()
        Xe, Ve = X.copy(), V.copy()
        Xe[idx] = newX
        Ve[idx[:2]] = newV[:2]
        assert np.array_equal(Xg, Xe) and np.array_equal(Vg, Ve)
        s.step(DT, 1)
        Xg, Vg, _ = s.get_state()
    Xo, Vo, _, _, _ = oracle.port_step(ocl, Xe, Ve, dt=DT, n_steps=1, dot_fp64=True, filter_pinned=True)
    assert np.array_equal(Xg, Xo) and np.array_equal(Vg, Vo)


def test_set_vertices_rejects_bad_input():
    desc, _, X, V = cloth()
    with ClothSolver(desc) as s:
        with pytest.raises(OcError) as e:
            s.set_vertices([len(X)], X=np.zeros((1, 3)))
        assert e.value.status == 2
        with pytest.raises(OcError) as e:
            s.set_vertices([3, 3], X=np.zeros((2, 3)))
        assert e.value.status == 1
        with pytest.raises(OcError) as e:
            s.set_vertices([3], V=np.full((1, 3), np.nan))
        assert e.value.status == 3
        with pytest.raises(OcError) as e:
            s.drag_vertex(len(X), [0.0, 0.0, 0.0])
        assert e.value.status == 2


@pytest.mark.parametrize("executor", ["streamed", "resident", "plain"])
def test_set_pins_equals_creating_with_those_pins(executor):
    new_pins = [0, 10, 20, 150, 356]
    desc_a, _, X, V = cloth()
    desc_b, _, _, _ = cloth(pins=new_pins)
    V = V.copy()
    V[new_pins] = 0.0
    with ClothSolver(desc_a, executor=executor) as a, ClothSolver(desc_b, executor=executor) as b:
        for s in (a, b):
            s.set_state(X, V)
        a.set_pins(new_pins)
        a.step(DT, 8)
        b.step(DT, 8)
        for x, y in zip(a.get_state(), b.get_state()):
            assert np.array_equal(x, y)
        a.set_pins([])  # no pins at all: the whole cloth falls
        a.step(DT, 2)
        assert np.all(np.isfinite(a.get_state()[0]))
