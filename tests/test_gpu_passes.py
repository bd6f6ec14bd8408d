"""GPU parity of the passes after the update (the rest of StepPhysics, IMP:873-880):
EllipsoidCollision (IMP:824-848) and ApplyProvotDynamicInverse (IMP:800-823), and the
reference-named interface ImplicitCloth that runs them.

Tolerances (stated here, used below):
* The passes alone are FP32 with the reference's operation order: bit-exact against the
  port on the same input, standalone (oc_apply_passes) and fused into the step.
* One step with the passes is bit-exact against the port run with the GPU's arithmetic
  (FP64 dots, pinned filter), as the step without them is.
* Through ImplicitCloth over 10 steps against the reference's own FP32 outputs: X within
  1e-5, V within 1e-4 relative (max-norm), the multi-step tolerance of the step alone.
"""
import numpy as np
import pytest

import oracle
from cases import golden, oracle_for, rel
from opencloth_gb300 import (PASS_ELLIPSOID, PASS_PROVOT, ClothDesc, ClothSolver, ImplicitCloth, OcError,
                             grid_cloth)

pytestmark = pytest.mark.gpu

TOL_X_10, TOL_V_10 = 1e-5, 1e-4
BOTH = PASS_ELLIPSOID | PASS_PROVOT


def strained_case(cols=33, rows=33, seed=5, passes=BOTH):
    """A cloth cutting through the reference's ellipsoid, stretched so that many springs
    exceed 1.01 x rest, with random velocities and pins that include two adjacent pinned
    vertices (a spring with both ends pinned)."""
    g = golden("stepphysics21_ref")
    rng = np.random.default_rng(seed)
    X, sp = grid_cloth(cols, rows, jitter=0.02, seed=seed)
    X = X.copy()
    X[:, 0] *= rng.uniform(1.0, 1.06, len(X)).astype(np.float32)
    X[:, 1] = (X[:, 1] - 1.0) * 1.03 + 0.9
    X[:, 2] = rng.normal(0.0, 0.3, len(X)).astype(np.float32)
    V = rng.normal(0.0, 0.05, X.shape).astype(np.float32)
    pins = np.array(sorted({0, 1, cols - 1, int(rng.integers(2, cols * rows))}), np.int32)
    desc = ClothDesc(n_vertices=cols * rows, springs=sp, pinned=pins, passes=passes, ellipsoid=g["ellipsoid"],
                     ellipsoid_inv=g["ellipsoid_inv"], cg_max_iter=50, cg_tol=1e-5)
    ocl = oracle.Cloth(cols * rows, sp, pinned=pins, passes=passes, ellipsoid=g["ellipsoid"],
                       ellipsoid_inv=g["ellipsoid_inv"], i_max=50, eps=1e-5)
    return desc, ocl, X, V


def test_case_exercises_both_passes():
    desc, ocl, X, V = strained_case()
    Xe, Ve = oracle.port_passes(ocl, X, V, PASS_ELLIPSOID)
    moved = np.any(Xe != X, axis=1)
    assert moved.sum() >= 10 and np.all(Ve[moved] == 0)
    Xp, Vp = oracle.port_passes(ocl, X, V, PASS_PROVOT)
    assert np.array_equal(Xp, X) and np.any(Vp != V, axis=1).sum() > 100
    assert np.any(Vp[:2] != V[:2])  # vertex 1 (pinned) is p2 of a spring from pinned 0


@pytest.mark.parametrize("passes", [PASS_ELLIPSOID, PASS_PROVOT, BOTH])
def test_apply_passes_bit_exact(passes):
    desc, ocl, X, V = strained_case(passes=0)
    with ClothSolver(desc) as s:
        s.set_state(X, V)
        s.apply_passes(passes)
        Xg, Vg, _ = s.get_state()
    Xo, Vo = oracle.port_passes(ocl, X, V, passes)
    assert np.array_equal(Xg, Xo) and np.array_equal(Vg, Vo)


@pytest.mark.parametrize("executor,graph", [("streamed", True), ("streamed", False), ("plain", False),
                                            ("resident", True), ("resident", False)])
def test_one_step_with_passes_bit_exact(executor, graph):
    desc, ocl, X, V = strained_case()
    with ClothSolver(desc, executor=executor, use_graph=graph) as s:
        s.set_state(X, V)
        s.step(1.0 / 60.0, 1)
        Xg, Vg, dVg = s.get_state()
    Xo, Vo, dVo, _, _ = oracle.port_step(ocl, X, V, n_steps=1, dot_fp64=True, filter_pinned=True)
    assert np.array_equal(Xg, Xo) and np.array_equal(Vg, Vo) and np.array_equal(dVg, dVo)


def test_batch_mixes_cloths_with_and_without_passes():
    """Per-cloth pass bits in one ragged batch: each cloth matches its own single run."""
    cases = [strained_case(17, 13, seed=1, passes=BOTH), strained_case(9, 21, seed=2, passes=0),
             strained_case(25, 25, seed=3, passes=PASS_PROVOT), strained_case(33, 33, seed=4, passes=PASS_ELLIPSOID)]
    with ClothSolver([c[0] for c in cases]) as s:
        s.set_state(np.concatenate([c[2] for c in cases]), np.concatenate([c[3] for c in cases]))
        s.step(1.0 / 60.0, 5)
        Xb, Vb, _ = s.get_state()
        off = s.offsets
    for k, (desc, _, X, V) in enumerate(cases):
        with ClothSolver(desc) as one:
            one.set_state(X, V)
            one.step(1.0 / 60.0, 5)
            X1, V1, _ = one.get_state()
        assert np.array_equal(Xb[off[k]:off[k + 1]], X1) and np.array_equal(Vb[off[k]:off[k + 1]], V1), k


def test_set_passes_toggles_the_step():
    desc, ocl, X, V = strained_case()
    plain = ClothDesc(**{**desc.__dict__, "passes": 0, "_keep": []})
    with ClothSolver(plain) as a, ClothSolver(desc) as b:
        for s in (a, b):
            s.set_state(X, V)
        b.set_passes(0)
        a.step(1.0 / 60.0, 3)
        b.step(1.0 / 60.0, 3)
        for x, y in zip(a.get_state(), b.get_state()):
            assert np.array_equal(x, y)
        b.set_passes(BOTH)
        b.step(1.0 / 60.0, 1)
        Xs, Vs, dVs = a.get_state()
        Xo, Vo, _, _, _ = oracle.port_step(ocl, Xs, Vs, dVs, n_steps=1, dot_fp64=True, filter_pinned=True)
        Xg, Vg, _ = b.get_state()
        assert np.array_equal(Xg, Xo) and np.array_equal(Vg, Vo)


def test_tape_refuses_passes():
    desc, _, X, V = strained_case()
    with ClothSolver(desc) as s:
        s.set_state(X, V)
        with pytest.raises(OcError) as e:
            s.tape_forward(1.0 / 60.0, 4, 2)
        assert e.value.status == 7  # OC_ERR_UNSUPPORTED


def _implicit_from_golden(g):
    """ImplicitCloth built the reference's way: positions, then AddSpring calls."""
    cl = ImplicitCloth(g["X0"], g["V0"], pinned=[0, g["cols"] - 1], gravity=tuple(g["gravity"]),
                       cg_max_iter=g["i_max"], cg_tol=g["eps"], executor="streamed", ellipsoid=g["ellipsoid"],
                       ellipsoid_inv=g["ellipsoid_inv"])
    cl.springs = g["springs"].copy()  # AddSpring's rest length is the current distance: same records
    return cl


def test_implicit_cloth_stepphysics_matches_reference():
    g = golden("stepphysics21_ref")
    cl = _implicit_from_golden(g)
    for _ in range(10):
        cl.StepPhysics(g["dt"])
    assert rel(cl.X, g["X32_10"]) <= TOL_X_10
    assert rel(cl.V, g["V32_10"]) <= TOL_V_10


def test_implicit_cloth_functions_match_port():
    """ComputeForces, IntegrateImplicit, EllipsoidCollision and ApplyProvotDynamicInverse
    called one by one, as a caller of the reference would, against the port."""
    g = golden("stepphysics21_ref")
    cl = _implicit_from_golden(g)
    ocl = oracle_for(g, explicit_pins=True)
    F = cl.ComputeForces()
    assert np.array_equal(F, oracle.port_forces(ocl, g["X0"], g["V0"]))
    X, V, dV = g["X0"], g["V0"], g["dV0"]
    no_pass = oracle.Cloth(ocl.n_vertices, g["springs"], pinned=[0, g["cols"] - 1], gravity=tuple(g["gravity"]),
                           i_max=g["i_max"], eps=g["eps"])
    for _ in range(5):
        cl.IntegrateImplicit(g["dt"])
        X, V, dV, _, _ = oracle.port_step(no_pass, X, V, dV, dt=g["dt"], n_steps=1, dot_fp64=True,
                                          filter_pinned=True)
        assert np.array_equal(cl.X, X) and np.array_equal(cl.V, V)
        cl.EllipsoidCollision()
        X, V = oracle.port_passes(ocl, X, V, PASS_ELLIPSOID)
        assert np.array_equal(cl.X, X) and np.array_equal(cl.V, V)
        cl.ApplyProvotDynamicInverse()
        X, V = oracle.port_passes(ocl, X, V, PASS_PROVOT)
        assert np.array_equal(cl.X, X) and np.array_equal(cl.V, V)


def test_implicit_cloth_add_spring_rest_lengths():
    """AddSpring takes the current distance as the rest length (IMP:370-380)."""
    X, sp = grid_cloth(6, 5)
    cl = ImplicitCloth(X, pinned=[0, 5])
    for r in sp:
        cl.AddSpring(int(r["p1"]), int(r["p2"]), float(r["ks"]), float(r["kd"]), int(r["type"]))
    assert np.array_equal(cl.springs["rest_length"], sp["rest_length"])
    cl.StepPhysics(1.0 / 60.0)
    assert np.all(np.isfinite(cl.X))
