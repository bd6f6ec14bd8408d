"""GPU parity: the sm_103a step against the oracle and the reference's own outputs.

Tolerances (stated here, used below).  "Relative" is the max-norm error over the
max-norm of the reference; "of the motion" is the max-norm error over the largest
displacement of the reference from the initial state, which a solver that did not move
the cloth fails.
* ComputeForces, the Jacobians and the assembly of A and b are FP32 with the
  reference's operation order and no FMA contraction: bit-exact against the port.
* The step differs from the FP32 reference only through the CG dot products, which
  accumulate in FP64: X within 1e-6 and V within 1e-5 relative after 1 step, X within
  1e-5 / V within 1e-4 after the last snapshot (600 steps at most); X within 1e-5 of the
  motion after 1 step and 1e-4 of the motion after the last snapshot.
* Against the port run with the GPU's arithmetic (FP64 dots, pinned filter) only the
  FP64 summation order differs: 1e-6 relative, 1e-4 of the motion.
* Against the FP64 build of the reference: X within 1e-4 relative after 600 steps.  Of
  the motion, the FP32 method itself is 6.1e-4 from FP64 after 600 steps of the 21 x 21
  cloth (the restatement in FP32 measures the same), so the bound there is 2e-3.
"""
import numpy as np
import pytest

import oracle
from cases import GOLDEN_CASES, desc_for, golden, oracle_for, rel, rel_disp, seeded_cloth
from opencloth_gb300 import FLAG_BREAKDOWN, FLAG_NON_FINITE, ClothSolver

pytestmark = pytest.mark.gpu

TOL_X_1, TOL_V_1 = 1e-6, 1e-5
TOL_X_600, TOL_V_600 = 1e-5, 1e-4
TOL_MOTION_1, TOL_MOTION_600 = 1e-5, 1e-4
TOL_PORT = 1e-6
TOL_FP64_X = 1e-4
TOL_FP64_MOTION = 2e-3
DT = 1.0 / 60.0


def solver_for(g, **kw):
    s = ClothSolver(desc_for(g), **kw)
    s.set_state(g["X0"], g["V0"], g["dV0"])
    return s


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_compute_forces_bit_exact(name):
    g = golden(name)
    with solver_for(g) as s:
        F = s.compute_forces()
    Fo = oracle.port_forces(oracle_for(g, explicit_pins=True), g["X0"], g["V0"])
    assert np.array_equal(F, Fo)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_assembly_bit_exact(name):
    g = golden(name)
    with solver_for(g) as s:
        A, b = s.assemble(g["dt"])
    _, Ao, bo = oracle.port_assemble(oracle_for(g, explicit_pins=True), g["X0"], g["V0"], g["dt"])
    assert np.array_equal(A, Ao)
    assert np.array_equal(b, bo)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_step_matches_reference_golden(name):
    g = golden(name)
    with solver_for(g) as s:
        done = 0
        for n in g["snaps32"]:
            s.step(g["dt"], int(n) - done)
            done = int(n)
            X, V, _ = s.get_state()
            tx, tv, tm = (TOL_X_1, TOL_V_1, TOL_MOTION_1) if n == 1 else (TOL_X_600, TOL_V_600, TOL_MOTION_600)
            assert rel(X, g[f"X32_{n}"]) <= tx, (name, n, rel(X, g[f"X32_{n}"]))
            assert rel(V, g[f"V32_{n}"]) <= tv, (name, n, rel(V, g[f"V32_{n}"]))
            assert rel_disp(X, g[f"X32_{n}"], g["X0"]) <= tm, (name, n, rel_disp(X, g[f"X32_{n}"], g["X0"]))


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_step_matches_port_with_gpu_arithmetic(name):
    g = golden(name)
    n = int(g["snaps32"][-1])
    with solver_for(g) as s:
        s.step(g["dt"], n)
        X, V, dV = s.get_state()
    Xo, Vo, dVo, _, _ = oracle.port_step(oracle_for(g, explicit_pins=True), g["X0"], g["V0"], g["dV0"], dt=g["dt"],
                                         n_steps=n, dot_fp64=True, filter_pinned=True)
    assert rel(X, Xo) <= TOL_PORT and rel(V, Vo) <= TOL_PORT and rel(dV, dVo) <= 10 * TOL_PORT
    assert rel_disp(X, Xo, g["X0"]) <= TOL_MOTION_600, rel_disp(X, Xo, g["X0"])


def test_one_step_bit_exact_against_port():
    g = golden("grid21_ref")
    with solver_for(g) as s:
        s.step(g["dt"], 1)
        X, V, dV = s.get_state()
    Xo, Vo, dVo, _, _ = oracle.port_step(oracle_for(g, explicit_pins=True), g["X0"], g["V0"], g["dV0"], dt=g["dt"],
                                         n_steps=1, dot_fp64=True, filter_pinned=True)
    assert np.array_equal(X, Xo) and np.array_equal(V, Vo) and np.array_equal(dV, dVo)


def test_error_against_fp64_reference():
    g = golden("grid21_ref")
    with solver_for(g) as s:
        s.step(g["dt"], 600)
        X, V, _ = s.get_state()
    assert rel(X, g["X64_600"]) <= TOL_FP64_X
    assert rel_disp(X, g["X64_600"], g["X0"]) <= TOL_FP64_MOTION


@pytest.mark.parametrize("executor,graph", [("streamed", True), ("streamed", False), ("plain", False),
                                            ("resident", True), ("resident", False)])
def test_executors_agree_bit_for_bit(executor, graph):
    g = golden("random7x5_ref")
    with solver_for(g) as base:
        base.step(g["dt"], 25)
        ref = base.get_state()
        ref_stats = base.stats()
    with solver_for(g, executor=executor, use_graph=graph) as s:
        s.step(g["dt"], 25)
        got = s.get_state()
        stats = s.stats()
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)
    assert np.array_equal(stats[0], ref_stats[0])


def test_large_jittered_cloth_converges_and_tracks_port():
    """A 129 x 129 cloth with the 1M-vertex configuration's parameters."""
    desc, ocl, X, V = seeded_cloth(129, 129, seed=11, random_params=False)
    with ClothSolver(desc) as s:
        s.set_state(X, V)
        s.step(1.0 / 60.0, 10)
        Xg, Vg, _ = s.get_state()
        it, rr, fl = s.stats()
    Xo, Vo, _, ito, rro = oracle.port_step(ocl, X, V, n_steps=10, dot_fp64=True, filter_pinned=True)
    assert fl[0] == 0 and rr[0] <= 1e-5 and 0 < it[0] <= 200
    assert it[0] == ito[-1]
    assert rel(Xg, Xo) <= TOL_PORT and rel(Vg, Vo) <= 1e-5


def test_state_round_trip_and_resume():
    g = golden("random7x5_ref")
    with solver_for(g) as s:
        X, V, dV = s.get_state()
        assert np.array_equal(X, g["X0"]) and np.array_equal(V, g["V0"]) and np.array_equal(dV, g["dV0"])
        s.step(g["dt"], 10)
        full = s.get_state()
    with solver_for(g) as a:
        a.step(g["dt"], 4)
        mid = a.get_state()
    with ClothSolver(desc_for(g)) as b:
        b.set_state(*mid)
        b.step(g["dt"], 6)
        resumed = b.get_state()
    for x, y in zip(full, resumed):
        assert np.array_equal(x, y)


def test_pinned_vertices_do_not_move():
    g = golden("grid21_ref")
    with solver_for(g) as s:
        s.step(g["dt"], 50)
        X, V, dV = s.get_state()
    for p in (0, g["cols"] - 1):
        assert np.array_equal(X[p], g["X0"][p]) and not V[p].any() and not dV[p].any()


def test_zero_length_spring_is_flagged_not_fatal():
    g = golden("grid21_ref")
    X = g["X0"].copy()
    X[22] = X[23]  # both endpoints of a structural spring coincide
    with ClothSolver(desc_for(g)) as s:
        s.set_state(X, g["V0"], g["dV0"])
        s.step(g["dt"], 1)
        _, _, fl = s.stats()
        assert fl[0] & FLAG_NON_FINITE
        s.set_state(g["X0"], g["V0"], np.zeros_like(X))  # the handle stays usable
        s.step(g["dt"], 1)
        X1, _, _ = s.get_state()
        _, _, fl = s.stats()
    assert fl[0] == 0 and np.isfinite(X1).all()


def test_non_finite_state_is_rejected():
    g = golden("grid21_ref")
    X = g["X0"].copy()
    X[5, 1] = np.nan
    with ClothSolver(desc_for(g)) as s:
        with pytest.raises(Exception) as e:
            s.set_state(X, g["V0"])
        assert getattr(e.value, "status", None) == 3


def test_iteration_cap_sets_not_converged():
    desc, _, X, V = seeded_cloth(33, 33, seed=3, i_max=1, eps=1e-9)
    with ClothSolver(desc) as s:
        s.set_state(X, V)
        s.step(1.0 / 60.0, 1)
        it, _, fl = s.stats()
    assert it[0] == 1 and fl[0] & 1


def test_indefinite_system_is_flagged():
    """dt = 1 with Ks = 500 makes A = I - h^2 Ks n n^T indefinite."""
    desc, _, X, V = seeded_cloth(9, 9, seed=4, i_max=50, eps=1e-9, velocity=0.1)
    desc.springs["ks"] = 500.0
    with ClothSolver(desc) as s:
        s.set_state(X, V)
        s.step(1.0, 1)
        it, _, fl = s.stats()
    assert fl[0] & (FLAG_BREAKDOWN | FLAG_NON_FINITE) or it[0] < 50
