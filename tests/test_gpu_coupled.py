"""GPU parity of the COUPLED Jacobian mode against its CPU restatement.

The reference has no coupled system; the oracle for this mode is the restatement in
oracle/oc_coupled_impl.h, itself checked against an independent scipy assembly and a
direct solve (tests/test_coupled_cpu.py).

Tolerances (stated here, used below):
* One step is bit-exact against the FP32 restatement: the kernels evaluate the same
  expressions in the same order, and the CG scalars come from FP64 sums of the same
  FP32 per-vertex terms (the GPU sums pairs of floats exactly within a warp first).
* Over 40 steps the two may part through a CG scalar rounded differently: X within 1e-6
  relative (max-norm) of the FP32 restatement.
* Against the FP64 restatement over 40 steps: X within 1e-4 relative.
"""
import numpy as np
import pytest

import oracle
from opencloth_gb300 import (JAC_COUPLED, JAC_REFERENCE, PASS_ELLIPSOID, PASS_PROVOT, ClothDesc, ClothSolver, OcError,
                             grid_cloth)

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def coupled_case(cols=17, rows=13, seed=3, jitter=0.1, eps=1e-6, i_max=400, passes=0, gravity=(0.0, -0.00981, 0.0)):
    """A jittered grid (stretched and compressed springs), random Ks (some zero), Kd of
    both signs, per-vertex mass, random velocities, three pins."""
    rng = np.random.default_rng(seed)
    X, sp = grid_cloth(cols, rows, seed=seed)
    X = (X + rng.normal(0.0, jitter * 4.0 / (cols - 1), X.shape)).astype(np.float32)
    sp["ks"] = np.exp(rng.uniform(np.log(1.0), np.log(500.0), len(sp))).astype(np.float32)
    sp["ks"][::17] = 0.0
    sp["kd"] = rng.uniform(-0.5, 0.1, len(sp)).astype(np.float32)
    V = rng.normal(0.0, 0.05, X.shape).astype(np.float32)
    pins = np.array([0, cols - 1, cols * rows // 2], np.int32)
    V[pins] = 0.0
    mass = rng.uniform(0.5, 2.0, cols * rows).astype(np.float32)
    E = Einv = None
    if passes:
        from opencloth_gb300 import reference_ellipsoid
        E, Einv = reference_ellipsoid()
    desc = ClothDesc(n_vertices=cols * rows, springs=sp, pinned=pins, mass=mass, gravity=gravity, cg_max_iter=i_max,
                     cg_tol=eps, jacobian_mode=JAC_COUPLED, passes=passes, ellipsoid=E, ellipsoid_inv=Einv)
    ocl = oracle.Cloth(cols * rows, sp, pinned=pins, mass=mass, gravity=gravity, i_max=i_max, eps=eps, passes=passes,
                       ellipsoid=E, ellipsoid_inv=Einv)
    return desc, ocl, X, V


def run(desc, X, V, n, **kw):
    with ClothSolver(desc, **kw) as s:
        s.set_state(X, V)
        s.step(DT, n)
        out = s.get_state()
        it, rr, fl = s.stats()
    return out, (it, rr, fl)


@pytest.mark.parametrize("seed", [3, 4])
def test_one_step_bit_exact(seed):
    desc, ocl, X, V = coupled_case(seed=seed)
    (Xg, Vg, dVg), (it, rr, fl) = run(desc, X, V, 1)
    Xo, Vo, dVo, ito, rro, flo = oracle.coupled_step(ocl, X, V, dt=DT, n_steps=1)
    assert np.array_equal(Xg, Xo) and np.array_equal(Vg, Vo) and np.array_equal(dVg, dVo)
    assert it[0] == ito[0] and fl[0] == flo[0] == 0 and it[0] > 3


def test_multi_step_tracks_restatements():
    desc, ocl, X, V = coupled_case()
    (Xg, Vg, _), _ = run(desc, X, V, 40)
    Xo, Vo, _, _, _, _ = oracle.coupled_step(ocl, X, V, dt=DT, n_steps=40)
    assert rel(Xg, Xo) <= 1e-6
    X64, _, _, _, _, _ = oracle.coupled_step(ocl, X, V, dt=DT, n_steps=40, fp64=True)
    assert rel(Xg, X64) <= 1e-4


@pytest.mark.parametrize("executor,graph", [("streamed", False), ("plain", False), ("auto", True)])
def test_executors_agree_bit_for_bit(executor, graph):
    desc, _, X, V = coupled_case()
    ref, ref_stats = run(desc, X, V, 10)
    got, stats = run(desc, X, V, 10, executor=executor, use_graph=graph)
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)
    assert np.array_equal(stats[0], ref_stats[0])


def test_resident_executor_refuses_coupled():
    desc, _, _, _ = coupled_case()
    with pytest.raises(OcError) as e:
        ClothSolver(desc, executor="resident")
    assert e.value.status == 7


def test_mixed_batch_matches_single_runs():
    """REFERENCE cloths (one small enough to be resident, one streamed) and COUPLED
    cloths in one handle: each cloth's result is its single run's, bit for bit."""
    c1 = coupled_case(9, 7, seed=5)
    c2 = coupled_case(21, 15, seed=6)
    Xr, spr = grid_cloth(33, 33, ks=(50.75, 50.75, 50.95), kd=(-0.25, -0.25, -0.25), jitter=1e-3, seed=7)
    ref_small = ClothDesc(n_vertices=len(Xr), springs=spr, pinned=np.array([0, 32], np.int32), cg_max_iter=50,
                          cg_tol=1e-5)
    Xb, spb = grid_cloth(160, 140, ks=(50.75, 50.75, 50.95), kd=(-0.25, -0.25, -0.25), jitter=1e-3, seed=8)
    ref_big = ClothDesc(n_vertices=len(Xb), springs=spb, pinned=np.array([0, 159], np.int32), cg_max_iter=50,
                        cg_tol=1e-5, jacobian_mode=JAC_REFERENCE)
    parts = [(c1[0], c1[2], c1[3]), (ref_small, Xr, np.zeros_like(Xr)), (c2[0], c2[2], c2[3]),
             (ref_big, Xb, np.zeros_like(Xb))]
    with ClothSolver([p[0] for p in parts]) as s:
        s.set_state(np.concatenate([p[1] for p in parts]), np.concatenate([p[2] for p in parts]))
        s.step(DT, 6)
        Xs, Vs, dVs = s.get_state()
        off = s.offsets
        it_b, _, fl_b = s.stats()
    for k, (d, X, V) in enumerate(parts):
        (X1, V1, dV1), (it1, _, fl1) = run(d, X, V, 6)
        sl = slice(off[k], off[k + 1])
        assert np.array_equal(Xs[sl], X1) and np.array_equal(Vs[sl], V1) and np.array_equal(dVs[sl], dV1), k
        assert it_b[k] == it1[0] and fl_b[k] == fl1[0], k


def test_coupled_with_passes_bit_exact():
    desc, ocl, X, V = coupled_case(passes=PASS_ELLIPSOID | PASS_PROVOT)
    X = X.copy()
    X[:, 1] -= 2.5  # the lower rows cut the ellipsoid centred at y = 2
    X[:, 1] = np.maximum(X[:, 1], 0.0)
    (Xg, Vg, dVg), _ = run(desc, X, V, 1)
    Xo, Vo, dVo, _, _, _ = oracle.coupled_step(ocl, X, V, dt=DT, n_steps=1)
    assert np.array_equal(Xg, Xo) and np.array_equal(Vg, Vo) and np.array_equal(dVg, dVo)


def test_stiff_cloth_at_large_step_stays_bounded():
    X, sp = grid_cloth(41, 41, ks=(5000.0, 5000.0, 5000.0), kd=(-1.0, -1.0, -1.0))
    X = X * np.float32(1.05)
    desc = ClothDesc(n_vertices=len(X), springs=sp, pinned=np.array([0, 40], np.int32), gravity=(0.0, 0.0, 0.0),
                     cg_max_iter=1000, cg_tol=1e-6, jacobian_mode=JAC_COUPLED)
    with ClothSolver(desc) as s:
        s.set_state(X, np.zeros_like(X))
        s.step(1.0 / 30.0, 200)
        Xs, Vs, _ = s.get_state()
        _, _, fl = s.stats()
    assert fl[0] == 0 and np.all(np.isfinite(Xs)) and np.abs(Vs).max() < 0.2

    def energy(P, W):
        l = np.linalg.norm(P[sp["p1"]].astype(np.float64) - P[sp["p2"]], axis=1)
        return 0.5 * np.sum(sp["ks"] * (l - sp["rest_length"]) ** 2) + 0.5 * np.sum(W.astype(np.float64) ** 2)

    assert energy(Xs, Vs) < 0.1 * energy(X, np.zeros_like(X))


def test_reference_only_entry_points_refuse_coupled():
    desc, _, X, V = coupled_case()
    with ClothSolver(desc) as s:
        s.set_state(X, V)
        with pytest.raises(OcError) as e:
            s.tape_forward(DT, 4, 2)
        assert e.value.status == 7
        with pytest.raises(OcError) as e:
            s.assemble(DT)
        assert e.value.status == 7
        F = s.compute_forces()  # the forces are the reference's in either mode
    assert np.array_equal(F, oracle.port_forces(coupled_case()[1], X, V))
