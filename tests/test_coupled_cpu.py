"""The COUPLED Jacobian mode's oracle, checked without a GPU.

The reference has no coupled system, so nothing of the reference can pin this mode.
The oracle (oracle/oc_coupled_impl.h) is checked instead against an independent
construction: the global 3N x 3N matrix and right-hand side assembled here with
vectorised numpy / scipy in FP64 from the mode's definition, and a direct sparse solve.

Tolerances: the FP64 oracle's matvec, diagonal blocks and right-hand side agree with the
independent assembly to 1e-12 relative (different summation order only); its CG at
tolerance 1e-12 agrees with the direct solve to 1e-8; the FP32 flavour tracks FP64 to
1e-5 relative over one step.
"""
import numpy as np
import pytest

import oracle
from opencloth_gb300 import grid_cloth

scipy_sparse = pytest.importorskip("scipy.sparse")
from scipy.sparse.linalg import spsolve  # noqa: E402

DT = 1.0 / 60.0


def case(cols=9, rows=7, seed=3, jitter=0.15, damping=-0.125):
    """A jittered grid with springs both stretched and compressed, random Ks (some
    zero) and Kd of both signs, random velocities and three pins."""
    rng = np.random.default_rng(seed)
    X, sp = grid_cloth(cols, rows, jitter=0.0, seed=seed)
    X = (X + rng.normal(0.0, jitter * 4.0 / (cols - 1), X.shape)).astype(np.float32)
    sp["ks"] = np.exp(rng.uniform(np.log(1.0), np.log(500.0), len(sp))).astype(np.float32)
    sp["ks"][::17] = 0.0
    sp["kd"] = rng.uniform(-0.5, 0.1, len(sp)).astype(np.float32)
    V = rng.normal(0.0, 0.1, X.shape).astype(np.float32)
    pins = np.array([0, cols - 1, cols * rows // 2], np.int32)
    V[pins] = 0.0
    mass = rng.uniform(0.5, 2.0, cols * rows).astype(np.float32)
    cl = oracle.Cloth(cols * rows, sp, pinned=pins, mass=mass, damping=damping, i_max=2000, eps=1e-12)
    return cl, sp, X, V, pins, mass


def assemble(sp, X, V, mass, damping, h):
    """Independent FP64 assembly of A, the stiffness Kt and b's spring term."""
    X = X.astype(np.float64)
    N = len(X)
    p1, p2 = sp["p1"].astype(np.int64), sp["p2"].astype(np.int64)
    dx = X[p1] - X[p2]
    l = np.linalg.norm(dx, axis=1)
    n = dx / l[:, None]
    ks = sp["ks"].astype(np.float64)
    kd = sp["kd"].astype(np.float64)
    ksn = np.maximum(ks, 0.0)
    kdn = np.maximum(-kd, 0.0)
    kst = ksn * np.maximum(1.0 - sp["rest_length"].astype(np.float64) / l, 0.0)
    nn = n[:, :, None] * n[:, None, :]
    eye = np.eye(3)[None]
    Kt = kst[:, None, None] * eye + (ksn - kst)[:, None, None] * nn
    B = h * kdn[:, None, None] * nn + h * h * Kt

    def glob(blocks):
        rows, cols, vals = [], [], []
        for (a, b_, sgn) in ((p1, p1, 1.0), (p1, p2, -1.0), (p2, p1, -1.0), (p2, p2, 1.0)):
            for r in range(3):
                for c in range(3):
                    rows.append(3 * a + r)
                    cols.append(3 * b_ + c)
                    vals.append(sgn * blocks[:, r, c])
        return scipy_sparse.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                                       shape=(3 * N, 3 * N))

    mprime = mass.astype(np.float64) + h * max(-damping, 0.0)
    A = glob(B) + scipy_sparse.diags(np.repeat(mprime, 3))
    return A.tocsr(), glob(Kt).tocsr()


def test_matvec_matches_independent_assembly():
    cl, sp, X, V, pins, mass = case()
    A, _ = assemble(sp, X, V, mass, -0.125, DT)
    rng = np.random.default_rng(1)
    for _ in range(3):
        w = rng.normal(size=X.shape)
        y = oracle.coupled_matvec(cl, X, w, DT).ravel()
        ref = A @ w.ravel()
        assert np.abs(y - ref).max() <= 1e-12 * np.abs(ref).max()


def test_system_blocks_and_rhs_match_independent_assembly():
    cl, sp, X, V, pins, mass = case()
    A, Kt = assemble(sp, X, V, mass, -0.125, DT)
    D6, P6, b = oracle.coupled_system(cl, X, V, DT)
    Ad = A.toarray()
    idx = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
    for i in range(len(X)):
        blk = Ad[3 * i:3 * i + 3, 3 * i:3 * i + 3]
        assert np.allclose([blk[r, c] for r, c in idx], D6[i], rtol=1e-12, atol=1e-15)
        Dm = np.array([[D6[i, 0], D6[i, 1], D6[i, 2]], [D6[i, 1], D6[i, 3], D6[i, 4]], [D6[i, 2], D6[i, 4], D6[i, 5]]])
        Pm = np.array([[P6[i, 0], P6[i, 1], P6[i, 2]], [P6[i, 1], P6[i, 3], P6[i, 4]], [P6[i, 2], P6[i, 4], P6[i, 5]]])
        assert np.allclose(Dm @ Pm, np.eye(3), atol=1e-12)
    F = oracle.port_forces(cl, X.astype(np.float64), V.astype(np.float64), fp64=True).ravel()
    ref = DT * (F - DT * (Kt @ V.astype(np.float64).ravel()))
    assert np.abs(b.ravel() - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("seed,jitter", [(3, 0.15), (4, 0.4), (5, 0.0)])
def test_system_is_spd(seed, jitter):
    """Symmetric and positive definite even with compressed springs, zero Ks and Kd of
    either sign: every spring block is clamped to positive semi-definite."""
    cl, sp, X, V, pins, mass = case(seed=seed, jitter=jitter)
    A, _ = assemble(sp, X, V, mass, -0.125, DT)
    Ad = A.toarray()
    assert np.abs(Ad - Ad.T).max() <= 1e-14 * np.abs(Ad).max()  # duplicates summed in any order
    assert np.linalg.eigvalsh(Ad).min() > 0.0
    # the safeguard matters here: the unclamped transverse term is indefinite somewhere
    l = np.linalg.norm(X[sp["p1"]].astype(np.float64) - X[sp["p2"]], axis=1)
    if jitter > 0:
        assert (l < sp["rest_length"]).any()


def test_cg_matches_direct_solve():
    cl, sp, X, V, pins, mass = case()
    A, Kt = assemble(sp, X, V, mass, -0.125, DT)
    _, _, dV, it, rr, fl = oracle.coupled_step(cl, X, V, dt=DT, n_steps=1, fp64=True)
    _, _, b = oracle.coupled_system(cl, X, V, DT)
    free = np.setdiff1d(np.arange(len(X)), pins)
    fd = (3 * free[:, None] + np.arange(3)).ravel()
    sol = spsolve(A[fd][:, fd].tocsc(), b.ravel()[fd])
    assert fl[0] == 0 and it[0] > 5
    assert np.abs(dV.ravel()[fd] - sol).max() <= 1e-8 * np.abs(sol).max()
    assert np.all(dV[pins] == 0.0)


def test_step_update_and_pins():
    """V += dV, X += h V; pinned vertices keep their (zero) velocity and position."""
    cl, sp, X, V, pins, mass = case()
    X1, V1, dV, _, _, _ = oracle.coupled_step(cl, X, V, dt=DT, n_steps=1, fp64=True)
    V64 = V.astype(np.float64) + dV
    X64 = X.astype(np.float64) + DT * V64
    X64[:, 1] = np.maximum(X64[:, 1], 0.0)
    assert np.allclose(V1, V64, rtol=0, atol=1e-15) and np.allclose(X1, X64, rtol=0, atol=1e-15)
    assert np.array_equal(X1[pins], X[pins].astype(np.float64))


def test_fp32_tracks_fp64():
    cl, sp, X, V, pins, mass = case()
    cl.eps = 1e-6
    Xa, Va, _, _, _, _ = oracle.coupled_step(cl, X, V, dt=DT, n_steps=1)
    Xb, Vb, _, _, _, _ = oracle.coupled_step(cl, X, V, dt=DT, n_steps=1, fp64=True)
    assert np.abs(Xa - Xb).max() <= 1e-5 * np.abs(Xb).max()
    assert np.abs(Va - Vb).max() <= 1e-4 * np.abs(Vb).max()


def test_stiff_cloth_stays_bounded_at_large_step():
    """The point of the coupled system: a stiff cloth at a large time step stays bounded
    and loses energy monotonically (no gravity, released from a 5% stretch; the two pins
    keep part of the stretch, so the energy settles near 5% of its start)."""
    X, sp = grid_cloth(11, 11, ks=(5000.0, 5000.0, 5000.0), kd=(-1.0, -1.0, -1.0))
    X = X * np.float32(1.05)
    cl = oracle.Cloth(len(X), sp, pinned=[0, 10], gravity=(0.0, 0.0, 0.0), i_max=500, eps=1e-8)

    def energy(P, W):
        l = np.linalg.norm(P[sp["p1"]] - P[sp["p2"]], axis=1)
        return 0.5 * np.sum(sp["ks"] * (l - sp["rest_length"]) ** 2) + 0.5 * np.sum(W * W)

    P, W = X.astype(np.float64), np.zeros(X.shape)
    e = [energy(P, W)]
    for _ in range(10):
        P, W, _, _, _, fl = oracle.coupled_step(cl, P, W, dt=1.0 / 30.0, n_steps=20, fp64=True)
        assert np.all(fl == 0) and np.all(np.isfinite(P))
        e.append(energy(P, W))
    assert np.all(np.diff(e) < 0) and e[-1] < 0.1 * e[0]
    assert np.abs(W).max() < 1e-3
