"""The persistent CG (k_cg_persist: every iteration of the streamed cloths in one
cooperative launch) against the two-kernel WHILE loop (OC_PERSIST=0): the same per-block
passes, the same fixed-order totals and scalar rules, so the same bits and the same
iteration counts."""
import os

import numpy as np
import pytest

from opencloth_gb300 import (FLAG_BREAKDOWN, FLAG_NON_FINITE, PASS_ELLIPSOID, PASS_PROVOT, ClothDesc, ClothSolver,
                             grid_cloth, reference_ellipsoid)

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0


def same_bits(a, b) -> bool:
    return np.array_equal(np.asarray(a).view(np.uint32), np.asarray(b).view(np.uint32))


def run(descs, X, V, steps, persist: bool, **kw):
    old = os.environ.get("OC_PERSIST")
    os.environ["OC_PERSIST"] = "1" if persist else "0"
    try:
        s = ClothSolver(descs, **kw)
    finally:
        if old is None:
            del os.environ["OC_PERSIST"]
        else:
            os.environ["OC_PERSIST"] = old
    with s:
        s.set_state(X, V)
        s.step(DT, steps)
        return s.get_state(), s.stats()


def cloth(cols, rows, seed, ks=(50.75, 50.75, 50.95), passes=0):
    rng = np.random.default_rng(seed)
    X, sp = grid_cloth(cols, rows, ks=ks, kd=(-0.25, -0.25, -0.25), jitter=1e-2, seed=seed)
    V = rng.normal(0.0, 0.01, X.shape).astype(np.float32)
    V[[0, cols - 1]] = 0.0
    E = Einv = None
    if passes:
        E, Einv = reference_ellipsoid()
    d = ClothDesc(n_vertices=cols * rows, springs=sp, pinned=np.array([0, cols - 1], np.int32), cg_max_iter=200,
                  cg_tol=1e-5, passes=passes, ellipsoid=E, ellipsoid_inv=Einv)
    return d, X, V


@pytest.mark.parametrize("graph", [True, False])
def test_single_large_cloth(graph):
    d, X, V = cloth(193, 161, 1)  # 31k vertices: streamed
    a, sa = run(d, X, V, 12, True, use_graph=graph)
    b, sb = run(d, X, V, 12, False, use_graph=graph)
    for x, y in zip(a, b):
        assert same_bits(x, y)
    assert np.array_equal(sa[0], sb[0]) and np.array_equal(sa[2], sb[2]) and sa[0][0] > 1


def test_several_streamed_cloths_beside_resident_ones():
    parts = [cloth(150, 140, 2), cloth(40, 40, 3), cloth(260, 90, 4, ks=(500.0, 400.0, 300.0)), cloth(17, 23, 5)]
    descs = [p[0] for p in parts]
    X = np.concatenate([p[1] for p in parts])
    V = np.concatenate([p[2] for p in parts])
    a, sa = run(descs, X, V, 10, True)
    b, sb = run(descs, X, V, 10, False)
    for x, y in zip(a, b):
        assert same_bits(x, y)
    assert np.array_equal(sa[0], sb[0]) and np.array_equal(sa[2], sb[2])


def test_many_streamed_cloths_of_different_lengths():
    """40 streamed cloths (more than the former 16-cloth limit), stiff and soft, so their
    CG loops end at different iterations and each cloth waits only for its own blocks:
    the same bits and iteration counts as the WHILE loop, and one launch for the CG."""
    rng = np.random.default_rng(9)
    parts = []
    for k in range(40):
        cols, rows = int(rng.integers(20, 90)), int(rng.integers(20, 90))
        ks = tuple(np.exp(rng.uniform(np.log(10.0), np.log(500.0), 3)))
        parts.append(cloth(cols, rows, 100 + k, ks=ks))
    descs = [p[0] for p in parts]
    X = np.concatenate([p[1] for p in parts])
    V = np.concatenate([p[2] for p in parts])
    a, sa = run(descs, X, V, 6, True, executor="streamed")
    b, sb = run(descs, X, V, 6, False, executor="streamed")
    for x, y in zip(a, b):
        assert same_bits(x, y)
    assert np.array_equal(sa[0], sb[0]) and np.array_equal(sa[2], sb[2])
    assert len(set(sa[0].tolist())) > 1  # the cloths stopped at different iterations
    with ClothSolver(descs, executor="streamed") as s:
        s.set_state(X, V)
        s.step(DT, 1)
        l0 = s.launch_count()
        s.step(DT, 3)
        assert s.launch_count() - l0 == 6  # per step: the stencil assembly and the persistent CG


def test_with_passes():
    d, X, V = cloth(150, 130, 6, ks=(5.0, 5.0, 5.0), passes=PASS_ELLIPSOID | PASS_PROVOT)
    X = X.copy()
    X[:, 1] -= 2.0
    a, _ = run(d, X, V, 8, True)
    b, _ = run(d, X, V, 8, False)
    for x, y in zip(a, b):
        assert same_bits(x, y)


def test_launch_count_is_per_step():
    d, X, V = cloth(193, 161, 7)
    with ClothSolver(d) as s:
        s.set_state(X, V)
        s.step(DT, 1)
        l0 = s.launch_count()
        s.step(DT, 5)
        # the stencil assembly and the persistent CG (with the update) per step
        assert s.launch_count() - l0 == 10
        s.set_launch_config(strip=1)
        l0 = s.launch_count()
        s.step(DT, 5)
        # with the strip sweep and the persistent CG, which forms the sweep's delta0 itself
        assert s.launch_count() - l0 == 10


def test_barrier_wait_runs_out_and_the_handle_steps_on():
    """One block of the persistent CG withholds its arrival at the first grid barrier
    and the others' waits run out after a short poll limit: the step reports
    OC_ERR_DEVICE_TIMEOUT (status 8), applies no update, and the handle then steps on
    with the same bits as a handle that never saw the fault."""
    from opencloth_gb300 import OcError
    from opencloth_gb300 import _native as N

    desc, X, V = cloth(65, 65, seed=31)
    with ClothSolver(desc, executor="streamed") as s, ClothSolver(desc, executor="streamed") as t:
        lib = N.load()
        for h in (s, t):
            h.set_state(X, V)
            h.step(DT, 1)
        before = s.get_state()
        assert lib.oc_test_barrier_timeout(s._h, 1, 2000) == 0
        s.step(DT, 1)
        with pytest.raises(OcError) as e:
            s.synchronize()
        assert e.value.status == 8
        after = s.get_state()
        assert same_bits(before[0], after[0]) and same_bits(before[1], after[1])  # no update applied
        assert lib.oc_test_barrier_timeout(s._h, -1, 0) == 0
        state = t.get_state()
        s.set_state(*state)
        s.step(DT, 3)
        t.step(DT, 3)
        for a, b in zip(s.get_state(), t.get_state()):
            assert same_bits(a, b)
        assert np.array_equal(s.stats()[0], t.stats()[0])


def test_stop_rules_per_cloth():
    """Streamed cloths that end their loops for every reason the scalar rule has, in one
    launch: converged, the iteration cap (OC_FLAG_NOT_CONVERGED after one iteration), no
    iterations at all (cg_max_iter 0) and an indefinite system (a stiffness whose h^2 Ks
    exceeds the mass, which breaks the CG down or ends it early).  Every block forms each
    cloth's totals and decisions itself; they must be the two-kernel loop's bits, flags
    and iteration counts."""
    specs = [(70, 60, 200, 1e-5, 50.0), (64, 52, 1, 1e-9, 50.0), (58, 66, 0, 1e-5, 50.0), (61, 57, 50, 1e-9, 5e5),
             (75, 40, 200, 1e-6, 20.0)]
    descs, Xs, Vs = [], [], []
    for k, (cols, rows, imax, tol, ks) in enumerate(specs):
        rng = np.random.default_rng(300 + k)
        X, sp = grid_cloth(cols, rows, ks=(ks, ks, ks), kd=(-0.25, -0.25, -0.25), jitter=1e-2, seed=300 + k)
        V = rng.normal(0.0, 0.05, X.shape).astype(np.float32)
        V[[0, cols - 1]] = 0.0
        descs.append(ClothDesc(n_vertices=cols * rows, springs=sp, pinned=np.array([0, cols - 1], np.int32),
                               cg_max_iter=imax, cg_tol=tol))
        Xs.append(X)
        Vs.append(V)
    X, V = np.concatenate(Xs), np.concatenate(Vs)
    a, sa = run(descs, X, V, 2, True, executor="streamed")
    b, sb = run(descs, X, V, 2, False, executor="streamed")
    for x, y in zip(a, b):
        assert same_bits(x, y)
    assert np.array_equal(sa[0], sb[0]) and np.array_equal(sa[2], sb[2])
    it, _, fl = sa
    assert it[1] == 1 and fl[1] & 1  # OC_FLAG_NOT_CONVERGED
    assert it[2] == 0
    assert fl[3] & (FLAG_BREAKDOWN | FLAG_NON_FINITE) or it[3] < 50
    assert it[0] > 1 and fl[0] == 0 and it[4] > 1
