"""Ragged batches: many cloths of uneven sizes in one handle.

Each instance of a batch must give exactly (bit for bit) what it gives solved alone,
including its own CG iteration count (per-instance convergence), and must track the
oracle within the step tolerance of test_gpu_parity.
"""
import numpy as np
import pytest

import oracle
from cases import rel, seeded_cloth
from opencloth_gb300 import ClothSolver

pytestmark = pytest.mark.gpu
DT = 1.0 / 60.0


def make_batch(n, seed, lo=4, hi=40):
    rng = np.random.default_rng(seed)
    items = []
    for k in range(n):
        cols, rows = int(rng.integers(lo, hi + 1)), int(rng.integers(lo, hi + 1))
        eps = float(rng.choice([1e-3, 1e-5, 1e-6]))
        imax = int(rng.choice([3, 10, 200]))
        items.append(seeded_cloth(max(cols, 3), max(rows, 3), seed=1000 * seed + k, i_max=imax, eps=eps,
                                  velocity=0.01))
    return items


@pytest.mark.parametrize("executor", ["streamed", "plain", "resident", "auto"])
def test_batch_equals_solo_runs(executor):
    items = make_batch(12, seed=1)
    descs = [it[0] for it in items]
    X0 = np.concatenate([it[2] for it in items])
    V0 = np.concatenate([it[3] for it in items])
    with ClothSolver(descs, executor=executor) as s:
        s.set_state(X0, V0)
        s.step(DT, 7)
        Xb, Vb, dVb = s.get_state()
        itb, rrb, flb = s.stats()
        off = s.offsets
    for k, (desc, _, X, V) in enumerate(items):
        with ClothSolver(desc, executor=executor) as solo:
            solo.set_state(X, V)
            solo.step(DT, 7)
            Xs, Vs, dVs = solo.get_state()
            its, rrs, fls = solo.stats()
        sl = slice(off[k], off[k + 1])
        assert np.array_equal(Xb[sl], Xs) and np.array_equal(Vb[sl], Vs) and np.array_equal(dVb[sl], dVs), k
        assert itb[k] == its[0] and flb[k] == fls[0] and rrb[k] == rrs[0]


def test_batch_tracks_oracle_per_instance():
    items = make_batch(6, seed=2)
    with ClothSolver([it[0] for it in items]) as s:
        s.set_state(np.concatenate([it[2] for it in items]), np.concatenate([it[3] for it in items]))
        s.step(DT, 5)
        Xb, Vb, _ = s.get_state()
        itb, _, _ = s.stats()
        off = s.offsets
    for k, (_, ocl, X, V) in enumerate(items):
        Xo, Vo, _, ito, _ = oracle.port_step(ocl, X, V, n_steps=5, dot_fp64=True, filter_pinned=True)
        sl = slice(off[k], off[k + 1])
        assert rel(Xb[sl], Xo) <= 1e-6 and rel(Vb[sl], Vo) <= 1e-5, k
        assert itb[k] == ito[-1], k


def test_instances_converge_independently():
    """Two identical cloths with different tolerances stop at different iterations."""
    a = seeded_cloth(20, 20, seed=5, eps=1e-2)
    b = seeded_cloth(20, 20, seed=5, eps=1e-6)
    with ClothSolver([a[0], b[0]]) as s:
        s.set_state(np.concatenate([a[2], b[2]]), np.concatenate([a[3], b[3]]))
        s.step(DT, 3)
        it, rr, _ = s.stats()
    assert it[0] < it[1]
    assert rr[0] <= 1e-2 and rr[1] <= 1e-6


def test_single_vertex_and_springless_instances():
    """Degenerate shapes in a batch: no springs at all, a free vertex, a pinned vertex."""
    from opencloth_gb300 import SPRING_DTYPE, ClothDesc

    lone = ClothDesc(n_vertices=1, springs=np.zeros(0, SPRING_DTYPE))
    pinned = ClothDesc(n_vertices=2, springs=np.zeros(0, SPRING_DTYPE), pinned=np.array([1], np.int32))
    grid = seeded_cloth(5, 5, seed=9)
    X = np.concatenate([np.array([[0.0, 3.0, 0.0]], np.float32), np.array([[0, 2, 0], [1, 2, 0]], np.float32),
                        grid[2]])
    with ClothSolver([lone, pinned, grid[0]]) as s:
        s.set_state(X, np.zeros_like(X))
        s.step(DT, 3)
        Xg, Vg, _ = s.get_state()
    lone_o = oracle.Cloth(1, np.zeros(0, oracle.SPRING_DTYPE), pinned=[])
    Xo, Vo, _, _, _ = oracle.port_step(lone_o, X[:1], np.zeros((1, 3), np.float32), n_steps=3, dot_fp64=True,
                                       filter_pinned=True)
    assert rel(Xg[:1], Xo) <= 1e-6 and Xg[0, 1] < 3.0
    assert np.array_equal(Xg[2], X[2])  # the pinned vertex stays


def large_batch(seed):
    """Sizes that exercise every resident launch shape: one CTA (<= 1024 vertices) and
    clusters of 2..16 CTAs (up to 128 x 128 = 16384 vertices)."""
    sides = [8, 11, 16, 23, 32, 40, 45, 64, 90, 100, 127, 128]
    return [seeded_cloth(n, n, seed=100 * seed + k, velocity=0.01) for k, n in enumerate(sides)]


def run_batch(items, executor, steps=6):
    with ClothSolver([it[0] for it in items], executor=executor) as s:
        s.set_state(np.concatenate([it[2] for it in items]), np.concatenate([it[3] for it in items]))
        s.step(DT, steps)
        X, V, dV = s.get_state()
        it, rr, fl = s.stats()
        return X, V, dV, it, rr, fl, s.offsets


def test_resident_matches_streamed():
    """Same arithmetic, different FP64 summation order across CTAs: within 1e-6."""
    items = large_batch(1)
    Xr, Vr, dVr, itr, rrr, flr, off = run_batch(items, "resident")
    Xs, Vs, dVs, its, rrs, fls, _ = run_batch(items, "streamed")
    for k in range(len(items)):
        sl = slice(off[k], off[k + 1])
        assert rel(Xr[sl], Xs[sl]) <= 1e-6 and rel(Vr[sl], Vs[sl]) <= 1e-5, k
        assert abs(int(itr[k]) - int(its[k])) <= 1 and flr[k] == fls[k] == 0, k
        assert rrr[k] <= 1e-5


def test_resident_tracks_oracle():
    items = large_batch(2)[::3]
    Xb, Vb, _, itb, _, _, off = run_batch(items, "resident", steps=4)
    for k, (_, ocl, X, V) in enumerate(items):
        Xo, Vo, _, ito, _ = oracle.port_step(ocl, X, V, n_steps=4, dot_fp64=True, filter_pinned=True)
        sl = slice(off[k], off[k + 1])
        assert rel(Xb[sl], Xo) <= 1e-6 and rel(Vb[sl], Vo) <= 1e-5, k
        assert abs(int(itb[k]) - int(ito[-1])) <= 1, k


def test_auto_mixes_resident_and_streamed_cloths():
    """A cloth above the resident size limit runs streamed beside resident cloths in one
    graph; each matches its solo run bit for bit."""
    items = [seeded_cloth(20, 20, seed=31), seeded_cloth(140, 140, seed=32), seeded_cloth(50, 50, seed=33)]
    Xb, Vb, dVb, itb, _, _, off = run_batch(items, "auto", steps=5)
    for k, (desc, _, X, V) in enumerate(items):
        with ClothSolver(desc) as solo:
            solo.set_state(X, V)
            solo.step(DT, 5)
            Xs, Vs, dVs = solo.get_state()
            its = solo.stats()[0]
        sl = slice(off[k], off[k + 1])
        assert np.array_equal(Xb[sl], Xs) and np.array_equal(Vb[sl], Vs) and np.array_equal(dVb[sl], dVs), k
        assert itb[k] == its[0]


def test_resident_rejects_oversize_cloth():
    from opencloth_gb300 import OcError

    big = seeded_cloth(200, 200, seed=5)[0]
    with pytest.raises(OcError) as e:
        ClothSolver(big, executor="resident")
    assert e.value.status == 7


def test_fused_resident_step_matches_separate_assembly(monkeypatch):
    """OC_RESIDENT_FUSED=1: the resident kernel assembles its cloths' systems itself.
    Same per-vertex arithmetic, delta0 summed per CTA instead of per assembly block: the
    states agree within 1e-6 (X) / 1e-5 (V), on grid cloths (stencil gather) and on a
    cloth whose shuffled spring order takes the CSR gather."""
    import dataclasses

    items = large_batch(3)[::2]
    d, ocl, X, V = seeded_cloth(30, 30, seed=77, velocity=0.01)
    perm = np.random.default_rng(5).permutation(len(d.springs))
    items.append((dataclasses.replace(d, springs=d.springs[perm]), ocl, X, V))
    monkeypatch.setenv("OC_RESIDENT_FUSED", "0")
    Xs, Vs, dVs, its, _, fls, off = run_batch(items, "resident")
    monkeypatch.setenv("OC_RESIDENT_FUSED", "1")
    Xf, Vf, dVf, itf, rrf, flf, _ = run_batch(items, "resident")
    for k in range(len(items)):
        sl = slice(off[k], off[k + 1])
        assert rel(Xf[sl], Xs[sl]) <= 1e-6 and rel(Vf[sl], Vs[sl]) <= 1e-5, k
        assert abs(int(itf[k]) - int(its[k])) <= 1 and flf[k] == fls[k] == 0 and rrf[k] <= 1e-5, k
