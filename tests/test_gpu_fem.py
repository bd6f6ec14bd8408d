"""GPU parity of the batched block-sparse CG with the FEM demo's semantics (FEM:837-922).

Tolerances (stated here, used below):
* Against the oracle run with the GPU's arithmetic (FP64 sums of the FP32 per-row dot
  terms): V within 1e-6 relative (max-norm over free rows).  The GPU's FP64 sums add
  the same terms in another order (float pairs within a warp, FP64 above), which can
  move d3 or d4 by an FP32 ulp.
* Against the reference CG's own FP32 result (golden): within twice the reference's
  FP32-to-FP64 distance on that system, or 1e-6.
* A system gives the same bits alone or in a batch, with or without the CUDA graph, and
  solved by one CTA on chip (the resident kernel, systems of up to 256 rows) or by the
  streamed kernels.
"""
import numpy as np
import pytest

import oracle
from cases import FEM_CASES, fem_golden
from opencloth_gb300 import OcError
from opencloth_gb300.fem import BsrSolver, fem_system

pytestmark = pytest.mark.gpu


def desc(sys_):
    return {"row_ptr": sys_.row_ptr, "col": sys_.col, "fixed": sys_.fixed, "i_max": sys_.i_max,
            "tolerance": sys_.tolerance, "tiny": sys_.tiny}


def solve(systems, use_graph=True, executor=0):
    with BsrSolver([desc(s) for s in systems], use_graph=use_graph, executor=executor) as s:
        s.set_system(np.concatenate([x.blocks for x in systems]), np.concatenate([x.b for x in systems]),
                     np.concatenate([x.V for x in systems]))
        s.solve()
        return s.solution()


def rel_free(a, b, sys_):
    free = sys_.fixed == 0
    return float(np.abs(a[free].astype(np.float64) - b[free]).max() / np.abs(b[free]).max())


@pytest.mark.parametrize("tag", FEM_CASES)
def test_matches_oracle_and_reference(tag):
    sys_, V32, _, V64, _ = fem_golden(tag)
    V, r = solve([sys_])
    Vo, ro = oracle.bsr_cg(sys_, dot_fp64=True)
    assert rel_free(V, Vo, sys_) <= 1e-6
    gap = rel_free(V32, V64, sys_)
    assert rel_free(V, V64, sys_) <= max(2.0 * gap, 1e-6)
    fixed = sys_.fixed == 1
    assert np.array_equal(V[fixed], sys_.V[fixed])  # fixed rows are never touched
    assert np.all(r[fixed] == 0.0)


def test_batch_and_graph_give_the_same_bits():
    systems = [fem_golden(t)[0] for t in FEM_CASES]
    Vb, rb = solve(systems)
    Vn, rn = solve(systems, use_graph=False)
    assert np.array_equal(Vb, Vn) and np.array_equal(rb, rn)
    off = np.cumsum([0] + [s.n for s in systems])
    for k, s in enumerate(systems):
        V1, r1 = solve([s])
        assert np.array_equal(Vb[off[k]:off[k + 1]], V1) and np.array_equal(rb[off[k]:off[k + 1]], r1), k


def test_iteration_counts_per_system():
    """i_max 0 (no iteration: V kept, residual = b - A V), 1 and 7, in one batch."""
    base = fem_golden("m30")[0]
    systems = []
    for imax in (0, 1, 7):
        s = oracle.BsrSystem(base.row_ptr, base.col, base.blocks, base.b, base.V, base.fixed, imax, base.tolerance,
                             base.tiny)
        systems.append(s)
    V, r = solve(systems)
    n = base.n
    for k, s in enumerate(systems):
        Vo, ro = oracle.bsr_cg(s, dot_fp64=True)
        assert rel_free(V[k * n:(k + 1) * n], Vo, s) <= 1e-6, k
        if s.i_max == 0:
            assert np.array_equal(V[:n], s.V)
            assert np.abs(r[:n] - ro).max() <= 1e-6 * np.abs(ro).max()


def test_generated_system_solves_like_the_oracle():
    g = fem_system(12, 5, 4, V=np.random.default_rng(3).normal(0.0, 0.2, (13 * 6 * 5, 3)))
    s = oracle.BsrSystem(g["row_ptr"], g["col"], g["blocks"], g["b"], g["V"], g["fixed"], 20)
    V, _ = solve([s])
    Vo, _ = oracle.bsr_cg(s, dot_fp64=True)
    assert rel_free(V, Vo, s) <= 1e-6


def test_validation():
    sys_ = fem_golden("m0")[0]
    with BsrSolver([desc(sys_)]) as s:
        # A refused system changes nothing: the next solve is the solve of the system
        # committed before it, bit for bit.
        s.set_system(sys_.blocks, sys_.b, sys_.V)  # infinities in fixed rows are the reference's own
        s.solve()
        V_ok, r_ok = s.solution()
        free_row = int(np.nonzero(sys_.fixed == 0)[0][0])
        for what in ("blocks", "b", "V"):
            s.set_system(sys_.blocks, sys_.b, sys_.V)  # the solve updates V in place: start over
            blocks, b, V = sys_.blocks.copy(), sys_.b.copy(), sys_.V.copy()
            if what == "blocks":
                blocks[sys_.row_ptr[free_row]] = np.nan
            elif what == "b":
                b[free_row, 1] = np.inf
            else:
                V[free_row, 2] = np.nan
            with pytest.raises(OcError) as e:
                s.set_system(blocks, b, V)
            assert e.value.status == 3, what
            s.solve()
            V2, r2 = s.solution()
            assert np.array_equal(V2.view(np.uint32), V_ok.view(np.uint32)), what
            assert np.array_equal(r2.view(np.uint32), r_ok.view(np.uint32)), what
    bad = desc(sys_)
    bad["col"] = sys_.col.copy()
    bad["col"][[0, 1]] = bad["col"][[1, 0]]  # not ascending within the row
    with pytest.raises(OcError) as e:
        BsrSolver([bad])
    assert e.value.status == 1
    bad["col"] = sys_.col.copy()
    bad["col"][3] = sys_.n
    with pytest.raises(OcError) as e:
        BsrSolver([bad])
    assert e.value.status == 2


def test_resident_gives_the_streamed_bits():
    """The demo's 176-row systems run resident under the default executor; the 375-row
    system is streamed beside them.  Every system gets the streamed executor's bits."""
    systems = [fem_golden(t)[0] for t in FEM_CASES]
    Vs, rs = solve(systems, executor=1)
    Va, ra = solve(systems)
    assert np.array_equal(Vs, Va) and np.array_equal(rs, ra)
    Vn, rn = solve(systems, use_graph=False)
    assert np.array_equal(Vs, Vn) and np.array_equal(rs, rn)
    small = systems[:3]
    Vr, rr = solve(small, executor=2)
    n = sum(x.n for x in small)
    assert np.array_equal(Vr, Vs[:n]) and np.array_equal(rr, rs[:n])
    with pytest.raises(OcError) as e:
        BsrSolver([desc(systems[3])], executor=2)  # 375 rows: more than one CTA's rows
    assert e.value.status == 7


def test_resident_iteration_counts_and_demo_mesh():
    """i_max 0, 1 and 7 in one resident batch, and a generated 10 x 3 x 3 demo mesh, against
    the oracle; the launch count is one kernel per solve."""
    base = fem_golden("m30")[0]
    systems = [oracle.BsrSystem(base.row_ptr, base.col, base.blocks, base.b, base.V, base.fixed, imax,
                                base.tolerance, base.tiny) for imax in (0, 1, 7)]
    g = fem_system(10, 3, 3, V=np.random.default_rng(5).normal(0.0, 0.2, (11 * 4 * 4, 3)))
    systems.append(oracle.BsrSystem(g["row_ptr"], g["col"], g["blocks"], g["b"], g["V"], g["fixed"], 20))
    with BsrSolver([desc(x) for x in systems], executor=2) as s:
        s.set_system(np.concatenate([x.blocks for x in systems]), np.concatenate([x.b for x in systems]),
                     np.concatenate([x.V for x in systems]))
        s.solve()
        V, r = s.solution()
        assert s.launch_count() == 1
    off = np.cumsum([0] + [x.n for x in systems])
    for k, x in enumerate(systems):
        Vo, ro = oracle.bsr_cg(x, dot_fp64=True)
        assert rel_free(V[off[k]:off[k + 1]], Vo, x) <= 1e-6, k
        if x.i_max == 0:
            assert np.array_equal(V[off[k]:off[k + 1]], x.V)
            assert np.abs(r[off[k]:off[k + 1]] - ro).max() <= 1e-6 * np.abs(ro).max()


def test_resident_edge_systems_give_the_streamed_bits():
    """Resident systems of different sizes in one launch (the shared-memory layout is
    sized for the largest), a system whose rows are all fixed, one with no blocks and
    one with i_max 0, beside a streamed system: the same bits as every system streamed."""
    rng = np.random.default_rng(11)

    def gen(dims, seed):
        n = (dims[0] + 1) * (dims[1] + 1) * (dims[2] + 1)
        g = fem_system(*dims, V=np.random.default_rng(seed).normal(0.0, 0.2, (n, 3)))
        return oracle.BsrSystem(g["row_ptr"], g["col"], g["blocks"], g["b"], g["V"], g["fixed"], 20)

    small, demo, big = gen((4, 2, 2), 1), gen((10, 3, 3), 2), gen((12, 5, 4), 3)
    all_fixed = oracle.BsrSystem(small.row_ptr, small.col, small.blocks, small.b, small.V,
                                 np.ones_like(small.fixed), 20)
    n0 = 40
    empty = oracle.BsrSystem(np.zeros(n0 + 1, np.int32), np.zeros(0, np.int32), np.zeros((0, 9), np.float32),
                             rng.normal(0.0, 1.0, (n0, 3)), rng.normal(0.0, 1.0, (n0, 3)), np.zeros(n0, np.uint8), 2)
    no_iter = oracle.BsrSystem(demo.row_ptr, demo.col, demo.blocks, demo.b, demo.V, demo.fixed, 0)
    systems = [small, demo, all_fixed, big, empty, no_iter]
    Vs, rs = solve(systems, executor=1)
    Va, ra = solve(systems)
    assert np.array_equal(Vs, Va, equal_nan=True) and np.array_equal(rs, ra, equal_nan=True)
    off = np.cumsum([0] + [x.n for x in systems])
    k = systems.index(all_fixed)
    assert np.array_equal(Va[off[k]:off[k + 1]], all_fixed.V) and np.all(ra[off[k]:off[k + 1]] == 0.0)
    for k in (0, 1, 3):
        Vo, _ = oracle.bsr_cg(systems[k], dot_fp64=True)
        assert rel_free(Va[off[k]:off[k + 1]], Vo, systems[k]) <= 1e-6, k


@pytest.mark.parametrize("variant", ["1", "2", "3", "5", "6", "7"])
def test_matrix_vector_variants_give_the_same_bits(variant, monkeypatch):
    """Every launch shape of the streamed matrix-vector pass (OC_BSR_VARIANT, read at
    create time: the unroll of the slot loop and the register cap) keeps each row's
    products in slot order and the default's thread-to-row map, so it gives the default's
    bits.  Systems of several slices and ragged last slices, batched, graph and
    host-driven."""
    rng = np.random.default_rng(11)
    gens = [fem_system(12, 5, 4, V=rng.normal(0.0, 0.2, (13 * 6 * 5, 3))),
            fem_system(7, 3, 9, V=rng.normal(0.0, 0.2, (8 * 4 * 10, 3)))]
    systems = [oracle.BsrSystem(g["row_ptr"], g["col"], g["blocks"], g["b"], g["V"], g["fixed"], 20) for g in gens]
    monkeypatch.delenv("OC_BSR_VARIANT", raising=False)
    V0, r0 = solve(systems, executor=1)
    monkeypatch.setenv("OC_BSR_VARIANT", variant)
    for graph in (True, False):
        V, r = solve(systems, use_graph=graph, executor=1)
        assert np.array_equal(V, V0) and np.array_equal(r, r0)
