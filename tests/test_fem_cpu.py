"""The FEM demo's block-sparse CG (FEM:837-922): the oracle's restatement pinned to the
reference, and the FEM system generator pinned to the reference's assembly (CPU only).

Bars: the FP32 restatement reproduces the reference CG bit for bit, and the FP64
restatement the reference's FP64 build, on systems the demo itself assembled (golden
fixtures everywhere; fresh runs where the reference tree exists).  The generator's
first-step system matches the reference's FP64 assembly to 1e-6 relative."""
import numpy as np
import pytest

import oracle
from cases import FEM_CASES, fem_golden
from opencloth_gb300.fem import fem_system, tet_block_mesh


@pytest.mark.parametrize("tag", FEM_CASES)
def test_port_matches_reference_cg_golden(tag):
    sys_, V32, r32, V64, r64 = fem_golden(tag)
    V, r = oracle.bsr_cg(sys_)
    assert np.array_equal(V, V32) and np.array_equal(r, r32)
    V, r = oracle.bsr_cg(sys_, fp64=True)
    assert np.array_equal(V, V64) and np.array_equal(r, r64)


@pytest.mark.parametrize("tag", FEM_CASES)
def test_fp64_dot_accumulation_stays_close(tag):
    """The GPU's arithmetic (FP64 sums of the FP32 per-row dot terms) against the
    reference's FP32 sequential sums: within the FP32 method's own distance from FP64."""
    sys_, V32, _, V64, _ = fem_golden(tag)
    V, _ = oracle.bsr_cg(sys_, dot_fp64=True)
    free = sys_.fixed == 0
    scale = np.abs(V64[free]).max()
    gap = np.abs(V32[free] - V64[free]).max() / scale
    assert np.abs(V[free] - V64[free]).max() / scale <= max(2.0 * gap, 1e-6)


def test_golden_cases_are_nontrivial():
    for tag in FEM_CASES:
        sys_, V32, r32, _, _ = fem_golden(tag)
        assert sys_.fixed.sum() > 0 and (~np.isfinite(sys_.blocks)).any()  # fixed rows carry FLT_MAX masses
        assert np.abs(V32 - sys_.V).max() > 0  # the solve moved V
        assert sys_.i_max == 20


def test_generator_pattern_matches_reference_mesh():
    sys_, _, _, _, _ = fem_golden("m0")
    g = fem_system(10, 3, 3, first_step=True)
    assert np.array_equal(g["row_ptr"], sys_.row_ptr) and np.array_equal(g["col"], sys_.col)
    assert np.array_equal(g["fixed"], sys_.fixed)
    free = sys_.fixed == 0
    fr = np.repeat(free, np.diff(sys_.row_ptr))
    # blocks against the FP32 reference: FP32 rounding of the same expressions
    assert np.abs(sys_.blocks[fr] - g["blocks"][fr]).max() <= 1e-6 * np.abs(g["blocks"][fr]).max()
    # b: the reference's FP32 b cancels terms ~1e5 to leave O(1): 1e-3 of noise
    assert np.abs(sys_.b[free] - g["b"][free]).max() <= 2e-3 * np.abs(g["b"][free]).max()


def test_mesh_generator_shapes():
    Xi, X, tets, fixed = tet_block_mesh(4, 2, 3)
    assert Xi.shape == (5 * 3 * 4, 3) and tets.shape == (5 * 4 * 2 * 3, 4)
    assert fixed.sum() == 3 * 4 and np.allclose(X - Xi, [0.0, 0.5, -0.15])


needs_fem = pytest.mark.skipif(not oracle.fem_available(), reason="reference FEM build not present here")


@needs_fem
def test_generator_matches_reference_fp64_assembly():
    import os
    import subprocess
    import tempfile

    with tempfile.TemporaryDirectory() as td:
        sp, op = os.path.join(td, "s.bin"), os.path.join(td, "o.bin")
        subprocess.run([str(oracle.fem_binary(True)), "--system", "0", sp, op], env=oracle._fem_env((6, 2, 3)),
                       check=True, capture_output=True)
        s64 = oracle.BsrSystem.from_bytes(open(sp, "rb").read())
    g = fem_system(6, 2, 3, first_step=True)
    free = s64.fixed == 0
    fr = np.repeat(free, np.diff(s64.row_ptr))
    assert np.array_equal(g["col"], s64.col)
    assert np.abs(s64.blocks[fr] - g["blocks"][fr]).max() <= 1e-6 * np.abs(g["blocks"][fr]).max()
    assert np.abs(s64.b[free] - g["b"][free]).max() <= 1e-6 * np.abs(g["b"][free]).max()


@needs_fem
@pytest.mark.parametrize("seed", [1, 2])
def test_port_matches_reference_cg_on_modified_systems(seed):
    """Fresh inputs: a demo system with a random warm start, random i_max and a random
    extra fixed set, through the reference's own CG."""
    rng = np.random.default_rng(seed)
    sys_, _, _ = oracle.fem_ref_system(int(rng.integers(0, 40)), (8, 3, 2))
    sys_.V = rng.normal(0.0, 0.3, sys_.V.shape).astype(np.float32)
    sys_.i_max = int(rng.integers(1, 40))
    fixed = sys_.fixed.copy()
    fixed[rng.choice(sys_.n, 5, replace=False)] = 1
    sys_.fixed = fixed
    V32, r32 = oracle.fem_ref_solve(sys_)
    V, r = oracle.bsr_cg(sys_)
    assert np.array_equal(V, V32) and np.array_equal(r, r32)


def _desc(sys_, **over):
    d = {"row_ptr": sys_.row_ptr.copy(), "col": sys_.col.copy(), "fixed": sys_.fixed.copy(), "i_max": sys_.i_max,
         "tolerance": sys_.tolerance, "tiny": sys_.tiny}
    d.update(over)
    return d


def test_create_validates_patterns_before_any_device_work():
    """oc_bsr_create checks every system's pattern and limits on the host first, so these
    fail the same way with or without a GPU: OC_ERR_INVALID_ARGUMENT (1) for a bad size,
    row pointer, column order (std::map order), limit or executor, OC_ERR_BAD_INDEX (2)
    for a column outside the system."""
    from opencloth_gb300 import OcError
    from opencloth_gb300.fem import BsrSolver

    sys_ = fem_golden("m0")[0]
    swapped = sys_.col.copy()
    swapped[[0, 1]] = swapped[[1, 0]]
    outside = sys_.col.copy()
    outside[3] = sys_.n
    negative = sys_.col.copy()
    negative[5] = -1
    shifted = sys_.row_ptr.copy()
    shifted[0] = 1
    cases = [
        ([_desc(sys_, col=swapped)], {}, 1),
        ([_desc(sys_, col=outside)], {}, 2),
        ([_desc(sys_, col=negative)], {}, 2),
        ([_desc(sys_, row_ptr=shifted)], {}, 1),
        ([_desc(sys_, i_max=-1)], {}, 1),
        ([_desc(sys_, tiny=-1.0)], {}, 1),
        ([_desc(sys_, tiny=float("nan"))], {}, 1),
        ([_desc(sys_), _desc(sys_, col=outside)], {}, 2),
        ([_desc(sys_)], {"executor": 9}, 1),
        ([_desc(sys_)], {"executor": -1}, 1),
    ]
    for descs, kw, status in cases:
        with pytest.raises(OcError) as e:
            BsrSolver(descs, **kw)
        assert e.value.status == status, (kw, status)
    with pytest.raises(OcError) as e:
        BsrSolver([])
    assert e.value.status == 1
