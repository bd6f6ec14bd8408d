"""The allocation-free solve (oc_pcg_solve_noalloc) against the step's own solve.

Callers that cannot allocate device memory (an engine with its own fixed device budget,
a real-time loop that must not call cudaMalloc) pass their own device buffers; the
solve's scratch is a static device array.  This checks, through the C ABI, that it
returns what oc_step's CG returns on the same system, on two calls in a row (the second
reuses the scratch the first left behind and starts from the first one's solution).
Collected last so that a failure here stops a run only after every other test ran.
"""
import ctypes as C

import numpy as np
import pytest

from cases import rel, seeded_cloth
from opencloth_gb300 import ClothSolver
from opencloth_gb300 import _native as N

pytestmark = pytest.mark.gpu
DT = 1.0 / 60.0
TOL = 1e-6  # the step-vs-port tolerance of test_gpu_parity


def test_noalloc_solve_matches_step_solve_on_two_calls():
    import torch

    lib = N.load()
    desc, _, X, V = seeded_cloth(129, 129, seed=21, random_params=False, velocity=0.01)
    n = desc.n_vertices
    assert n <= 65536
    mask = np.zeros(n, np.uint8)
    mask[desc.pinned] = 1
    d_pin = torch.from_numpy(mask).cuda()
    with ClothSolver(desc) as s:
        s.set_state(X, V, np.zeros_like(X))
        warm = np.zeros_like(X)
        for call in range(2):
            A9, b = s.assemble(DT)  # the system the next step solves
            s.step(DT, 1)
            _, _, dV = s.get_state()
            step_iters = int(s.stats()[0][0])

            d_A = torch.from_numpy(np.ascontiguousarray(A9.reshape(-1))).cuda()
            d_b = torch.from_numpy(np.ascontiguousarray(b.reshape(-1))).cuda()
            d_x = torch.from_numpy(np.ascontiguousarray(warm.reshape(-1))).cuda()
            torch.cuda.synchronize()
            iters, flags = C.c_int32(-1), C.c_uint32(99)
            st = lib.oc_pcg_solve_noalloc(d_A.data_ptr(), d_b.data_ptr(), d_x.data_ptr(), d_pin.data_ptr(), n,
                                          desc.cg_max_iter, desc.cg_tol, C.byref(iters), C.byref(flags), None)
            assert st == 0, (call, N.STATUS_NAMES.get(st, st))
            x = d_x.cpu().numpy().reshape(-1, 3)
            assert rel(x, dV) <= TOL, (call, rel(x, dV))
            # The two solves group delta0's FP64 partials by different block partitions
            # (about 2^-48 apart), which could move the stop test by one iteration.
            assert abs(iters.value - step_iters) <= 1 and flags.value == 0, (call, iters.value, step_iters,
                                                                             flags.value)
            warm = dV


def test_noalloc_solve_rejects_oversize_and_bad_arguments():
    lib = N.load()
    it, fl = C.c_int32(), C.c_uint32()
    assert lib.oc_pcg_solve_noalloc(None, None, None, None, 10, 10, 1e-3, C.byref(it), C.byref(fl), None) == 1
    # Sizes beyond the static scratch are refused before any device work.
    big = 65536 + 1
    assert lib.oc_pcg_solve_noalloc(1, 1, 1, None, big, 10, 1e-3, C.byref(it), C.byref(fl), None) == 7


def test_noalloc_solve_ignores_pinned_rows_system():
    """A pinned row's block and right-hand side are not used: a zero diagonal there (what a
    caller that filters pinned rows out of its own assembly may leave) still solves, and the
    free rows match the solve of the system with the pinned rows' original values."""
    import torch

    lib = N.load()
    desc, _, X, V = seeded_cloth(33, 17, seed=5, random_params=False, velocity=0.01)
    n = desc.n_vertices
    mask = np.zeros(n, np.uint8)
    mask[desc.pinned] = 1
    with ClothSolver(desc) as s:
        s.set_state(X, V, np.zeros_like(X))
        A9, b = s.assemble(DT)
    out = []
    for zero in (False, True):
        A, bb = A9.copy(), b.copy()
        if zero:
            A[desc.pinned] = 0.0
            bb[desc.pinned] = 123.0
        d_A = torch.from_numpy(np.ascontiguousarray(A.reshape(-1))).cuda()
        d_b = torch.from_numpy(np.ascontiguousarray(bb.reshape(-1))).cuda()
        d_x = torch.zeros(3 * n, dtype=torch.float32, device="cuda")
        d_pin = torch.from_numpy(mask).cuda()
        torch.cuda.synchronize()
        iters, flags = C.c_int32(-1), C.c_uint32(99)
        st = lib.oc_pcg_solve_noalloc(d_A.data_ptr(), d_b.data_ptr(), d_x.data_ptr(), d_pin.data_ptr(), n,
                                      desc.cg_max_iter, desc.cg_tol, C.byref(iters), C.byref(flags), None)
        assert st == 0 and flags.value == 0, (zero, st, flags.value)
        out.append(d_x.cpu().numpy().reshape(-1, 3))
    assert np.array_equal(out[0], out[1])
    assert not out[1][desc.pinned].any()
