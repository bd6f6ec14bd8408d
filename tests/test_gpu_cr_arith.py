"""The step's branch-free correctly rounded reciprocal, square root and quotient against
CUDA's IEEE intrinsics (__frcp_rn, __fsqrt_rn, __fdiv_rn) on the device.

The force, Jacobian and preconditioner arithmetic (IMP:720-727, 744-770, 312-314) takes
straight-line Markstein correction steps when its arguments lie in [2^-60, 2^60] and the
intrinsics otherwise; the step stays bit-exact only if both give the same bits.  The
reciprocal and square root are checked for every float of the range (an exhaustive
check), the quotient on random pairs from the ranges the springs produce."""
import ctypes as C

import pytest

from opencloth_gb300 import _native as N

pytestmark = pytest.mark.gpu


def test_branch_free_arithmetic_gives_the_ieee_bits():
    lib = N.load()
    counts = (C.c_uint64 * 3)()
    assert lib.oc_test_cr_arith(0, 1 << 32, 20261204, counts) == 0
    assert list(counts) == [0, 0, 0], f"mismatches (rcp, sqrt, div): {list(counts)}"


def test_rejects_bad_arguments():
    lib = N.load()
    assert lib.oc_test_cr_arith(0, 0, 0, None) == 1
