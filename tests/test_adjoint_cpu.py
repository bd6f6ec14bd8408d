"""The FP64 CPU adjoint (oracle/oc_adjoint.c), which the GPU adjoint is compared against,
against FP64 central differences of the same method."""
import numpy as np
import pytest

import oracle
from adjoint_cases import DT, fd_direction, make_case


@pytest.fixture(scope="module")
def case():
    return make_case(cols=7, rows=6, steps=8, seed=3)


@pytest.fixture(scope="module")
def grads(case):
    cl = oracle.Cloth(len(case["X"]), case["springs"], pinned=case["pins"], i_max=1000, eps=1e-10,
                      ext_force=case["ext"])
    Xo, _, _, _, _ = oracle.port_step(cl, case["X"], case["V0"], n_steps=case["steps"], fp64=True, dot_fp64=True,
                                      filter_pinned=True)
    n = len(case["X"])
    gX = 2.0 * (Xo - case["target"]) / n
    return oracle.port_adjoint(cl, case["X"], case["V0"], gX, dt=DT, n_steps=case["steps"])


@pytest.mark.parametrize("name,key", [("ks", "gKs"), ("kd", "gKd"), ("V0", "gV0"), ("ext", "gExt")])
def test_fp64_adjoint_matches_central_differences(case, grads, name, key):
    rng = np.random.default_rng(7)
    for _ in range(3):
        shape = case["springs"].shape if name in ("ks", "kd") else case["X"].shape
        u = rng.normal(size=shape)
        fd, d = fd_direction(case, name, u)
        ad = float(np.sum(grads[key].reshape(d.shape) * d))
        assert abs(fd - ad) <= 1e-5 * abs(fd) + 1e-18, (name, fd, ad)
