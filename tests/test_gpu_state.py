"""State transfer through the C ABI: page-locked and pageable host arrays both go through
the handle's staging buffer and the copy engine and must move the same bits; input that
holds a NaN or Inf is refused before anything is committed."""
import numpy as np
import pytest

from cases import seeded_cloth
from opencloth_gb300 import ClothSolver

pytestmark = pytest.mark.gpu
DT = 1.0 / 60.0


def pinned(shape):
    import torch

    return torch.empty(shape, dtype=torch.float32, pin_memory=True).numpy()


def test_pinned_and_pageable_state_agree():
    desc, _, X, V = seeded_cloth(33, 21, seed=12, velocity=0.01)
    dV = np.random.default_rng(3).normal(0.0, 1e-3, X.shape).astype(np.float32)
    out = {}
    for kind in ("pageable", "pinned"):
        with ClothSolver(desc) as s:
            if kind == "pinned":
                Xi, Vi, dVi = pinned(X.shape), pinned(X.shape), pinned(X.shape)
                Xi[:], Vi[:], dVi[:] = X, V, dV
            else:
                Xi, Vi, dVi = X.copy(), V.copy(), dV.copy()
            s.set_state(Xi, Vi, dVi)
            s.step(DT, 4)
            Xo, Vo, dVo = (pinned(X.shape), pinned(X.shape), pinned(X.shape)) if kind == "pinned" else (
                np.empty_like(X), np.empty_like(X), np.empty_like(X))
            s.get_state_into(Xo, Vo, dVo)
            out[kind] = (Xo.copy(), Vo.copy(), dVo.copy())
            # a partial read: positions only
            Xp = pinned(X.shape) if kind == "pinned" else np.empty_like(X)
            s.get_state_into(Xp, None, None)
            assert np.array_equal(Xp, Xo)
    for a, b in zip(out["pageable"], out["pinned"]):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_pinned_non_finite_input_rejected():
    from opencloth_gb300 import OcError

    desc, _, X, V = seeded_cloth(9, 9, seed=2)
    Xi = pinned(X.shape)
    Xi[:] = X
    Xi[4, 1] = np.nan
    with ClothSolver(desc) as s:
        with pytest.raises(OcError) as e:
            s.set_state(Xi, V)
        assert e.value.status == 3


@pytest.mark.parametrize("executor", ["auto", "plain"])
def test_step_host_equals_set_step_get(executor):
    """oc_step_host (StepPhysics on host arrays, one wait) moves the same bits as
    oc_set_state + oc_step + oc_get_state, for every executor's step."""
    desc, _, X, V = seeded_cloth(40, 23, seed=21, velocity=0.01)
    with ClothSolver(desc, executor=executor) as a, ClothSolver(desc, executor=executor) as b:
        a.set_state(X, V, np.zeros_like(X))
        b.set_state(X, V, np.zeros_like(X))
        Xa, Va = X.copy(), V.copy()
        Xb, Vb = X.copy(), V.copy()
        for _ in range(3):
            a.step_host(Xa, Va, DT, 2)
            b.set_state(Xb, Vb)
            b.step(DT, 2)
            Xb, Vb, _ = b.get_state()
        assert np.array_equal(Xa.view(np.uint32), Xb.view(np.uint32))
        assert np.array_equal(Va.view(np.uint32), Vb.view(np.uint32))


def test_step_host_rejects_non_finite_input():
    """A NaN or Inf in oc_step_host's input fails with OC_ERR_NON_FINITE and changes
    neither the device state nor the caller's arrays; the handle then steps on as if the
    call had not happened."""
    from opencloth_gb300 import OcError

    desc, _, X, V = seeded_cloth(9, 9, seed=2, velocity=0.01)
    with ClothSolver(desc) as s, ClothSolver(desc) as t:
        for h in (s, t):
            h.set_state(X, V)
            h.step(DT, 2)
        before = s.get_state()
        for bad in ((7, 2, np.inf), (40, 0, np.nan)):
            Xi, Vi = X.copy(), V.copy()
            (Xi if bad[2] == np.inf else Vi)[bad[0], bad[1]] = bad[2]
            Xc, Vc = Xi.copy(), Vi.copy()
            with pytest.raises(OcError) as e:
                s.step_host(Xi, Vi, DT, 1)
            assert e.value.status == 3
            assert np.array_equal(Xi, Xc, equal_nan=True) and np.array_equal(Vi, Vc, equal_nan=True)
            after = s.get_state()
            for a, b in zip(before, after):
                assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
        s.step(DT, 3)
        t.step(DT, 3)
        for a, b in zip(s.get_state(), t.get_state()):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_set_state_rejects_non_finite_input_without_effect():
    from opencloth_gb300 import OcError

    desc, _, X, V = seeded_cloth(9, 9, seed=4, velocity=0.01)
    with ClothSolver(desc) as s:
        s.set_state(X, V)
        s.step(DT, 1)
        before = s.get_state()
        dV = np.zeros_like(X)
        dV[5, 1] = np.nan
        with pytest.raises(OcError) as e:
            s.set_state(X, V, dV)
        assert e.value.status == 3
        for a, b in zip(before, s.get_state()):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("cols,rows", [(33, 21), (16, 8), (5, 3)])
def test_device_state_aligned_and_unaligned_give_the_same_bits(cols, rows):
    """The device-pointer state functions take packed float triples at any 4-byte
    alignment: 16-byte aligned and unaligned arrays round-trip the same bits, for vertex
    counts that are and are not multiples of four, and agree with the host path."""
    import torch

    desc, _, X, V = seeded_cloth(cols, rows, seed=5, velocity=0.01)
    dV = np.random.default_rng(7).normal(0.0, 1e-3, X.shape).astype(np.float32)
    n3 = X.size
    sp = (n3 + 8 + 3) // 4 * 4  # floats between the arrays: a multiple of four
    res = {}
    for off in (0, 1):  # floats of offset: 0 keeps 16-byte alignment, 1 breaks it
        buf = torch.zeros(3 * sp, dtype=torch.float32, device="cuda")
        ins = [buf[k * sp + off: k * sp + off + n3] for k in range(3)]
        for t, a in zip(ins, (X, V, dV)):
            t.copy_(torch.from_numpy(a.reshape(-1)))
        assert all((t.data_ptr() % 16 == 0) == (off == 0) for t in ins)
        with ClothSolver(desc) as s:
            s.set_state_device(ins[0].data_ptr(), ins[1].data_ptr(), ins[2].data_ptr())
            s.synchronize()
            Xh, Vh, dVh = s.get_state()
            assert np.array_equal(Xh, X) and np.array_equal(Vh, V) and np.array_equal(dVh, dV)
            s.step(DT, 3)
            out = torch.zeros(3 * sp, dtype=torch.float32, device="cuda")
            outs = [out[k * sp + off: k * sp + off + n3] for k in range(3)]
            s.get_state_device(outs[0].data_ptr(), outs[1].data_ptr(), outs[2].data_ptr())
            s.synchronize()
            got = [t.cpu().numpy().reshape(-1, 3) for t in outs]
            ref = s.get_state()
            for g, r in zip(got, ref):
                assert np.array_equal(g.view(np.uint32), np.asarray(r).view(np.uint32))
            res[off] = got
    for a, b in zip(res[0], res[1]):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
