"""GPU adjoint of the implicit step (oc_tape_forward / oc_tape_backward).

Tolerance: the GPU runs the forward in FP32 with the CG to 1e-6; against FP64 central
differences (eps 1e-4 relative) of the same method, the directional derivatives along
six random directions per parameter group (Ks, Kd, initial velocity, external force, and
joint directions) agree within 1e-3 relative as a vector, ||ad - fd|| / ||fd||.  What
limits the agreement is the FP32 final state: an
exact FP64 adjoint seeded with the GPU's final positions shows the same error, so the
case is a 200-step trajectory whose loss residual X_T - target (~7e-3) sits far above
FP32 position resolution near y = 5 (~5e-7).  Gradient vectors agree with the FP64 CPU
adjoint within 1e-2 in norm.
"""
import numpy as np
import pytest

import oracle
from adjoint_cases import DT, fd_direction, make_case
from opencloth_gb300 import ClothDesc, ClothSolver

pytestmark = pytest.mark.gpu


def gpu_grads(case, every=10, executor="auto", cg_tol=1e-6, budget=0, info=None, intervals=None, layout=None):
    desc = ClothDesc(n_vertices=len(case["X"]), springs=case["springs"], pinned=case["pins"], cg_max_iter=500,
                     cg_tol=cg_tol)
    with ClothSolver(desc, executor=executor) as s:
        s.set_ext_force(case["ext"])
        s.set_state(case["X"], case["V0"], np.zeros_like(case["X"]))
        s.tape_forward(DT, case["steps"], every, budget, intervals=intervals)
        if info is not None:
            info.append(s.tape_info())
        if layout is not None:
            layout.append(s.tape_layout())
        X, _, _ = s.get_state()
        gX = 2.0 * (X - case["target"]) / len(X)
        g = s.tape_backward(gX)
        Xf, _, _ = s.get_state()
    assert np.array_equal(X, Xf)  # the handle is left at the final state
    return g, X


@pytest.fixture(scope="module")
def case():
    return make_case(cols=10, rows=8, steps=200, seed=5, v_sigma=0.1)


@pytest.fixture(scope="module")
def cpu(case):
    cl = oracle.Cloth(len(case["X"]), case["springs"], pinned=case["pins"], i_max=1000, eps=1e-10,
                      ext_force=case["ext"])
    Xo, _, _, _, _ = oracle.port_step(cl, case["X"], case["V0"], n_steps=case["steps"], fp64=True, dot_fp64=True,
                                      filter_pinned=True)
    gX = 2.0 * (Xo - case["target"]) / len(Xo)
    return oracle.port_adjoint(cl, case["X"], case["V0"], gX, dt=DT, n_steps=case["steps"])


def rms_rel(ad, fd):
    """Relative error of the vector of directional derivatives over the sampled
    directions: ||ad - fd|| / ||fd||.  A single direction whose derivative nearly cancels
    would otherwise dominate."""
    ad, fd = np.asarray(ad, np.float64), np.asarray(fd, np.float64)
    return float(np.linalg.norm(ad - fd) / max(np.linalg.norm(fd), 1e-300))


def nrel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64).ravel() - np.asarray(b, np.float64).ravel()) /
                 max(np.linalg.norm(np.asarray(b, np.float64).ravel()), 1e-30))


def test_gpu_adjoint_matches_fp64_cpu_adjoint(case, cpu):
    g, _ = gpu_grads(case)
    assert nrel(g["dKs"], cpu["gKs"]) <= 1e-2
    assert nrel(g["dKd"], cpu["gKd"]) <= 1e-2
    assert nrel(g["dV0"], cpu["gV0"]) <= 1e-2
    assert nrel(g["dext"], cpu["gExt"]) <= 1e-2
    assert nrel(g["dX0"], cpu["gX0"]) <= 1e-2


@pytest.mark.parametrize("name,key", [("ks", "dKs"), ("kd", "dKd"), ("V0", "dV0"), ("ext", "dext")])
def test_gpu_adjoint_matches_central_differences(case, name, key):
    g, _ = gpu_grads(case)
    rng = np.random.default_rng(11)
    fds, ads = [], []
    for _ in range(6):
        shape = case["springs"].shape if name in ("ks", "kd") else case["X"].shape
        u = rng.normal(size=shape)
        fd, d = fd_direction(case, name, u)
        fds.append(fd)
        ads.append(float(np.sum(g[key].astype(np.float64).reshape(d.shape) * d)))
    assert rms_rel(ads, fds) <= 1e-3, (name, fds, ads)


def test_gpu_adjoint_joint_direction_central_differences(case):
    from adjoint_cases import fd_joint

    g, _ = gpu_grads(case)
    rng = np.random.default_rng(12)
    keys = {"ks": "dKs", "kd": "dKd", "V0": "dV0", "ext": "dext"}
    fds, ads = [], []
    for _ in range(6):
        u = {"ks": rng.normal(size=case["springs"].shape), "kd": rng.normal(size=case["springs"].shape),
             "V0": rng.normal(size=case["X"].shape), "ext": rng.normal(size=case["X"].shape)}
        fd, d = fd_joint(case, u)
        fds.append(fd)
        ads.append(sum(float(np.sum(g[keys[k]].astype(np.float64).reshape(d[k].shape) * d[k])) for k in keys))
    assert rms_rel(ads, fds) <= 1e-3, (fds, ads)


def test_checkpoint_interval_does_not_change_gradients(case):
    ga, _ = gpu_grads(case, every=1)
    gb, _ = gpu_grads(case, every=13)
    gc, _ = gpu_grads(case, every=case["steps"])
    for k in ga:
        assert np.array_equal(ga[k], gb[k]) and np.array_equal(ga[k], gc[k]), k


def state_bytes(nv):
    """Bytes of one state of a cloth in the recompute tape: X and V (float4) and three
    planes of the handle's plane stride (the vertex count rounded up to 64)."""
    return 32 * nv + 12 * ((nv + 63) // 64 * 64)


def test_tapes_and_intervals_give_the_same_gradients(case):
    """The replay tape (the default interval, and intervals 1 and 7) and the recompute tape
    (no segment kept from the forward, and some): the same gradients bit for bit.  The
    replay tape rebuilds each state from its checkpoint with the step's own update; the
    recompute tape re-runs the steps; either way the reverse pass sees the same states."""
    st, every = state_bytes(len(case["X"])), 10
    n_ck = -(-case["steps"] // every)
    lay = []
    g0, _ = gpu_grads(case, every=every, layout=lay)
    runs = [gpu_grads(case, intervals=[1], layout=lay), gpu_grads(case, intervals=[7], layout=lay),
            gpu_grads(case, every=every, budget=st * (n_ck + 1 + every), layout=lay),
            gpu_grads(case, every=every, budget=st * (n_ck + 1 + 6 * every), layout=lay)]
    assert [k for k, _ in lay] == ["replay"] * 3 + ["recompute"] * 2
    assert [e.tolist() for _, e in lay[:3]] == [[every], [1], [7]]
    for g, _ in runs:
        for k in g0:
            assert np.array_equal(g0[k], g[k]), k


def test_per_cloth_intervals_give_the_same_gradients(case):
    """A batch of three cloths on the replay tape with a different interval per cloth: the
    same gradients bit for bit as one interval for all; under a byte budget that holds
    the replay tape, every cloth gets the default interval ceil(sqrt(steps))."""
    cases = [case, make_case(cols=9, rows=11, steps=case["steps"], seed=8),
             make_case(cols=12, rows=6, steps=case["steps"], seed=9)]
    descs = [ClothDesc(n_vertices=len(c["X"]), springs=c["springs"], pinned=c["pins"], cg_max_iter=500, cg_tol=1e-6)
             for c in cases]

    def grads(**kw):
        with ClothSolver(descs) as s:
            s.set_ext_force(np.concatenate([c["ext"] for c in cases]))
            s.set_state(np.concatenate([c["X"] for c in cases]), np.concatenate([c["V0"] for c in cases]))
            s.tape_forward(DT, case["steps"], 10, **kw)
            layout, info = s.tape_layout(), s.tape_info()
            X, _, _ = s.get_state()
            off = s.offsets
            gX = np.concatenate([2.0 * (X[off[k]:off[k + 1]] - c["target"]) / len(c["X"])
                                 for k, c in enumerate(cases)])
            return s.tape_backward(gX), layout, info

    g0, lay0, info0 = grads()
    assert lay0[0] == "replay" and lay0[1].tolist() == [10, 10, 10]
    g1, lay1, _ = grads(intervals=[1, 13, 200])
    assert lay1[1].tolist() == [1, 13, 200]
    g2, lay2, info2 = grads(intervals=[7, 1, 3])
    assert lay2[1].tolist() == [7, 1, 3]
    with ClothSolver(descs) as s:
        s.set_state(np.concatenate([c["X"] for c in cases]), np.concatenate([c["V0"] for c in cases]))
        s.tape_forward(DT, case["steps"], 0, info0[1])
        kind, ev = s.tape_layout()
        assert kind == "replay" and ev.tolist() == [15, 15, 15] and s.tape_info()[1] <= info0[1]
    for g in (g1, g2):
        for k in g0:
            assert np.array_equal(g0[k], g[k]), k


def test_streamed_and_resident_forward_give_the_same_gradients(case):
    ga, Xa = gpu_grads(case, executor="streamed")
    gb, Xb = gpu_grads(case, executor="resident")
    assert np.array_equal(Xa, Xb)
    for k in ga:
        assert nrel(ga[k], gb[k]) <= 1e-5, k


def test_batched_adjoint_equals_solo(case):
    other = make_case(cols=9, rows=11, steps=case["steps"], seed=8)
    cases = [case, other]
    descs = [ClothDesc(n_vertices=len(c["X"]), springs=c["springs"], pinned=c["pins"], cg_max_iter=500, cg_tol=1e-6)
             for c in cases]
    with ClothSolver(descs) as s:
        s.set_ext_force(np.concatenate([c["ext"] for c in cases]))
        s.set_state(np.concatenate([c["X"] for c in cases]), np.concatenate([c["V0"] for c in cases]))
        s.tape_forward(DT, case["steps"], 10)
        X, _, _ = s.get_state()
        off = s.offsets
        gX = np.concatenate([2.0 * (X[off[k]:off[k + 1]] - c["target"]) / len(c["X"]) for k, c in enumerate(cases)])
        g = s.tape_backward(gX)
    so = np.cumsum([0] + [len(c["springs"]) for c in cases])
    for k, c in enumerate(cases):
        solo, _ = gpu_grads(c)
        sl, ss = slice(off[k], off[k + 1]), slice(so[k], so[k + 1])
        assert np.array_equal(g["dV0"][sl], solo["dV0"]) and np.array_equal(g["dKs"][ss], solo["dKs"]), k


def test_torch_autograd_function(case):
    torch = pytest.importorskip("torch")
    from opencloth_gb300.autograd import trajectory

    desc = ClothDesc(n_vertices=len(case["X"]), springs=case["springs"], pinned=case["pins"], cg_max_iter=500,
                     cg_tol=1e-6)
    with ClothSolver(desc) as s:
        ks = torch.tensor(case["springs"]["ks"], requires_grad=True)
        kd = torch.tensor(case["springs"]["kd"], requires_grad=True)
        v0 = torch.tensor(case["V0"], requires_grad=True)
        ext = torch.tensor(case["ext"], requires_grad=True)
        # The loss in float64, as gpu_grads computes its seed: X - target cancels.
        target = torch.tensor(case["target"], dtype=torch.float64)
        X = trajectory(s, case["X"], ks, kd, v0, ext, DT, case["steps"], 10)
        loss = ((X.double() - target) ** 2).sum(dim=1).mean()
        loss.backward()
        g, _ = gpu_grads(case)
        assert np.allclose(ks.grad.numpy(), g["dKs"], rtol=1e-5, atol=1e-12)
        # One gradient step on Ks lowers the loss.
        with torch.no_grad():
            ks2 = ks * (1.0 - 1e-3 * ks.grad / max(float(ks.grad.abs().max()), 1e-30))
        X2 = trajectory(s, case["X"], ks2, kd.detach(), v0.detach(), ext.detach(), DT, case["steps"], 10)
        loss2 = ((X2.double() - target) ** 2).sum(dim=1).mean()
        assert float(loss2.detach()) < float(loss.detach())


def test_displacement_mode_tracks_the_positions_forward_and_its_gradients(case, cpu):
    """The displacement-mode taped forward (start positions + FP32 displacement, precise
    elongations): its final state agrees with the step's own forward (1e-5 of the motion)
    and with the FP64 method at least as closely; its gradients agree with the FP64 CPU
    adjoint within the positions mode's 1e-2, and the handle is left at the final
    positions."""
    desc = ClothDesc(n_vertices=len(case["X"]), springs=case["springs"], pinned=case["pins"], cg_max_iter=500,
                     cg_tol=1e-6)
    X0 = case["X"].astype(np.float64)
    cl = oracle.Cloth(len(case["X"]), case["springs"], pinned=case["pins"], i_max=1000, eps=1e-10,
                      ext_force=case["ext"])
    X64, _, _, _, _ = oracle.port_step(cl, case["X"], case["V0"], n_steps=case["steps"], fp64=True, dot_fp64=True,
                                       filter_pinned=True)
    out = {}
    for mode in (False, True):
        with ClothSolver(desc) as s:
            s.set_tape_mode(mode)
            s.set_ext_force(case["ext"])
            s.set_state(case["X"], case["V0"], np.zeros_like(case["X"]))
            s.tape_forward(DT, case["steps"], 10)
            Xp, _, _ = s.get_state()
            XT = X0 + s.tape_displacement() if mode else Xp.astype(np.float64)
            g = s.tape_backward(2.0 * (XT - case["target"]) / len(XT))
            assert np.array_equal(s.get_state()[0], Xp)
        out[mode] = (XT, g, Xp)
    motion = np.abs(X64 - X0).max()
    err_pos = np.abs(out[False][0] - X64).max() / motion
    err_disp = np.abs(out[True][0] - X64).max() / motion
    assert np.abs(out[True][0] - out[False][0]).max() / motion <= 1e-5
    assert err_disp <= max(err_pos, 1e-7), (err_disp, err_pos)
    assert np.abs(out[True][2] - out[True][0]).max() <= 1e-6  # the positions are start + u, rounded
    for k_gpu, k_cpu in (("dKs", "gKs"), ("dKd", "gKd"), ("dV0", "gV0"), ("dext", "gExt")):
        a = out[True][1][k_gpu].astype(np.float64).ravel()
        b = cpu[k_cpu].ravel()
        assert np.linalg.norm(a - b) <= 1e-2 * np.linalg.norm(b), k_gpu


def test_displacement_mode_on_a_batch_equals_solo_handles():
    """The displacement mode on a batch of 17 cloths, 16 small (resident) and one above
    the resident cut-off (streamed, its CG in the cooperative launch): every small cloth's
    displacement and gradients are those of a handle holding that cloth alone, bit for
    bit; the streamed cloth's agree within 1e-5 relative (its vertex blocks, and so its
    partial sums, are cut for the batch).  A COUPLED handle has no adjoint and refuses the
    mode (status 7)."""
    from opencloth_gb300 import JAC_COUPLED, OcError, grid_cloth

    rng = np.random.default_rng(11)
    cloths = []
    for k in range(17):
        n = int(rng.integers(5, 12)) if k else 140  # one cloth above the resident cut-off
        X, sp = grid_cloth(n, n, jitter=1e-2, seed=k)
        V0 = rng.normal(0.0, 0.05, X.shape).astype(np.float32)
        V0[[0, n - 1]] = 0.0
        cloths.append((ClothDesc(n_vertices=n * n, springs=sp, pinned=np.array([0, n - 1], np.int32),
                                 cg_max_iter=300, cg_tol=1e-6), X, V0))

    def run(items):
        with ClothSolver([d for d, _, _ in items]) as s:
            s.set_tape_mode(True)
            X = np.concatenate([x for _, x, _ in items])
            s.set_state(X, np.concatenate([v for _, _, v in items]), np.zeros_like(X))
            s.tape_forward(DT, 12, 4)
            u = s.tape_displacement()
            g = s.tape_backward(np.full_like(X, 1e-3))
            return u, g

    u, g = run(cloths)
    off = np.cumsum([0] + [d.n_vertices for d, _, _ in cloths])
    so = np.cumsum([0] + [len(d.springs) for d, _, _ in cloths])
    def close(a, b):
        return np.linalg.norm(a.astype(np.float64) - b) <= 1e-5 * np.linalg.norm(b.astype(np.float64))

    for k, item in enumerate(cloths):
        us, gs = run([item])
        sl, ss = slice(off[k], off[k + 1]), slice(so[k], so[k + 1])
        same = np.array_equal if k else close
        assert same(u[sl], us), k
        for key in ("dV0", "dext", "dX0"):
            assert same(g[key][sl], gs[key]), (k, key)
        for key in ("dKs", "dKd"):
            assert same(g[key][ss], gs[key]), (k, key)
    d, X, V0 = cloths[1]
    desc = ClothDesc(n_vertices=d.n_vertices, springs=d.springs, pinned=d.pinned, jacobian_mode=JAC_COUPLED)
    with ClothSolver(desc) as s:
        with pytest.raises(OcError) as e:
            s.set_tape_mode(True)
        assert e.value.status == 7
        with pytest.raises(OcError):
            s.tape_displacement()
