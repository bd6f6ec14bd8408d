"""Launch configurations and the autotuner on the GPU: re-planning a handle keeps its
state and results, every configuration steps within the parity tolerance of the default
one, and the tuned handle gives the same bits as a handle set to the same configuration
explicitly."""
import numpy as np
import pytest

from cases import rel
from opencloth_gb300 import ClothDesc, ClothSolver, grid_cloth

pytestmark = pytest.mark.gpu
DT = 1.0 / 60.0


def same_bits(a, b) -> bool:
    return np.array_equal(np.asarray(a).view(np.uint32), np.asarray(b).view(np.uint32))


def mixed(seed=5):
    """Grid cloths that go resident, one too large to (streamed, strip sweep), and one with
    per-spring Ks (incidence-record gather)."""
    rng = np.random.default_rng(seed)
    descs, Xs, Vs = [], [], []
    for n in (12, 40, 77, 140):
        X, sp = grid_cloth(n, n, ks=tuple(rng.uniform(20, 200, 3)), kd=tuple(rng.uniform(-0.5, -0.05, 3)),
                           jitter=1e-3, seed=seed + n)
        if n == 40:
            sp["ks"] = (sp["ks"] * np.exp(rng.normal(0, 0.1, len(sp)))).astype(np.float32)
        V = rng.normal(0, 0.01, X.shape).astype(np.float32)
        V[[0, n - 1]] = 0
        descs.append(ClothDesc(n_vertices=n * n, springs=sp, pinned=np.array([0, n - 1], np.int32), cg_max_iter=200,
                               cg_tol=1e-5))
        Xs.append(X)
        Vs.append(V)
    return descs, np.concatenate(Xs), np.concatenate(Vs)


def stepped(descs, X, V, steps, cfg=None):
    with ClothSolver(descs) as s:
        if cfg:
            s.set_launch_config(**cfg)
        s.set_state(X, V)
        s.step(DT, steps)
        return s.get_state(), s.launch_config()


CONFIGS = [dict(strip=1), dict(strip=1, strip_rows=3, strip_variant=3), dict(persist=0), dict(resident_max_vertices=0),
           dict(resident_vcta=512, resident_threads=128), dict(resident_fused=1), dict(gather_variant=1),
           dict(resident_max_vertices=2000, resident_vcta=2048, resident_threads=512)]


@pytest.mark.parametrize("cfg", CONFIGS, ids=lambda c: ",".join(f"{k}={v}" for k, v in c.items()))
def test_every_configuration_steps_within_tolerance(cfg):
    descs, X, V = mixed()
    (Xa, Va, _), base = stepped(descs, X, V, 15)
    (Xb, Vb, _), got = stepped(descs, X, V, 15, cfg)
    for k, v in cfg.items():
        assert got[k] == v
    assert rel(Xb, Xa) <= 1e-6 and rel(Vb, Va) <= 1e-4


def test_replanning_back_gives_the_same_bits():
    descs, X, V = mixed()
    (Xa, Va, dVa), base = stepped(descs, X, V, 10)
    with ClothSolver(descs) as s:
        s.set_state(X, V)
        s.step(DT, 3)
        s.set_launch_config(strip=1, persist=0, resident_max_vertices=0)
        s.set_launch_config(**base)
        s.set_state(X, V, np.zeros_like(X))
        s.step(DT, 10)
        Xb, Vb, dVb = s.get_state()
    assert same_bits(Xa, Xb) and same_bits(Va, Vb) and same_bits(dVa, dVb)


def test_autotune_keeps_the_state_and_matches_an_explicit_handle(tmp_path):
    descs, X, V = mixed(9)
    cache = str(tmp_path / "tune.txt")
    with ClothSolver(descs) as s:
        s.set_state(X, V)
        s.step(DT, 2)
        before = s.get_state()
        cfg, ms = s.autotune(DT, cache_path=cache)
        assert ms > 0.0
        after = s.get_state()
        for a, b in zip(before, after):
            assert same_bits(a, b)
        assert s.launch_config() == cfg
        s.step(DT, 8)
        tuned = s.get_state()
    with ClothSolver(descs) as t:
        t.set_launch_config(**cfg)
        t.set_state(*before)
        t.step(DT, 8)
        explicit = t.get_state()
    for a, b in zip(tuned, explicit):
        assert same_bits(a, b)
    # A second handle on the same cloths takes the stored choice without timing.
    with ClothSolver(descs) as u:
        u.set_state(X, V)
        cfg2, ms2 = u.autotune(DT, cache_path=cache)
    assert cfg2 == cfg and ms2 == 0.0


def test_invalid_configuration_is_refused_and_kept():
    from opencloth_gb300 import OcError

    descs, X, V = mixed()
    with ClothSolver(descs) as s:
        base = s.launch_config()
        with pytest.raises(OcError) as e:
            s.set_launch_config(resident_vcta=3000)
        assert e.value.status == 1
        assert s.launch_config() == base
    with ClothSolver(descs[:3], executor="resident") as r:
        base = r.launch_config()
        with pytest.raises(OcError) as e:
            r.set_launch_config(resident_max_vertices=100)  # the resident executor needs every cloth
        assert e.value.status == 7
        assert r.launch_config() == base
