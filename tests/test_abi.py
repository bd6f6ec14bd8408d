"""The C ABI without a GPU: the library loads, exports every declared symbol, and
rejects bad input with the documented status before any device work."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from opencloth_gb300 import SPRING_DTYPE, ClothDesc, ClothSolver, OcError, grid_cloth, grid_spring_count
from opencloth_gb300 import _native as N

INCLUDE = Path(__file__).resolve().parents[1] / "include"


def declared_symbols():
    names = set()
    for h in INCLUDE.glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(oc_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    lib = N.load()
    names = declared_symbols()
    assert "oc_create" in names and "oc_step" in names
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) <= set(N.SIGNATURES), set(names) - set(N.SIGNATURES)


def test_status_strings():
    lib = N.load()
    for code, name in N.STATUS_NAMES.items():
        assert lib.oc_status_string(code).decode() == name


@pytest.mark.parametrize("cols,rows", [(3, 3), (21, 21), (8, 128), (1025, 1025)])
def test_grid_spring_count_formula(cols, rows):
    u, v = cols, rows
    expect = v * (u - 1) + u * (v - 1) + 2 * (v - 1) * (u - 1) + v * (u - 1) + u * (v - 1)
    assert grid_spring_count(cols, rows) == expect
    if cols * rows < 5000:
        X, sp = grid_cloth(cols, rows)
        assert len(sp) == expect and X.shape == (cols * rows, 3)


def test_grid_builder_lattice_and_rest_lengths():
    X, sp = grid_cloth(5, 4, size=4.0)
    assert np.allclose(X[0], [-2, 5, 0]) and np.allclose(X[4], [2, 5, 0]) and np.allclose(X[-1], [2, 1, 0])
    d = X[sp["p1"]] - X[sp["p2"]]
    assert np.allclose(np.sqrt((d * d).sum(1)), sp["rest_length"])
    assert set(np.unique(sp["type"])) == {0, 1, 2}


def test_grid_jitter_is_seeded_and_keeps_rest_lengths():
    X1, s1 = grid_cloth(9, 9, jitter=0.01, seed=5)
    X2, s2 = grid_cloth(9, 9, jitter=0.01, seed=5)
    X3, _ = grid_cloth(9, 9, jitter=0.01, seed=6)
    X0, s0 = grid_cloth(9, 9)
    assert np.array_equal(X1, X2) and not np.array_equal(X1, X3)
    assert np.array_equal(s1, s0)  # rest lengths come from the exact lattice
    spacing = 4.0 / 8
    assert 0.002 < np.std(X1 - X0) / spacing < 0.02


def _desc(**kw):
    X, sp = grid_cloth(4, 4)
    base = dict(n_vertices=16, springs=sp, pinned=np.array([0, 3], np.int32))
    base.update(kw)
    return ClothDesc(**base)


def _status(desc):
    with pytest.raises(OcError) as e:
        ClothSolver(desc)
    return e.value.status


def test_create_rejects_out_of_range_endpoint():
    _, sp = grid_cloth(4, 4)
    sp["p2"][5] = 16
    assert _status(_desc(springs=sp)) == 2  # OC_ERR_BAD_INDEX


def test_create_rejects_negative_endpoint():
    _, sp = grid_cloth(4, 4)
    sp["p1"][0] = -1
    assert _status(_desc(springs=sp)) == 2


def test_create_rejects_self_loop():
    _, sp = grid_cloth(4, 4)
    sp["p2"][3] = sp["p1"][3]
    assert _status(_desc(springs=sp)) == 4  # OC_ERR_DEGENERATE


def test_create_rejects_non_finite_parameters():
    _, sp = grid_cloth(4, 4)
    sp["ks"][2] = np.nan
    assert _status(_desc(springs=sp)) == 3  # OC_ERR_NON_FINITE
    assert _status(_desc(gravity=(0.0, np.inf, 0.0))) == 3


def test_create_rejects_bad_pins_mass_and_sizes():
    assert _status(_desc(pinned=np.array([16], np.int32))) == 2
    assert _status(_desc(mass=np.zeros(16, np.float32))) == 1
    assert _status(_desc(mass=np.full(16, np.nan, np.float32))) == 3
    assert _status(_desc(cg_max_iter=-1)) == 1
    assert _status(_desc(n_vertices=0)) == 1


def test_create_rejects_negative_rest_length():
    _, sp = grid_cloth(4, 4)
    sp["rest_length"][1] = -0.5
    assert _status(_desc(springs=sp)) == 1


def test_null_handle_calls_fail_cleanly():
    lib = N.load()
    assert lib.oc_step(None, C.c_float(0.01), 1) == 1
    assert lib.oc_set_state(None, None, None, None) == 1
    assert lib.oc_get_stats(None, None, None, None) == 1
    lib.oc_destroy(None)


def _c_layout(struct: str, fields) -> list:
    """sizeof and offsetof of a header struct, from a probe compiled with the host C compiler."""
    import shutil
    import subprocess
    import tempfile

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    body = "".join(f'printf("%zu\\n", offsetof({struct}, {f}));' for f in fields)
    src = ('#include <stddef.h>\n#include <stdio.h>\n#include "opencloth_gb.h"\n'
           f'int main(void) {{ printf("%zu\\n", sizeof({struct})); {body} return 0; }}\n')
    with tempfile.TemporaryDirectory() as td:
        c = Path(td) / "probe.c"
        c.write_text(src)
        exe = Path(td) / "probe"
        subprocess.run([cc, f"-I{INCLUDE}", str(c), "-o", str(exe)], check=True, capture_output=True)
        out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return [int(v) for v in out.split()]


@pytest.mark.parametrize("cls,struct", [(N.ClothDescC, "oc_cloth_desc"), (N.OptionsC, "oc_options"),
                                        (N.Spring, "oc_spring"), (N.BsrDescC, "oc_bsr_desc")])
def test_ctypes_structs_match_the_header(cls, struct):
    fields = [f[0] for f in cls._fields_]
    got = _c_layout(struct, fields)
    assert got[0] == C.sizeof(cls), struct
    assert got[1:] == [getattr(cls, f).offset for f in fields], struct


def test_spring_record_layout_matches_c():
    assert SPRING_DTYPE.itemsize == C.sizeof(N.Spring) == 24


def test_create_rejects_bad_passes():
    assert _status(_desc(passes=4)) == 1  # unknown pass bit: OC_ERR_INVALID_ARGUMENT
    bad = np.eye(4, dtype=np.float32).ravel()
    bad[5] = np.nan
    assert _status(_desc(passes=1, ellipsoid=bad, ellipsoid_inv=np.eye(4).ravel())) == 3  # OC_ERR_NON_FINITE
    assert _status(_desc(passes=2, provot_ratio=-1.0)) == 1


def test_describe_detects_reference_grids():
    """Grid cloths of the reference's lattice use the stencil assembly; anything else
    (random per-spring parameters, a missing spring) the incidence gather."""
    from opencloth_gb300 import describe

    for cols, rows in ((3, 3), (6, 6), (21, 21), (9, 7), (128, 128), (1025, 65)):
        X, sp = grid_cloth(cols, rows, jitter=1e-3)
        assert describe(ClothDesc(n_vertices=cols * rows, springs=sp)) == [(cols, rows)]
    X, sp = grid_cloth(9, 7)
    odd = sp.copy()
    odd["ks"][10] = 1.0
    assert describe(ClothDesc(n_vertices=63, springs=odd)) == [(0, 0)]
    assert describe(ClothDesc(n_vertices=63, springs=np.delete(sp, 5))) == [(0, 0)]
