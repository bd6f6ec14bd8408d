"""Test infrastructure: the oracle for the implicit cloth step.

Only ``tests/``, ``bench.py`` (its CPU-baseline leg and reference arm) and
``__graft_entry__.smoke()`` may use this package, and only as the reference that results
are compared against or as the timed CPU baseline.  The product (``opencloth_gb300``) never imports it.

Two oracles:

* the *port* — ``oc_oracle.c``, a C restatement of the reference step
  (OpenCloth_Implicit/OpenCloth_Implicit/main.cpp:698-798, :308-330) in FP32 and FP64,
  built here and on any host with gcc;
* the *reference itself* — ``_ref/ref_step_f32`` / ``_ref/ref_step_f64``, the
  reference's own source compiled headless by ``build_ref.sh`` where the reference tree
  is present.  Tests pin the port to it bit for bit, and committed golden fixtures
  (``tests/golden/``) carry its outputs to hosts without it.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import struct
import subprocess
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF = HERE / "_ref"
PORT_LIB = BUILD / "liboc_oracle.so"

SPRING_DTYPE = np.dtype(
    [("p1", "<i4"), ("p2", "<i4"), ("rest_length", "<f4"), ("ks", "<f4"), ("kd", "<f4"), ("type", "<i4")]
)


def build(reference: bool = True) -> None:
    """Compile the port (always) and the reference harness (when the tree is present)."""
    BUILD.mkdir(exist_ok=True)
    srcs = [HERE / "oc_oracle.c", HERE / "oc_oracle_impl.h", HERE / "oc_coupled_impl.h", HERE / "oc_bsr_impl.h",
            HERE / "oc_oracle.h", HERE / "oc_adjoint.c", HERE / "oc_grid.c", Path(__file__)]
    if not PORT_LIB.exists() or any(s.stat().st_mtime > PORT_LIB.stat().st_mtime for s in srcs):
        tmp = PORT_LIB.with_suffix(".so.tmp")
        subprocess.run(["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                        str(HERE / "oc_oracle.c"), str(HERE / "oc_adjoint.c"), str(HERE / "oc_grid.c"), "-o", str(tmp),
                        "-lm"], check=True)
        os.replace(tmp, PORT_LIB)
    if reference:
        subprocess.run(["bash", str(HERE / "build_ref.sh")], check=True, capture_output=True)


class Params(C.Structure):
    _fields_ = [
        ("n_vertices", C.c_int32), ("n_springs", C.c_int32), ("springs", C.c_void_p), ("pinned", C.c_void_p),
        ("num_x", C.c_int32), ("mass", C.c_void_p), ("ext_force", C.c_void_p), ("gravity", C.c_float * 3),
        ("damping", C.c_float), ("i_max", C.c_int32), ("eps", C.c_float), ("dot_fp64", C.c_int32),
        ("filter_pinned", C.c_int32), ("passes", C.c_int32), ("ellipsoid", C.c_double * 16),
        ("ellipsoid_inv", C.c_double * 16), ("provot_ratio", C.c_double),
    ]

PASS_ELLIPSOID = 1
PASS_PROVOT = 2


_port = None


def port() -> C.CDLL:
    global _port
    if _port is None:
        if not PORT_LIB.exists():
            build(reference=False)
        lib = C.CDLL(str(PORT_LIB))
        P = C.POINTER(Params)
        for sfx, real in (("f32", C.c_float), ("f64", C.c_double)):
            getattr(lib, f"ocr_compute_forces_{sfx}").argtypes = [P, C.c_void_p, C.c_void_p, C.c_void_p]
            getattr(lib, f"ocr_assemble_{sfx}").argtypes = [P, real, C.c_void_p, C.c_void_p, C.c_void_p,
                                                            C.c_void_p, C.c_void_p]
            f = getattr(lib, f"ocr_step_{sfx}")
            f.argtypes = [P, real, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
            f.restype = C.c_int
            getattr(lib, f"ocr_passes_{sfx}").argtypes = [P, C.c_void_p, C.c_void_p]
            getattr(lib, f"ocr_coupled_matvec_{sfx}").argtypes = [P, real] + [C.c_void_p] * 3
            getattr(lib, f"ocr_coupled_system_{sfx}").argtypes = [P, real] + [C.c_void_p] * 6
            f = getattr(lib, f"ocr_coupled_step_{sfx}")
            f.argtypes = [P, real, C.c_int32] + [C.c_void_p] * 6
            f.restype = C.c_int
            f = getattr(lib, f"ocr_bsr_cg_{sfx}")
            f.argtypes = [C.c_int32] + [C.c_void_p] * 6 + [C.c_int32, C.c_float, C.c_int32, C.c_void_p]
            f.restype = C.c_int
        lib.ocr_adjoint_f64.argtypes = [P, C.c_double, C.c_int32] + [C.c_void_p] * 10
        lib.ocr_adjoint_f64.restype = C.c_int
        lib.ocr_grid_spring_count.argtypes = [C.c_int32, C.c_int32]
        lib.ocr_grid_spring_count.restype = C.c_int64
        lib.ocr_grid_build.argtypes = [C.c_int32, C.c_int32, C.c_float, C.c_void_p, C.c_void_p, C.c_float,
                                       C.c_uint64, C.c_void_p, C.c_void_p]
        lib.ocr_grid_build.restype = C.c_int
        _port = lib
    return _port


def grid_cloth(cols: int, rows: int, size: float = 4.0, ks=(0.75, 0.75, 0.95), kd=(-0.25, -0.25, -0.25),
               jitter: float = 0.0, seed: int = 0):
    """InitGL's cloth (IMP:497-565) on the x-y plane, row 0 on top, built by the oracle
    (oc_grid.c): ``(X, springs)`` with positions (cols*rows, 3) float32 and spring records
    in the reference's creation order; ``jitter`` is the position noise sigma as a
    fraction of the grid spacing, applied after the rest lengths are taken.  The same
    arguments give the same arrays as the library's ``grid_cloth``."""
    lib = port()
    ns = int(lib.ocr_grid_spring_count(cols, rows))
    if ns < 0:
        raise ValueError("grid_cloth needs at least 3 x 3 vertices")
    X = np.zeros((cols * rows, 3), np.float32)
    springs = np.zeros(ns, SPRING_DTYPE)
    ks_a = np.ascontiguousarray(ks, np.float32)
    kd_a = np.ascontiguousarray(kd, np.float32)
    rc = lib.ocr_grid_build(cols, rows, float(size), ks_a.ctypes.data, kd_a.ctypes.data, float(jitter),
                            seed & (2**64 - 1), X.ctypes.data, springs.ctypes.data)
    if rc != 0:
        raise ValueError("ocr_grid_build rejected its arguments")
    return X, springs


class Cloth:
    """Inputs of one cloth for the oracle (mirrors oc_cloth_desc)."""

    def __init__(self, n_vertices, springs, pinned=None, num_x=None, mass=None, ext_force=None,
                 gravity=(0.0, -0.00981, 0.0), damping=-0.125, i_max=10, eps=1e-3, passes=0, ellipsoid=None,
                 ellipsoid_inv=None, provot_ratio=1.01, ellipsoid64=None, ellipsoid_inv64=None):
        # The ellipsoid (column-major 4x4 and its inverse) as the FP32 reference holds it;
        # the FP64 flavour uses the *64 copies when given (the FP64 reference computes the
        # matrices in double), else the FP32 values widened.
        self.passes = int(passes)
        z = np.zeros(16)
        self.ellipsoid = z if ellipsoid is None else np.asarray(ellipsoid, np.float32).astype(np.float64).ravel()
        self.ellipsoid_inv = (z if ellipsoid_inv is None
                              else np.asarray(ellipsoid_inv, np.float32).astype(np.float64).ravel())
        self.ellipsoid64 = self.ellipsoid if ellipsoid64 is None else np.asarray(ellipsoid64, np.float64).ravel()
        self.ellipsoid_inv64 = (self.ellipsoid_inv if ellipsoid_inv64 is None
                                else np.asarray(ellipsoid_inv64, np.float64).ravel())
        self.provot_ratio = float(provot_ratio)
        self.n_vertices = int(n_vertices)
        self.springs = np.ascontiguousarray(springs, SPRING_DTYPE)
        self.pinned = pinned  # index array or None (then the reference pins {0, num_x})
        self.num_x = num_x
        self.mass = mass
        self.ext_force = ext_force
        self.gravity = tuple(float(g) for g in gravity)
        self.damping = float(damping)
        self.i_max = int(i_max)
        self.eps = float(eps)

    def params(self, dot_fp64: bool, filter_pinned: bool, fp64: bool = False):
        keep = []
        p = Params()
        p.n_vertices = self.n_vertices
        p.n_springs = int(self.springs.shape[0])
        p.springs = self.springs.ctypes.data if self.springs.size else None
        keep.append(self.springs)
        if self.pinned is not None:
            mask = np.zeros(self.n_vertices, np.uint8)
            mask[np.asarray(self.pinned, np.int64)] = 1
            keep.append(mask)
            p.pinned = mask.ctypes.data
        else:
            p.pinned = None
        p.num_x = -1 if self.num_x is None else int(self.num_x)
        if self.mass is not None:
            m = np.ascontiguousarray(self.mass, np.float32)
            keep.append(m)
            p.mass = m.ctypes.data
        if self.ext_force is not None:
            e = np.ascontiguousarray(self.ext_force, np.float32).reshape(-1)
            keep.append(e)
            p.ext_force = e.ctypes.data
        p.gravity[:] = self.gravity
        p.damping = self.damping
        p.i_max = self.i_max
        p.eps = self.eps
        p.dot_fp64 = 1 if dot_fp64 else 0
        p.filter_pinned = 1 if filter_pinned else 0
        p.passes = self.passes
        p.ellipsoid[:] = [float(v) for v in (self.ellipsoid64 if fp64 else self.ellipsoid)]
        p.ellipsoid_inv[:] = [float(v) for v in (self.ellipsoid_inv64 if fp64 else self.ellipsoid_inv)]
        p.provot_ratio = self.provot_ratio
        return p, keep


def port_step(cloth: Cloth, X, V, dV=None, dt=1.0 / 60.0, n_steps=1, fp64=False, dot_fp64=False,
              filter_pinned=False):
    """Run the port; returns (X, V, dV, iters[n_steps], rel_residual[n_steps])."""
    lib = port()
    real = np.float64 if fp64 else np.float32
    X = np.array(X, real).reshape(-1)
    V = np.array(V, real).reshape(-1)
    dV = np.zeros_like(X) if dV is None else np.array(dV, real).reshape(-1)
    iters = np.zeros(max(n_steps, 1), np.int32)
    rr = np.zeros(max(n_steps, 1), np.float64)
    p, keep = cloth.params(dot_fp64, filter_pinned, fp64)
    fn = lib.ocr_step_f64 if fp64 else lib.ocr_step_f32
    dtv = float(np.float32(dt))
    rc = fn(C.byref(p), dtv, int(n_steps), X.ctypes.data, V.ctypes.data, dV.ctypes.data, iters.ctypes.data,
            rr.ctypes.data)
    if rc != 0:
        raise RuntimeError("oracle port step failed")
    del keep
    return X.reshape(-1, 3), V.reshape(-1, 3), dV.reshape(-1, 3), iters[:n_steps], rr[:n_steps]


def port_passes(cloth: Cloth, X, V, passes, fp64=False):
    """The passes (bit 1 EllipsoidCollision, bit 2 ApplyProvotDynamicInverse) alone on
    copies of (X, V), with the cloth's matrices, ratio and pins."""
    lib = port()
    real = np.float64 if fp64 else np.float32
    X = np.ascontiguousarray(X, real).reshape(-1).copy()
    V = np.ascontiguousarray(V, real).reshape(-1).copy()
    p, keep = cloth.params(False, False, fp64)
    p.passes = int(passes)
    (lib.ocr_passes_f64 if fp64 else lib.ocr_passes_f32)(C.byref(p), X.ctypes.data, V.ctypes.data)
    del keep
    return X.reshape(-1, 3), V.reshape(-1, 3)


def coupled_step(cloth: Cloth, X, V, dV=None, dt=1.0 / 60.0, n_steps=1, fp64=False):
    """The COUPLED Jacobian mode: (X, V, dV, iters, rel_residual, flags) after n_steps."""
    lib = port()
    real = np.float64 if fp64 else np.float32
    X = np.ascontiguousarray(X, real).reshape(-1).copy()
    V = np.ascontiguousarray(V, real).reshape(-1).copy()
    dV = np.zeros_like(X) if dV is None else np.ascontiguousarray(dV, real).reshape(-1).copy()
    iters = np.zeros(max(n_steps, 1), np.int32)
    rr = np.zeros(max(n_steps, 1), np.float64)
    fl = np.zeros(max(n_steps, 1), np.uint32)
    p, keep = cloth.params(True, True, fp64)
    fn = lib.ocr_coupled_step_f64 if fp64 else lib.ocr_coupled_step_f32
    rc = fn(C.byref(p), float(real(dt)), int(n_steps), X.ctypes.data, V.ctypes.data, dV.ctypes.data,
            iters.ctypes.data, rr.ctypes.data, fl.ctypes.data)
    del keep
    if rc != 0:
        raise MemoryError("oracle coupled step failed")
    return X.reshape(-1, 3), V.reshape(-1, 3), dV.reshape(-1, 3), iters[:n_steps], rr[:n_steps], fl[:n_steps]


def coupled_matvec(cloth: Cloth, X, w, dt, fp64=True):
    """y = A w of the COUPLED system at positions X (no pin filter)."""
    lib = port()
    real = np.float64 if fp64 else np.float32
    X = np.ascontiguousarray(X, real).reshape(-1)
    w = np.ascontiguousarray(w, real).reshape(-1)
    y = np.zeros_like(w)
    p, keep = cloth.params(True, True, fp64)
    (lib.ocr_coupled_matvec_f64 if fp64 else lib.ocr_coupled_matvec_f32)(C.byref(p), float(real(dt)), X.ctypes.data,
                                                                         w.ctypes.data, y.ctypes.data)
    del keep
    return y.reshape(-1, 3)


def coupled_system(cloth: Cloth, X, V, dt, fp64=True):
    """(D6, P6, b) of the COUPLED system: diagonal blocks, their inverses, right-hand side."""
    lib = port()
    real = np.float64 if fp64 else np.float32
    X = np.ascontiguousarray(X, real).reshape(-1)
    V = np.ascontiguousarray(V, real).reshape(-1)
    F = port_forces(cloth, X, V, fp64).reshape(-1).astype(real)
    D6 = np.zeros(6 * cloth.n_vertices, real)
    P6 = np.zeros_like(D6)
    b = np.zeros(3 * cloth.n_vertices, real)
    p, keep = cloth.params(True, True, fp64)
    (lib.ocr_coupled_system_f64 if fp64 else lib.ocr_coupled_system_f32)(
        C.byref(p), float(real(dt)), X.ctypes.data, V.ctypes.data, F.ctypes.data, D6.ctypes.data, P6.ctypes.data,
        b.ctypes.data)
    del keep
    return D6.reshape(-1, 6), P6.reshape(-1, 6), b.reshape(-1, 3)


class BsrSystem:
    """One block-sparse system of the FEM demo's CG (FEM:837-922): block rows in CSR
    (ascending columns), blocks (nnzb, 9) float32 with m[c][r] at 3c + r, b and the warm
    start V (n, 3), fixed flags, i_max, tolerance and tiny."""

    def __init__(self, row_ptr, col, blocks, b, V, fixed, i_max=20, tolerance=1e-3, tiny=1e-10):
        self.row_ptr = np.ascontiguousarray(row_ptr, np.int32)
        self.col = np.ascontiguousarray(col, np.int32)
        self.blocks = np.ascontiguousarray(blocks, np.float32).reshape(-1, 9)
        self.b = np.ascontiguousarray(b, np.float32).reshape(-1, 3)
        self.V = np.ascontiguousarray(V, np.float32).reshape(-1, 3)
        self.fixed = np.ascontiguousarray(fixed, np.uint8)
        self.i_max = int(i_max)
        self.tolerance = float(np.float32(tolerance))
        self.tiny = float(np.float32(tiny))

    @property
    def n(self) -> int:
        return len(self.row_ptr) - 1

    def to_bytes(self) -> bytes:
        head = b"OCB1" + np.array([self.n, len(self.col), self.i_max], np.int32).tobytes() + \
            np.array([self.tolerance, self.tiny], np.float32).tobytes()
        return b"".join([head, self.row_ptr.tobytes(), self.col.tobytes(), self.blocks.tobytes(), self.b.tobytes(),
                         self.V.tobytes(), self.fixed.tobytes()])

    @classmethod
    def from_bytes(cls, data: bytes) -> "BsrSystem":
        n, nnzb, i_max = np.frombuffer(data, np.int32, 3, 4)
        tol, tiny = np.frombuffer(data, np.float32, 2, 16)
        o = 24
        rp = np.frombuffer(data, np.int32, n + 1, o); o += 4 * (n + 1)
        col = np.frombuffer(data, np.int32, nnzb, o); o += 4 * nnzb
        blk = np.frombuffer(data, np.float32, 9 * nnzb, o); o += 36 * nnzb
        b = np.frombuffer(data, np.float32, 3 * n, o); o += 12 * n
        V = np.frombuffer(data, np.float32, 3 * n, o); o += 12 * n
        fixed = np.frombuffer(data, np.uint8, n, o)
        return cls(rp, col, blk, b, V, fixed, int(i_max), float(tol), float(tiny))


def bsr_cg(sys_: BsrSystem, fp64=False, dot_fp64=False):
    """The restatement of ConjugateGradientSolver (FEM:837-922): (V, residual)."""
    lib = port()
    real = np.float64 if fp64 else np.float32
    x = sys_.V.astype(real).reshape(-1).copy()
    b = sys_.b.astype(real).reshape(-1)
    res = np.zeros_like(x)
    fn = lib.ocr_bsr_cg_f64 if fp64 else lib.ocr_bsr_cg_f32
    rc = fn(sys_.n, sys_.row_ptr.ctypes.data, sys_.col.ctypes.data, sys_.blocks.ctypes.data, b.ctypes.data,
            x.ctypes.data, sys_.fixed.ctypes.data, sys_.i_max, sys_.tiny, 1 if dot_fp64 else 0, res.ctypes.data)
    if rc != 0:
        raise MemoryError("oracle bsr cg failed")
    return x.reshape(-1, 3), res.reshape(-1, 3)


def fem_binary(fp64: bool = False) -> Path:
    return REF / ("fem_step_f64" if fp64 else "fem_step_f32")


def fem_available() -> bool:
    return fem_binary().exists() and fem_binary(True).exists()


def _fem_env(dims):
    return dict(os.environ, OC_FEM_X=str(int(dims[0])), OC_FEM_Y=str(int(dims[1])), OC_FEM_Z=str(int(dims[2])))


def fem_ref_system(steps: int, dims=(10, 3, 3)):
    """The reference FEM demo (mesh of dims cubes, InitGL FEM:424-426) after `steps`
    steps: the system its CG receives in the next step, and the CG's own (V, residual)."""
    with tempfile.TemporaryDirectory() as td:
        sp, op = os.path.join(td, "sys.bin"), os.path.join(td, "sol.bin")
        subprocess.run([str(fem_binary()), "--system", str(int(steps)), sp, op], env=_fem_env(dims), check=True,
                       capture_output=True)
        sys_ = BsrSystem.from_bytes(open(sp, "rb").read())
        sol = np.fromfile(op, np.float32)
    n3 = 3 * sys_.n
    return sys_, sol[:n3].reshape(-1, 3), sol[n3:].reshape(-1, 3)


def fem_ref_solve(sys_: BsrSystem, fp64: bool = False, timed: bool = False):
    """The reference's ConjugateGradientSolver run on `sys_`: (V, residual[, seconds])."""
    with tempfile.TemporaryDirectory() as td:
        sp, op = os.path.join(td, "sys.bin"), os.path.join(td, "sol.bin")
        open(sp, "wb").write(sys_.to_bytes())
        r = subprocess.run([str(fem_binary(fp64)), "--solve", sp, op] + (["--time"] if timed else []), check=True,
                           capture_output=True, text=True)
        sol = np.fromfile(op, np.float64 if fp64 else np.float32)
    n3 = 3 * sys_.n
    out = (sol[:n3].reshape(-1, 3), sol[n3:].reshape(-1, 3))
    if timed:
        out = out + (json.loads(r.stdout.strip().splitlines()[-1])["seconds"],)
    return out


def ref_pick(X, point, radius=0.1) -> int:
    """OnMouseDown's picking loop, IMP:399-405: the first i with
    glm::distance(X[i], pt) < 0.1 (FP32 length of pt - X[i], squares summed left to
    right; compared in double, as the literal 0.1 is), else -1."""
    X = np.asarray(X, np.float32).reshape(-1, 3)
    p = np.asarray(point, np.float32).reshape(3)
    d = p[None, :] - X
    sq = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
    dist = np.sqrt(sq, dtype=np.float32)
    hit = np.nonzero(dist.astype(np.float64) < float(radius))[0]
    return int(hit[0]) if hit.size else -1


def ref_drag(X, V, index, delta):
    """OnMouseMove's drag of the selected vertex, IMP:433-438, on copies of (X, V):
    V = 0; X.x += dx; X.y += dy only if the result stays > 0; X.z += dz (FP32)."""
    X = np.array(X, np.float32).reshape(-1, 3)
    V = np.array(V, np.float32).reshape(-1, 3)
    d = np.asarray(delta, np.float32)
    V[index] = 0.0
    X[index, 0] = np.float32(X[index, 0] + d[0])
    ny = np.float32(X[index, 1] + d[1])
    if ny > 0:
        X[index, 1] = ny
    X[index, 2] = np.float32(X[index, 2] + d[2])
    return X, V


def port_forces(cloth: Cloth, X, V, fp64=False):
    lib = port()
    real = np.float64 if fp64 else np.float32
    X = np.ascontiguousarray(X, real).reshape(-1)
    V = np.ascontiguousarray(V, real).reshape(-1)
    F = np.zeros_like(X)
    p, keep = cloth.params(False, False)
    (lib.ocr_compute_forces_f64 if fp64 else lib.ocr_compute_forces_f32)(C.byref(p), X.ctypes.data,
                                                                         V.ctypes.data, F.ctypes.data)
    del keep
    return F.reshape(-1, 3)


def port_assemble(cloth: Cloth, X, V, dt, fp64=False):
    """(F, A as (N,3,3) [column][row], b)."""
    lib = port()
    real = np.float64 if fp64 else np.float32
    X = np.ascontiguousarray(X, real).reshape(-1)
    V = np.ascontiguousarray(V, real).reshape(-1)
    F = port_forces(cloth, X, V, fp64).reshape(-1).astype(real)
    A9 = np.zeros(9 * cloth.n_vertices, real)
    b = np.zeros(3 * cloth.n_vertices, real)
    p, keep = cloth.params(False, False)
    (lib.ocr_assemble_f64 if fp64 else lib.ocr_assemble_f32)(C.byref(p), float(np.float32(dt)), X.ctypes.data,
                                                             V.ctypes.data, F.ctypes.data, A9.ctypes.data,
                                                             b.ctypes.data)
    del keep
    return F.reshape(-1, 3), A9.reshape(-1, 3, 3), b.reshape(-1, 3)


# ---- the reference itself, built headless --------------------------------------------

def ref_binary(fp64: bool = False) -> Path:
    return REF / ("ref_step_f64" if fp64 else "ref_step_f32")


def ref_available() -> bool:
    b = ref_binary()
    if not b.exists():
        return False
    try:
        env = dict(os.environ, OC_NUMX="2", OC_NUMY="2")
        with tempfile.TemporaryDirectory() as td:
            r = subprocess.run([str(b), "--topology", os.path.join(td, "t.bin")], env=env, capture_output=True,
                               timeout=30)
        return r.returncode == 0
    except OSError:
        return False


def _ref_env(num_x, num_y, i_max, eps, passes=0):
    return dict(os.environ, OC_NUMX=str(num_x), OC_NUMY=str(num_y), OC_IMAX=str(int(i_max)),
                OC_EPS="%.17g" % float(np.float32(eps)), OC_PASSES=str(int(passes)))


def ref_ellipsoid(fp64: bool = False):
    """The reference's ellipsoid matrix and its inverse (16 reals each, column-major),
    from the FP32 build (float32) or the FP64 build (float64)."""
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "ell.bin")
        subprocess.run([str(ref_binary(fp64)), "--ellipsoid", out], env=_ref_env(20, 20, 10, 1e-3), check=True,
                       capture_output=True)
        b = np.fromfile(out, np.float64 if fp64 else np.float32)
    return b[:16].copy(), b[16:32].copy()


def ref_topology(num_x: int, num_y: int):
    """InitGL()'s springs and positions for a (num_x+1) x (num_y+1) grid."""
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "topo.bin")
        subprocess.run([str(ref_binary()), "--topology", out], env=_ref_env(num_x, num_y, 10, 1e-3), check=True,
                       capture_output=True)
        b = open(out, "rb").read()
    n, s = struct.unpack_from("<ii", b, 0)
    X = np.frombuffer(b, np.float32, 3 * n, 8).reshape(n, 3).copy()
    sp = np.frombuffer(b, SPRING_DTYPE, s, 8 + 12 * n).copy()
    return X, sp


def ref_run(cloth: Cloth, num_x: int, num_y: int, X, V, dV=None, dt=1.0 / 60.0, snaps=(1,), fp64=False,
            timed=False):
    """Step the reference itself; returns {step: (X, V, dV)} (and seconds if timed)."""
    n = cloth.n_vertices
    assert n == (num_x + 1) * (num_y + 1)
    X = np.ascontiguousarray(X, np.float32).reshape(-1)
    V = np.ascontiguousarray(V, np.float32).reshape(-1)
    dV = np.zeros_like(X) if dV is None else np.ascontiguousarray(dV, np.float32).reshape(-1)
    snaps = sorted(int(s) for s in snaps)
    g = cloth.gravity
    hdr = b"OCI1" + struct.pack("<5i", n, cloth.springs.shape[0], num_x, num_y, cloth.i_max)
    hdr += struct.pack("<5f", cloth.eps, dt, g[0], g[1], g[2]) + struct.pack("<i", len(snaps))
    blob = hdr + np.asarray(snaps, np.int32).tobytes() + X.tobytes() + V.tobytes() + dV.tobytes()
    blob += cloth.springs.tobytes()
    with tempfile.TemporaryDirectory() as td:
        inp, out = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        open(inp, "wb").write(blob)
        cmd = [str(ref_binary(fp64)), inp, out] + (["--time"] if timed else [])
        r = subprocess.run(cmd, env=_ref_env(num_x, num_y, cloth.i_max, cloth.eps, cloth.passes), capture_output=True,
                           text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference run failed: {r.stderr}")
        b = open(out, "rb").read()
    assert b[:4] == b"OCO1"
    rsize, nsnap = struct.unpack_from("<ii", b, 4)
    dtype = np.float64 if rsize == 8 else np.float32
    off = 12
    res = {}
    for _ in range(nsnap):
        (step,) = struct.unpack_from("<i", b, off)
        off += 4
        arrs = []
        for _k in range(3):
            arrs.append(np.frombuffer(b, dtype, 3 * n, off).reshape(n, 3).copy())
            off += 3 * n * rsize
        res[step] = tuple(arrs)
    if timed:
        import json
        return res, json.loads(r.stdout.strip().splitlines()[-1])["seconds"]
    return res


def port_adjoint(cloth: Cloth, X0, V0, gX_T, gV_T=None, dt=1.0 / 60.0, n_steps=1):
    """FP64 adjoint (pin filter on).  Returns dict with X_T, V_T, gX0, gV0, gKs, gKd, gExt."""
    lib = port()
    n3 = 3 * cloth.n_vertices
    X0 = np.ascontiguousarray(X0, np.float64).reshape(-1)
    V0 = np.ascontiguousarray(V0, np.float64).reshape(-1)
    gX_T = np.ascontiguousarray(gX_T, np.float64).reshape(-1)
    gV = None if gV_T is None else np.ascontiguousarray(gV_T, np.float64).reshape(-1)
    out = {k: np.zeros(n3) for k in ("X_T", "V_T", "gX0", "gV0", "gExt")}
    out["gKs"] = np.zeros(len(cloth.springs))
    out["gKd"] = np.zeros(len(cloth.springs))
    p, keep = cloth.params(True, True)
    rc = lib.ocr_adjoint_f64(C.byref(p), float(np.float32(dt)), int(n_steps), X0.ctypes.data, V0.ctypes.data,
                             gX_T.ctypes.data, None if gV is None else gV.ctypes.data, out["X_T"].ctypes.data,
                             out["V_T"].ctypes.data, out["gX0"].ctypes.data, out["gV0"].ctypes.data,
                             out["gKs"].ctypes.data, out["gKd"].ctypes.data, out["gExt"].ctypes.data)
    del keep
    if rc != 0:
        raise RuntimeError("oracle adjoint failed")
    for k in ("X_T", "V_T", "gX0", "gV0", "gExt"):
        out[k] = out[k].reshape(-1, 3)
    return out
