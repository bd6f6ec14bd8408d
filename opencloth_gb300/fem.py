"""The FEM demo's block-sparse conjugate gradient on the GPU, and FEM systems to feed it.

``BsrSolver`` wraps the C ABI's ``oc_bsr_*`` entry points: a batch of block-row systems
solved with the semantics of ConjugateGradientSolver in
OpenCloth_CoRotated_Linear_FEM/OpenCloth_CoRotated_Linear_FEM/main.cpp (FEM:837-922).

``fem_system`` builds the system that demo hands its CG at the undeformed state, for
meshes of any size: the mesh of GenerateBlocks (FEM:329-386), the element stiffness of
CalculateK (FEM:240-327), the lumped masses of RecalcMassMatrix (FEM:388-405) and the
assembly of StiffnessAssembly / DynamicsAssembly (FEM:659-698, 790-831) with the
rotations at identity.  It is vectorised numpy in FP64, rounded to FP32 at the end.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _native as N
from ._native import OcError, ptr

# Material constants of the FEM demo (FEM:68-79).
NU = 0.33
YOUNG = 500000.0
DENSITY = 1000.0
MASS_DAMPING = 1.0
FLT_MAX = float(np.finfo(np.float32).max)


def tet_block_mesh(xdim: int, ydim: int, zdim: int, width=0.1, height=0.1, depth=0.1):
    """GenerateBlocks (FEM:329-386): rest positions Xi, current positions X (offset by
    0.5 in y and -zdim/2 * depth in z), tetrahedra (5 per cube, alternating) and the
    fixed flags (Xi.x < 0.01)."""
    xs, ys, zs = np.meshgrid(np.arange(xdim + 1), np.arange(ydim + 1), np.arange(zdim + 1), indexing="ij")
    Xi = np.stack([width * xs, height * zs, depth * ys], axis=-1).reshape(-1, 3).astype(np.float64)
    X = Xi.copy()
    X[:, 1] += 0.5
    X[:, 2] -= (zdim / 2.0) * depth
    fixed = (Xi[:, 0] < 0.01).astype(np.uint8)
    i, j, k = np.meshgrid(np.arange(xdim), np.arange(ydim), np.arange(zdim), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    p0 = (i * (ydim + 1) + j) * (zdim + 1) + k
    p1 = p0 + 1
    p3 = ((i + 1) * (ydim + 1) + j) * (zdim + 1) + k
    p2 = p3 + 1
    p7 = ((i + 1) * (ydim + 1) + (j + 1)) * (zdim + 1) + k
    p6 = p7 + 1
    p4 = (i * (ydim + 1) + (j + 1)) * (zdim + 1) + k
    p5 = p4 + 1
    odd = (i + j + k) % 2 == 1
    a = np.stack([np.stack(t, 1) for t in ((p1, p2, p6, p3), (p3, p6, p4, p7), (p1, p4, p6, p5), (p1, p3, p4, p0),
                                           (p1, p6, p4, p3))], 1)
    b = np.stack([np.stack(t, 1) for t in ((p2, p0, p5, p1), (p2, p7, p0, p3), (p2, p5, p7, p6), (p0, p7, p5, p4),
                                           (p2, p0, p7, p5))], 1)
    tets = np.where(odd[:, None, None], a, b).reshape(-1, 4)
    return Xi, X, tets.astype(np.int64), fixed


def _tet_shapes(xdim: int, ydim: int, zdim: int, tets: np.ndarray):
    """Every cube of the mesh has the same size, so a tetrahedron's rest shape depends
    only on its cube's parity and its place among the cube's five: the shape index of
    each tetrahedron and one representative tetrahedron of each shape."""
    ncube = xdim * ydim * zdim
    i, j, k = np.unravel_index(np.arange(ncube), (xdim, ydim, zdim))
    shape = (((i + j + k) % 2)[:, None] * 5 + np.arange(5)[None, :]).ravel()
    rep = np.array([np.argmax(shape == t) if (shape == t).any() else 0 for t in range(10)])
    return shape, rep


def element_stiffness(Xi: np.ndarray, tets: np.ndarray):
    """CalculateK (FEM:240-327): per tetrahedron the volume and the 4 x 4 blocks Ke[i][j]
    (3 x 3, first index the row as the demo uses them, FEM:666-669)."""
    d15 = YOUNG / (1.0 + NU) / (1.0 - 2 * NU)
    d16, d17, d18 = (1.0 - NU) * d15, NU * d15, YOUNG / 2 / (1.0 + NU)
    x0, x1, x2, x3 = (Xi[tets[:, c]] for c in range(4))
    e1, e2, e3 = x1 - x0, x2 - x0, x3 - x0
    vol = np.einsum("ij,ij->i", e1, np.cross(e2, e3)) / 6.0
    det = np.linalg.det(np.stack([e1, e2, e3], axis=1))
    inv = 1.0 / det
    B = np.empty((len(tets), 4, 3))
    B[:, 1, 0] = (e2[:, 2] * e3[:, 1] - e2[:, 1] * e3[:, 2]) * inv
    B[:, 2, 0] = (e1[:, 1] * e3[:, 2] - e1[:, 2] * e3[:, 1]) * inv
    B[:, 3, 0] = (e1[:, 2] * e2[:, 1] - e1[:, 1] * e2[:, 2]) * inv
    B[:, 1, 1] = (e2[:, 0] * e3[:, 2] - e2[:, 2] * e3[:, 0]) * inv
    B[:, 2, 1] = (e1[:, 2] * e3[:, 0] - e1[:, 0] * e3[:, 2]) * inv
    B[:, 3, 1] = (e1[:, 0] * e2[:, 2] - e1[:, 2] * e2[:, 0]) * inv
    B[:, 1, 2] = (e2[:, 1] * e3[:, 0] - e2[:, 0] * e3[:, 1]) * inv
    B[:, 2, 2] = (e1[:, 0] * e3[:, 1] - e1[:, 1] * e3[:, 0]) * inv
    B[:, 3, 2] = (e1[:, 1] * e2[:, 0] - e1[:, 0] * e2[:, 1]) * inv
    B[:, 0] = -B[:, 1] - B[:, 2] - B[:, 3]
    bi, bj = B[:, :, None, :], B[:, None, :, :]  # (T, 4, 1, 3) and (T, 1, 4, 3)
    b19, b20, b21 = bi[..., 0], bi[..., 1], bi[..., 2]
    b22, b23, b24 = bj[..., 0], bj[..., 1], bj[..., 2]
    Ke = np.empty((len(tets), 4, 4, 3, 3))
    Ke[..., 0, 0] = d16 * b19 * b22 + d18 * (b20 * b23 + b21 * b24)
    Ke[..., 0, 1] = d17 * b19 * b23 + d18 * (b20 * b22)
    Ke[..., 0, 2] = d17 * b19 * b24 + d18 * (b21 * b22)
    Ke[..., 1, 0] = d17 * b20 * b22 + d18 * (b19 * b23)
    Ke[..., 1, 1] = d16 * b20 * b23 + d18 * (b19 * b22 + b21 * b24)
    Ke[..., 1, 2] = d17 * b20 * b24 + d18 * (b21 * b23)
    Ke[..., 2, 0] = d17 * b21 * b22 + d18 * (b19 * b24)
    Ke[..., 2, 1] = d17 * b21 * b23 + d18 * (b20 * b24)
    Ke[..., 2, 2] = d16 * b21 * b24 + d18 * (b20 * b23 + b19 * b22)
    Ke *= vol[:, None, None, None, None]
    return vol, Ke


def fem_system(xdim: int, ydim: int, zdim: int, dt: float = 1.0 / 60.0, V=None, i_max: int = 20,
               gravity=(0.0, -9.81, 0.0), first_step: bool = False):
    """The system the FEM demo's CG receives at the undeformed state (rotations at
    identity) for a mesh of xdim x ydim x zdim cubes, with velocities V (default 0).
    Returns a dict: row_ptr, col, blocks (nnzb, 9) with m[c][r] at 3c + r, b, V, fixed,
    i_max, tolerance, tiny (the demo's FEM:132-134).

    first_step=True reproduces the demo's very first assembly: its stiffness rows are
    std::maps whose entries are created by operator[] on first use, and the vendored
    glm's default mat3 is the identity (dep/glm/glm/core/type_mat3x3.inl:54-61), so in
    the first StiffnessAssembly every block starts from I before the element blocks are
    added; from the second step on ClearStiffnessAssembly (FEM:414-422) zeroes them."""
    Xi, X, tets, fixed = tet_block_mesh(xdim, ydim, zdim)
    n = len(Xi)
    shape, rep = _tet_shapes(xdim, ydim, zdim, tets)
    vol_s, Ke_s = element_stiffness(Xi, tets[rep])
    vol = vol_s[shape]
    # StiffnessAssembly with Re = I (FEM:659-698): K[ti][tj] += Ke[i][j] for j >= i and
    # K[tj][ti] += Ke[i][j]^T for j > i.  Every contribution is one of 10 shapes x 16
    # local blocks (or a transpose), so the assembly is a sparse count matrix (entry x
    # block code) times the table of the 320 distinct blocks.
    import scipy.sparse as sps

    ii, jj = np.triu_indices(4)
    strict = ii < jj
    table = np.concatenate([Ke_s.reshape(-1, 9), np.swapaxes(Ke_s, -1, -2).reshape(-1, 9)])  # codes 0..159, 160..319
    code_up = shape[:, None] * 16 + (ii * 4 + jj)[None, :]
    code_lo = 160 + shape[:, None] * 16 + (ii * 4 + jj)[strict][None, :]
    r = np.concatenate([tets[:, ii].ravel(), tets[:, jj[strict]].ravel()])
    c = np.concatenate([tets[:, jj].ravel(), tets[:, ii[strict]].ravel()])
    code = np.concatenate([code_up.ravel(), code_lo.ravel()])
    uniq, inv = np.unique(r * n + c, return_inverse=True)
    counts = sps.csr_matrix((np.ones(len(inv)), (inv, code)), shape=(len(uniq), 320))
    K = np.asarray(counts @ table).reshape(-1, 3, 3)
    urow, ucol = uniq // n, uniq % n
    if first_step:
        K = K + np.eye(3)[None]
    row_ptr = np.concatenate([[0], np.cumsum(np.bincount(urow, minlength=n))])
    row_start = row_ptr[:-1][np.bincount(urow, minlength=n) > 0]  # every row has its diagonal block
    # F0 = -K Xi (FEM:691-694), F = m g (FEM:572-580), masses (FEM:388-405).
    mass = np.where(fixed == 1, FLT_MAX, 1.0 / n)
    mass = mass + np.bincount(tets.ravel(), weights=np.repeat(DENSITY * vol * 0.25, 4), minlength=n)
    # the element sums (F0) never see the identity start of the first assembly
    KXi = np.add.reduceat(np.einsum("kab,kb->ka", K - np.eye(3)[None] if first_step else K, Xi[ucol]), row_start)
    KX = np.add.reduceat(np.einsum("kab,kb->ka", K, X[ucol]), row_start)
    F = np.asarray(gravity)[None, :] * mass[:, None]
    Vel = np.zeros((n, 3)) if V is None else np.asarray(V, np.float64).reshape(n, 3)
    # DynamicsAssembly (FEM:790-831): A = K dt^2 + (m + dt c m) I on the diagonal,
    # b = (-K X - F0 + F) dt + V m.
    A = K * (dt * dt)
    diag = urow == ucol
    with np.errstate(over="ignore", invalid="ignore"):
        md = mass[urow[diag]] + dt * (MASS_DAMPING * mass[urow[diag]])
        A[diag, 0, 0] += md
        A[diag, 1, 1] += md
        A[diag, 2, 2] += md
        b = (-KX + KXi + F) * dt + Vel * mass[:, None]
        blocks = A.reshape(-1, 9).astype(np.float32)  # the demo's m[a][b] (row a) at 3a + b
    return {"row_ptr": row_ptr.astype(np.int32), "col": ucol.astype(np.int32), "blocks": blocks,
            "b": b.astype(np.float32), "V": Vel.astype(np.float32), "fixed": fixed, "i_max": int(i_max),
            "tolerance": 1e-3, "tiny": 1e-10}


class BsrSolver:
    """A batch of block-sparse systems solved with the FEM demo's CG (FEM:837-922).

    ``systems``: dicts (or objects) with row_ptr, col, fixed, i_max, tolerance, tiny.
    ``set_system`` takes blocks (nnzb, 9), b and V (rows, 3), concatenated over the
    systems; ``solve`` runs the CG; ``solution`` returns (V, residual).  ``executor``:
    0 (auto: systems of up to 256 rows whose blocks fit in shared memory are solved by
    one CTA each), 1 (every system streamed) or 2 (every system resident)."""

    def __init__(self, systems: Sequence, device: int = 0, use_graph: bool = True, stream: int | None = None,
                 executor: int = 0):
        self._lib = N.load()
        self._keep = []
        descs = (N.BsrDescC * len(systems))()
        for d, sysd in zip(descs, systems):
            g = sysd.get if isinstance(sysd, dict) else (lambda k, o=sysd: getattr(o, k))
            rp = np.ascontiguousarray(g("row_ptr"), np.int32)
            col = np.ascontiguousarray(g("col"), np.int32)
            fx = np.ascontiguousarray(g("fixed"), np.uint8)
            self._keep += [rp, col, fx]
            d.n_rows = len(rp) - 1
            d.nnzb = len(col)
            d.row_ptr = ptr(rp)
            d.col = ptr(col) if col.size else None
            d.fixed = ptr(fx)
            d.cg_max_iter = int(g("i_max"))
            d.tolerance = float(g("tolerance"))
            d.tiny = float(g("tiny"))
        opts = N.OptionsC()
        self._lib.oc_default_options(C.byref(opts))
        opts.device = device
        opts.use_graph = 1 if use_graph else 0
        opts.stream = stream
        opts.executor = int(executor)
        h = C.c_void_p()
        st = self._lib.oc_bsr_create(descs, len(systems), C.byref(opts), C.byref(h))
        if st != N.OC_OK:
            raise OcError(st, "oc_bsr_create")
        self._h = h
        rows, nnzb, nsys = C.c_int64(), C.c_int64(), C.c_int32()
        self._call(self._lib.oc_bsr_get_counts(self._h, C.byref(rows), C.byref(nnzb), C.byref(nsys)))
        self.n_rows, self.nnzb, self.n_systems = rows.value, nnzb.value, nsys.value

    def _call(self, st: int) -> None:
        if st != N.OC_OK:
            raise OcError(st, self._lib.oc_bsr_last_error(self._h).decode())

    def set_system(self, blocks=None, b=None, V=None) -> None:
        arrs = []
        for a, width in ((blocks, 9), (b, 3), (V, 3)):
            arrs.append(None if a is None else np.ascontiguousarray(a, np.float32).reshape(-1, width))
        self._call(self._lib.oc_bsr_set_system(self._h, *(ptr(a) for a in arrs)))

    def solve(self) -> None:
        self._call(self._lib.oc_bsr_solve(self._h))

    def synchronize(self) -> None:
        self._call(self._lib.oc_bsr_synchronize(self._h))

    def solution(self):
        x = np.empty((self.n_rows, 3), np.float32)
        r = np.empty((self.n_rows, 3), np.float32)
        self._call(self._lib.oc_bsr_get_solution(self._h, ptr(x), ptr(r)))
        return x, r

    def profile(self, n_solves: int = 1) -> dict:
        """Per kernel: total ms, launches and algorithmic bytes over n_solves un-graphed
        solves timed with CUDA events."""
        names = C.create_string_buffer(32 * 8)
        ms = np.zeros(8)
        launches = np.zeros(8, np.int64)
        byts = np.zeros(8)
        n = C.c_int32()
        self._call(self._lib.oc_bsr_profile(self._h, int(n_solves), 8, names, ptr(ms), ptr(launches), ptr(byts),
                                            C.byref(n)))
        raw = names.raw
        return {raw[32 * k: 32 * (k + 1)].split(b"\0", 1)[0].decode(): {
            "ms_total": float(ms[k]), "launches": int(launches[k]), "bytes": float(byts[k])} for k in range(n.value)}

    def launch_count(self) -> int:
        n = C.c_int64()
        self._call(self._lib.oc_bsr_get_launch_count(self._h, C.byref(n)))
        return int(n.value)

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.oc_bsr_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        self.close()
