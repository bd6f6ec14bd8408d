"""Host-side interface of the GB300 implicit cloth step.

Two layers over the C ABI (include/opencloth_gb.h):

* ``ClothSolver`` — a handle over one or many cloths (a ragged batch), with state
  transfer, stepping, statistics and the debug entry points.
* ``ImplicitCloth`` — the reference's own interface for one cloth
  (OpenCloth_Implicit/OpenCloth_Implicit/main.cpp): arrays ``X``, ``V``, ``springs``
  and the functions ``AddSpring`` (IMP:370), ``ComputeForces`` (IMP:698),
  ``IntegrateImplicit`` (IMP:775) and ``StepPhysics`` (IMP:873), operating on host
  arrays the caller may edit between steps (IMP:439-444).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np

from . import _native as N
from ._native import SPRING_DTYPE, OcError, ptr

STRUCTURAL_SPRING, SHEAR_SPRING, BEND_SPRING = 0, 1, 2
DEFAULT_DAMPING = -0.125  # IMP:104
DEFAULT_GRAVITY = (0.0, -0.00981, 0.0)  # IMP:108

_EXECUTORS = {"auto": N.EXEC_AUTO, "streamed": N.EXEC_STREAMED, "resident": N.EXEC_RESIDENT,
              "plain": N.EXEC_PLAIN}


def _check(lib, status: int, handle=None, what: str = "") -> None:
    if status != N.OC_OK:
        msg = lib.oc_last_error(handle).decode() if handle else what
        raise OcError(status, msg or what)


@dataclass
class ClothDesc:
    """One cloth: springs (``SPRING_DTYPE`` records) over ``n_vertices`` vertices."""

    n_vertices: int
    springs: np.ndarray
    mass: np.ndarray | None = None
    pinned: np.ndarray | None = None
    ext_force: np.ndarray | None = None
    gravity: tuple = DEFAULT_GRAVITY
    velocity_damping: float = DEFAULT_DAMPING
    cg_max_iter: int = 10  # IMP:128
    cg_tol: float = 1e-3  # IMP:126
    jacobian_mode: int = N.JAC_REFERENCE
    # Passes after the update (PASS_ELLIPSOID | PASS_PROVOT), StepPhysics' order
    # (IMP:873-880).  The ellipsoid: object -> world 4x4 and its inverse, 16 floats
    # column-major (m[c][r] at 4c + r, glm's layout); ``reference_ellipsoid()`` builds them.
    passes: int = 0
    ellipsoid: np.ndarray | None = None
    ellipsoid_inv: np.ndarray | None = None
    provot_ratio: float = 1.01  # IMP:808
    _keep: list = field(default_factory=list, repr=False)

    def to_c(self) -> N.ClothDescC:
        sp = np.ascontiguousarray(self.springs, dtype=SPRING_DTYPE)
        mass = None if self.mass is None else np.ascontiguousarray(self.mass, dtype=np.float32)
        pinned = None if self.pinned is None else np.ascontiguousarray(self.pinned, dtype=np.int32)
        ext = None if self.ext_force is None else np.ascontiguousarray(self.ext_force, dtype=np.float32)
        self._keep = [sp, mass, pinned, ext]
        d = N.ClothDescC()
        d.n_vertices = int(self.n_vertices)
        d.n_springs = int(sp.shape[0])
        d.springs = ptr(sp) if sp.size else None
        d.mass = ptr(mass)
        d.pinned = ptr(pinned) if pinned is not None and pinned.size else None
        d.n_pinned = 0 if pinned is None else int(pinned.size)
        d.ext_force = ptr(ext)
        d.gravity[:] = [float(g) for g in self.gravity]
        d.velocity_damping = float(self.velocity_damping)
        d.cg_max_iter = int(self.cg_max_iter)
        d.cg_tol = float(self.cg_tol)
        d.jacobian_mode = int(self.jacobian_mode)
        d.passes = int(self.passes)
        if self.ellipsoid is not None:
            d.ellipsoid[:] = [float(v) for v in np.asarray(self.ellipsoid, np.float32).ravel()]
            inv = self.ellipsoid_inv
            if inv is None:
                inv = np.linalg.inv(column_major(self.ellipsoid).astype(np.float64)).astype(np.float32).T
            d.ellipsoid_inv[:] = [float(v) for v in np.asarray(inv, np.float32).ravel()]
        d.provot_ratio = float(self.provot_ratio)
        return d


def column_major(m) -> np.ndarray:
    """16 column-major floats -> the 4x4 matrix they hold (row index first)."""
    return np.asarray(m, np.float32).reshape(4, 4).T


def reference_ellipsoid():
    """The reference's ellipsoid (InitGL, IMP:583-586): translate (0, 2, 0), rotate 45
    degrees about x, scale (1, 1, 0.5), and its inverse; 16 floats each, column-major.
    Computed in float64 and rounded, so an element may differ from glm's FP32 product by
    an ulp."""
    c, s_ = np.cos(np.radians(45.0)), np.sin(np.radians(45.0))
    T = np.eye(4)
    T[1, 3] = 2.0
    R = np.array([[1, 0, 0, 0], [0, c, -s_, 0], [0, s_, c, 0], [0, 0, 0, 1]], np.float64)
    S = np.diag([1.0, 1.0, 0.5, 1.0])
    M = T @ R @ S
    return (M.T.ravel().astype(np.float32), np.linalg.inv(M).T.ravel().astype(np.float32))


def describe(descs) -> list:
    """Per cloth, (cols, rows) of the grid whose stencil the step uses for it, or (0, 0)
    for the general incidence gather (host only: no device needed)."""
    descs = [descs] if isinstance(descs, ClothDesc) else list(descs)
    lib = N.load()
    arr = (N.ClothDescC * len(descs))(*[d.to_c() for d in descs])
    cols = np.zeros(len(descs), np.int32)
    rows = np.zeros(len(descs), np.int32)
    _check(lib, lib.oc_describe_instances(arr, len(descs), ptr(cols), ptr(rows)), what="oc_describe_instances")
    return list(zip(cols.tolist(), rows.tolist()))


def grid_spring_count(cols: int, rows: int) -> int:
    lib = N.load()
    n = C.c_int32()
    _check(lib, lib.oc_grid_spring_count(cols, rows, C.byref(n)), what="oc_grid_spring_count")
    return int(n.value)


def grid_cloth(cols: int, rows: int, size: float = 4.0, ks=(0.75, 0.75, 0.95), kd=(-0.25, -0.25, -0.25),
               jitter: float = 0.0, seed: int = 0):
    """The reference's cloth (InitGL, IMP:497-565) on the x-y plane, row 0 on top.

    Returns ``(X, springs)``: positions (cols*rows, 3) float32 and spring records in
    the reference's creation order.  ``jitter`` is the position noise sigma as a
    fraction of the grid spacing, applied after rest lengths are taken.
    """
    lib = N.load()
    ns = grid_spring_count(cols, rows)
    X = np.zeros((cols * rows, 3), np.float32)
    springs = np.zeros(ns, SPRING_DTYPE)
    ks_a = np.asarray(ks, np.float32)
    kd_a = np.asarray(kd, np.float32)
    _check(lib, lib.oc_grid_build(cols, rows, float(size), ptr(ks_a), ptr(kd_a), float(jitter),
                                  C.c_uint64(seed & (2**64 - 1)), ptr(X), ptr(springs)), what="oc_grid_build")
    return X, springs


def grid_pins(cols: int) -> np.ndarray:
    """The reference's hard-coded pins, vertices 0 and numX (IMP:705, IMP:730-732)."""
    return np.array([0, cols - 1], np.int32)


class ClothSolver:
    """A solver handle over one cloth or a ragged batch of cloths."""

    def __init__(self, descs: ClothDesc | Sequence[ClothDesc], executor: str = "auto", device: int = 0,
                 use_graph: bool = True, stream: int | None = None, vertices_per_thread: int = 0):
        self._lib = N.load()
        if isinstance(descs, ClothDesc):
            descs = [descs]
        self.descs = list(descs)
        arr = (N.ClothDescC * len(self.descs))(*[d.to_c() for d in self.descs])
        opts = N.OptionsC()
        self._lib.oc_default_options(C.byref(opts))
        opts.executor = _EXECUTORS[executor]
        opts.device = device
        opts.stream = stream
        opts.use_graph = 1 if use_graph else 0
        opts.vertices_per_thread = vertices_per_thread
        h = C.c_void_p()
        st = self._lib.oc_create(arr, len(self.descs), C.byref(opts), C.byref(h))
        if st != N.OC_OK:
            raise OcError(st, "oc_create failed (details on stderr)")
        self._h = h
        nv, ns, ni = C.c_int64(), C.c_int64(), C.c_int32()
        self._call(self._lib.oc_get_counts(self._h, C.byref(nv), C.byref(ns), C.byref(ni)))
        self.n_vertices, self.n_springs, self.n_instances = nv.value, ns.value, ni.value
        self.offsets = np.zeros(self.n_instances + 1, np.int64)
        self._call(self._lib.oc_get_vertex_offsets(self._h, ptr(self.offsets)))

    def _call(self, status: int) -> None:
        _check(self._lib, status, self._h)

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.oc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _vec(self, a) -> np.ndarray | None:
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=np.float32).reshape(-1)
        if a.size != 3 * self.n_vertices:
            raise ValueError(f"expected {3 * self.n_vertices} floats, got {a.size}")
        return a

    def set_state(self, X=None, V=None, dV=None) -> None:
        X, V, dV = self._vec(X), self._vec(V), self._vec(dV)
        self._call(self._lib.oc_set_state(self._h, ptr(X), ptr(V), ptr(dV)))

    def get_state(self):
        X = np.empty((self.n_vertices, 3), np.float32)
        V = np.empty_like(X)
        dV = np.empty_like(X)
        self._call(self._lib.oc_get_state(self._h, ptr(X), ptr(V), ptr(dV)))
        return X, V, dV

    def get_state_into(self, X=None, V=None, dV=None) -> None:
        """Read the state into caller-owned contiguous float32 arrays (any may be None)."""
        for a in (X, V, dV):
            if a is not None and (a.dtype != np.float32 or not a.flags.c_contiguous or a.size != 3 * self.n_vertices):
                raise ValueError("get_state_into needs contiguous float32 arrays of 3 * n_vertices")
        self._call(self._lib.oc_get_state(self._h, ptr(X), ptr(V), ptr(dV)))

    def set_state_device(self, X=0, V=0, dV=0) -> None:
        """Device pointers (ints) to packed float triples; 0 leaves an array unchanged."""
        self._call(self._lib.oc_set_state_device(self._h, X or None, V or None, dV or None))

    def get_state_device(self, X=0, V=0, dV=0) -> None:
        self._call(self._lib.oc_get_state_device(self._h, X or None, V or None, dV or None))

    def step(self, dt: float, n_steps: int = 1) -> None:
        self._call(self._lib.oc_step(self._h, float(dt), int(n_steps)))

    def step_host(self, X, V, dt: float, n_steps: int = 1) -> None:
        """StepPhysics on host arrays: X and V (contiguous float32, 3 per vertex; either may
        be None) are copied in, stepped n_steps times and written back in place."""
        for a in (X, V):
            if a is not None and (a.dtype != np.float32 or not a.flags.c_contiguous or a.size != 3 * self.n_vertices):
                raise ValueError("step_host needs contiguous float32 arrays of 3 * n_vertices")
        self._call(self._lib.oc_step_host(self._h, float(dt), int(n_steps), ptr(X), ptr(V)))

    def synchronize(self) -> None:
        self._call(self._lib.oc_synchronize(self._h))

    def set_passes(self, passes: int, instance: int = -1) -> None:
        """Passes after the update (PASS_* bits) of one cloth, or of all (-1)."""
        self._call(self._lib.oc_set_passes(self._h, int(instance), int(passes)))

    def pick_vertex(self, point, radius: float = 0.1, instance: int = 0) -> int:
        """The reference's picking (IMP:399-405): lowest index of cloth ``instance`` within
        ``radius`` of ``point``, or -1."""
        p = np.ascontiguousarray(point, np.float32).reshape(3)
        out = C.c_int32()
        self._call(self._lib.oc_pick_vertex(self._h, int(instance), ptr(p), float(radius), C.byref(out)))
        return int(out.value)

    def drag_vertex(self, index: int, delta, instance: int = 0) -> None:
        """The reference's drag (IMP:433-438): V = 0, X += delta, y kept above 0."""
        d = np.ascontiguousarray(delta, np.float32).reshape(3)
        self._call(self._lib.oc_drag_vertex(self._h, int(instance), int(index), ptr(d)))

    def set_vertices(self, indices, X=None, V=None) -> None:
        """Overwrite positions and/or velocities of the given (handle-global) vertices."""
        idx = np.ascontiguousarray(indices, np.int64).reshape(-1)
        Xa = None if X is None else np.ascontiguousarray(X, np.float32).reshape(-1, 3)
        Va = None if V is None else np.ascontiguousarray(V, np.float32).reshape(-1, 3)
        for a in (Xa, Va):
            if a is not None and len(a) != len(idx):
                raise ValueError("one position / velocity triple per index")
        self._call(self._lib.oc_set_vertices(self._h, len(idx), ptr(idx), ptr(Xa), ptr(Va)))

    def set_pins(self, pins, instance: int = 0) -> None:
        """Replace the pin set of cloth ``instance`` (instance-local indices)."""
        p = np.ascontiguousarray(pins, np.int32).reshape(-1)
        self._call(self._lib.oc_set_pins(self._h, int(instance), ptr(p) if p.size else None, int(p.size)))

    def apply_passes(self, passes: int) -> None:
        """Run the passes once on the current state, no step (EllipsoidCollision,
        ApplyProvotDynamicInverse called on their own)."""
        self._call(self._lib.oc_apply_passes(self._h, int(passes)))

    def stats(self):
        it = np.zeros(self.n_instances, np.int32)
        rr = np.zeros(self.n_instances, np.float64)
        fl = np.zeros(self.n_instances, np.uint32)
        self._call(self._lib.oc_get_stats(self._h, ptr(it), ptr(rr), ptr(fl)))
        return it, rr, fl

    # ---- differentiation ---------------------------------------------------------
    def set_spring_params(self, ks=None, kd=None) -> None:
        """Per-spring Ks / Kd over all springs of the handle (instance by instance)."""
        ks = None if ks is None else np.ascontiguousarray(ks, np.float32).reshape(-1)
        kd = None if kd is None else np.ascontiguousarray(kd, np.float32).reshape(-1)
        for a in (ks, kd):
            if a is not None and a.size != self.n_springs:
                raise ValueError(f"expected {self.n_springs} values")
        self._call(self._lib.oc_set_spring_params(self._h, ptr(ks), ptr(kd)))

    def set_ext_force(self, ext) -> None:
        """Constant per-vertex external force (3 floats per vertex)."""
        self._call(self._lib.oc_set_ext_force(self._h, ptr(self._vec(ext))))

    def tape_forward(self, dt: float, n_steps: int, checkpoint_every: int = 0, budget_bytes: int = 0,
                     intervals=None) -> None:
        """Run n_steps taped for tape_backward.  intervals: every cloth's checkpoint
        interval on the replay tape (oc_tape_forward_intervals); otherwise the tape and
        the intervals follow checkpoint_every and budget_bytes (oc_tape_forward)."""
        if intervals is not None:
            ev = np.ascontiguousarray(np.broadcast_to(np.asarray(intervals, np.int32), (self.n_instances,)))
            self._call(self._lib.oc_tape_forward_intervals(self._h, float(dt), int(n_steps), ptr(ev)))
            return
        self._call(self._lib.oc_tape_forward(self._h, float(dt), int(n_steps), int(checkpoint_every),
                                             int(budget_bytes)))

    def tape_layout(self):
        """The last tape's kind ("replay" or "recompute") and every cloth's interval."""
        kind = C.c_int32()
        ev = np.zeros(self.n_instances, np.int32)
        self._call(self._lib.oc_tape_layout(self._h, C.byref(kind), ptr(ev)))
        return ("replay", "recompute")[kind.value], ev

    GRADIENTS = ("dX0", "dV0", "dKs", "dKd", "dext")

    def tape_backward(self, dL_dX, dL_dV=None, want=GRADIENTS) -> dict:
        """Gradients of a loss of the final state with respect to the initial state, the
        per-spring Ks / Kd and the constant external force; `want` names the ones copied
        out (the reverse pass computes all of them either way)."""
        gX = self._vec(dL_dX)
        gV = self._vec(dL_dV)
        out = {}
        for k in want:
            out[k] = np.zeros(self.n_springs if k in ("dKs", "dKd") else (self.n_vertices, 3), np.float32)
        p = {k: (ptr(out[k]) if k in out else None) for k in self.GRADIENTS}
        self._call(self._lib.oc_tape_backward(self._h, ptr(gX), ptr(gV), p["dX0"], p["dV0"], p["dKs"], p["dKd"],
                                              p["dext"]))
        return out

    def set_tape_mode(self, displacement: bool) -> None:
        """Taped forward in the displacement mode (start positions + FP32 displacement,
        precise elongations) or in positions (the step itself)."""
        self._call(self._lib.oc_set_tape_mode(self._h, 1 if displacement else 0))

    def tape_displacement(self) -> np.ndarray:
        """The final displacement of the last displacement-mode taped forward."""
        u = np.empty((self.n_vertices, 3), np.float32)
        self._call(self._lib.oc_tape_displacement(self._h, ptr(u)))
        return u

    def tape_info(self):
        every, nbytes = C.c_int32(), C.c_int64()
        self._call(self._lib.oc_tape_info(self._h, C.byref(every), C.byref(nbytes)))
        return int(every.value), int(nbytes.value)

    def launch_config(self) -> dict:
        """The handle's launch configuration (oc_launch_config) as a dict."""
        c = N.LaunchConfigC()
        self._call(self._lib.oc_get_launch_config(self._h, C.byref(c)))
        return {name: int(getattr(c, name)) for name, _ in N.LaunchConfigC._fields_}

    def set_launch_config(self, **fields) -> None:
        """Change fields of the launch configuration (re-plans the handle's launches)."""
        cfg = self.launch_config()
        unknown = set(fields) - set(cfg)
        if unknown:
            raise KeyError(f"unknown launch configuration fields: {sorted(unknown)}")
        cfg.update(fields)
        c = N.LaunchConfigC(**cfg)
        self._call(self._lib.oc_set_launch_config(self._h, C.byref(c)))

    def autotune(self, dt: float, cache_path: str | None = None, use_cache: bool = True, store: bool = True):
        """Time candidate launch configurations on the current state (which is kept) and
        keep the fastest; returns (configuration dict, measured ms per step, 0 when it came
        from the cache)."""
        c = N.LaunchConfigC()
        ms = C.c_double()
        flags = (N.TUNE_USE_CACHE if use_cache else 0) | (N.TUNE_STORE if store else 0)
        path = cache_path.encode() if cache_path else None
        self._call(self._lib.oc_autotune(self._h, float(dt), path, flags, C.byref(c), C.byref(ms)))
        return {name: int(getattr(c, name)) for name, _ in N.LaunchConfigC._fields_}, float(ms.value)

    def tune_key(self) -> str:
        buf = C.create_string_buffer(256)
        self._call(self._lib.oc_tune_key_of(self._h, buf, 256))
        return buf.value.decode()

    def launch_count(self) -> int:
        n = C.c_int64()
        self._call(self._lib.oc_get_launch_count(self._h, C.byref(n)))
        return int(n.value)

    def compute_forces(self) -> np.ndarray:
        F = np.empty((self.n_vertices, 3), np.float32)
        self._call(self._lib.oc_compute_forces(self._h, ptr(F)))
        return F

    def assemble(self, dt: float):
        """A_i as (N, 3, 3) indexed [column][row] like glm, and b_i as (N, 3)."""
        A9 = np.empty((self.n_vertices, 3, 3), np.float32)
        b = np.empty((self.n_vertices, 3), np.float32)
        self._call(self._lib.oc_assemble(self._h, float(dt), ptr(A9), ptr(b)))
        return A9, b

    def profile(self, dt: float, n_steps: int) -> dict:
        names = C.create_string_buffer(32 * 8)
        ms = np.zeros(8, np.float64)
        launches = np.zeros(8, np.int64)
        byts = np.zeros(8, np.float64)
        n = C.c_int32()
        self._call(self._lib.oc_profile_steps(self._h, float(dt), int(n_steps), 8, names, ptr(ms), ptr(launches),
                                              ptr(byts), C.byref(n)))
        raw = names.raw
        out = {}
        for k in range(n.value):
            name = raw[32 * k: 32 * (k + 1)].split(b"\0", 1)[0].decode()
            out[name] = {"ms_total": float(ms[k]), "launches": int(launches[k]), "bytes": float(byts[k])}
        return out


class ImplicitCloth:
    """The reference's step interface for one cloth, on host arrays.

    ``X``, ``V`` (and the warm start ``dV``) are float32 (N, 3) arrays the caller may
    read and edit between steps.  ``springs`` starts empty; ``AddSpring`` appends a
    spring whose rest length is the current distance of its endpoints (IMP:370-380).
    The device handle is created on the first step and rebuilt if springs change.
    """

    def __init__(self, X: np.ndarray, V: np.ndarray | None = None, pinned: Sequence[int] | None = None,
                 gravity=DEFAULT_GRAVITY, velocity_damping: float = DEFAULT_DAMPING, mass=None,
                 cg_max_iter: int = 10, cg_tol: float = 1e-3, executor: str = "auto", ellipsoid=None,
                 ellipsoid_inv=None):
        self.X = np.ascontiguousarray(X, np.float32).reshape(-1, 3).copy()
        self.V = np.zeros_like(self.X) if V is None else np.ascontiguousarray(V, np.float32).reshape(-1, 3).copy()
        self.dV = np.zeros_like(self.X)
        self.F = np.zeros_like(self.X)
        self.springs = np.zeros(0, SPRING_DTYPE)
        self.pinned = None if pinned is None else np.asarray(pinned, np.int32)
        self.gravity = tuple(gravity)
        self.velocity_damping = float(velocity_damping)
        self.mass = mass
        self.cg_max_iter = int(cg_max_iter)
        self.cg_tol = float(cg_tol)
        self.executor = executor
        if ellipsoid is None:
            ellipsoid, ellipsoid_inv = reference_ellipsoid()
        self.ellipsoid = np.asarray(ellipsoid, np.float32).ravel()
        self.ellipsoid_inv = None if ellipsoid_inv is None else np.asarray(ellipsoid_inv, np.float32).ravel()
        self._solver: ClothSolver | None = None
        self._springs_seen = None
        self._passes = 0

    def AddSpring(self, a: int, b: int, ks: float, kd: float, type: int) -> None:  # noqa: N802 (reference name)
        d = self.X[a] - self.X[b]
        rest = np.sqrt(np.float32(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]), dtype=np.float32)
        rec = np.array([(a, b, rest, ks, kd, type)], SPRING_DTYPE)
        self.springs = np.concatenate([self.springs, rec])

    def _handle(self) -> ClothSolver:
        key = (self.springs.tobytes(), None if self.pinned is None else self.pinned.tobytes())
        if self._solver is None or self._springs_seen != key:
            if self._solver is not None:
                self._solver.close()
            desc = ClothDesc(n_vertices=self.X.shape[0], springs=self.springs, pinned=self.pinned,
                             mass=self.mass, gravity=self.gravity, velocity_damping=self.velocity_damping,
                             cg_max_iter=self.cg_max_iter, cg_tol=self.cg_tol, ellipsoid=self.ellipsoid,
                             ellipsoid_inv=self.ellipsoid_inv)
            self._solver = ClothSolver(desc, executor=self.executor)
            self._springs_seen = key
            self._passes = 0
        return self._solver

    def _step(self, dt: float, passes: int) -> None:
        s = self._handle()
        if self._passes != passes:
            s.set_passes(passes)
            self._passes = passes
        s.set_state(self.X, self.V, self.dV)
        s.step(dt, 1)
        self.X, self.V, self.dV = s.get_state()

    def _apply(self, passes: int) -> None:
        s = self._handle()
        s.set_state(self.X, self.V, self.dV)
        s.apply_passes(passes)
        self.X, self.V, self.dV = s.get_state()

    def ComputeForces(self) -> np.ndarray:  # noqa: N802
        s = self._handle()
        s.set_state(self.X, self.V, self.dV)
        self.F = s.compute_forces()
        return self.F

    def IntegrateImplicit(self, dt: float) -> None:  # noqa: N802
        self._step(dt, 0)

    def EllipsoidCollision(self) -> None:  # noqa: N802 (IMP:824)
        self._apply(N.PASS_ELLIPSOID)

    def ApplyProvotDynamicInverse(self) -> None:  # noqa: N802 (IMP:800)
        self._apply(N.PASS_PROVOT)

    def StepPhysics(self, dt: float) -> None:  # noqa: N802
        """ComputeForces(); IntegrateImplicit(dt); EllipsoidCollision();
        ApplyProvotDynamicInverse(); (IMP:873-880), as one step on the device."""
        self._step(dt, N.PASS_ELLIPSOID | N.PASS_PROVOT)
