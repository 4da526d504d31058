"""rs_gb300 -- the GB300 Repulsive-Surfaces hot path behind the crate's own entry points.

A thin Python host over ``librsgpu.so`` (C ABI in ``include/rsgpu.h``). The names mirror the
reference crate ``ddg-repulsive-surfaces`` (m1el/ddg-tools):

* ``Exponents`` (RS/src/kernel.rs:26-76), ``BhOptions`` (RS/src/energy/mod.rs:62-102);
* ``BhTree.build / attach / refit / try_energy / energy_and_differential /
  try_face_partials`` (RS/src/energy/barnes_hut.rs:156-471);
* ``energy()`` (RS/src/energy/mod.rs:168-219) returning an ``EnergyReport`` (:130-146);
* ``RsError`` carrying the crate's error kind (RS/src/error.rs).

There is no CPU fallback: if the library or a CUDA device is missing, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
import time
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import generators  # noqa: F401

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "librsgpu.so"

_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_vp = C.c_void_p
_dp = C.POINTER(C.c_double)


class SolverOptions(C.Structure):
    """rs_solver_options of include/rsgpu.h (HierarchicalOptions, RS/src/solve/iterative.rs:348-395)."""

    _fields_ = [("chi", C.c_double), ("leaf_size", C.c_int), ("leaf_pairs", C.c_int),
                ("restart", C.c_int), ("tolerance", C.c_double), ("max_iterations", C.c_int),
                ("tp_weight", C.c_double), ("low_order", C.c_int), ("eps_rel", C.c_double),
                ("eps_multi_rel", C.c_double), ("barycenter_per_component", C.c_int),
                ("vcycles", C.c_int), ("preconditioner", C.c_int),
                ("clamp_laplacian", C.c_int), ("coarse", C.c_int), ("inner_plain", C.c_int)]


class FlowOptions(C.Structure):
    """rs_flow_options of include/rsgpu.h (FlowOptions, RS/src/step/options.rs:290-382)."""

    _fields_ = [("alpha", C.c_double), ("beta", C.c_double), ("theta", C.c_double),
                ("leaf_size", C.c_int), ("solver", SolverOptions), ("hold_area", C.c_int),
                ("hold_volume", C.c_int), ("armijo_c", C.c_double), ("max_halvings", C.c_int),
                ("newton_max", C.c_int), ("ccd", C.c_int), ("ccd_gap", C.c_double),
                ("ccd_max_iterations", C.c_int), ("ccd_close_factor", C.c_double),
                ("start_rule", C.c_int), ("start_value", C.c_double), ("first_rule", C.c_int),
                ("first_value", C.c_double), ("tau_min_rel", C.c_double), ("newton_fixed", C.c_int),
                ("newton_tolerance", C.c_double), ("area_target", C.c_double),
                ("volume_target", C.c_double), ("guard_projection", C.c_int),
                ("retry_max_iterations", C.c_int), ("dense_fallback", C.c_int)]


# StartRule codes of rs_flow_options.start_rule / first_rule
START_ABSOLUTE, START_MAX_DISPLACEMENT, START_REFERENCE, START_GROW_PREVIOUS = 0, 1, 2, 3


class CcdOptions(C.Structure):
    """rs_ccd_options of include/rsgpu.h (CcdOptions, RS/src/ccd.rs:86-111): gap 0.05 of the
    reference length (0: the mean edge length of the start), 100 advances, close factor 0.5."""

    _fields_ = [("gap", C.c_double), ("reference_length", C.c_double), ("max_iterations", C.c_int),
                ("close_factor", C.c_double)]


class RsError(RuntimeError):
    """An error of the library: ``kind`` is the crate's RsError variant name, ``operation`` the
    failing operation word (RsError::Gpu { operation, detail }, RS/src/gpu/cuda.rs:19-24)."""

    def __init__(self, code: int, kind: str, operation: str, detail: str):
        super().__init__(f"{kind} ({operation}): {detail}")
        self.code, self.kind, self.operation, self.detail = code, kind, operation, detail


_lib = None


def load_library(path: str | os.PathLike | None = None):
    """Loads librsgpu.so from the package directory (built by ``build.build()``)."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RsError(10, "Gpu", "context", f"{p} is missing: run rs_gb300.build.build() first")
    L = C.CDLL(str(p))
    for name in ("rs_last_error", "rs_last_error_operation", "rs_last_error_kind"):
        getattr(L, name).restype = C.c_char_p
    sig = {
        "rs_device_count": [C.POINTER(C.c_int)],
        "rs_ccd_create": [_vp, C.c_int, C.c_int, _u32p, C.POINTER(_vp)],
        "rs_ccd_first_contact": [_vp, _f64p, _f64p, C.c_double, C.POINTER(CcdOptions), _dp, _i64p],
        "rs_ccd_last_seconds": [_vp, _dp],
        "rs_ccd_set_band": [_vp, C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)],
        "rs_ccd_intersecting_pairs": [_vp, _f64p, C.c_int64, _u32p, C.POINTER(C.c_int64)],
        "rs_device_info": [C.c_int, C.c_char_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                           C.POINTER(C.c_uint64)],
        "rs_ctx_create": [C.c_int, C.POINTER(_vp)],
        "rs_ctx_stream": [_vp, C.POINTER(_vp)],
        "rs_ctx_synchronize": [_vp],
        "rs_ctx_info": [_vp, C.c_char_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                        C.POINTER(C.c_int)],
        "rs_ctx_launch_count": [_vp, C.POINTER(C.c_int64)],
        "rs_surface_validate": [C.c_int, C.c_int, _u32p, _f64p],
        "rs_face_tree_build": [C.c_int, C.c_int, _u32p, _f64p, C.c_int, C.c_int, _u32p, _u32p,
                               _u32p, _u32p, _f64p, _f64p, C.POINTER(C.c_int)],
        "rs_bh_build": [_vp, C.c_int, C.c_int, _u32p, _f64p, C.c_double, C.c_int, C.POINTER(_vp)],
        "rs_bh_attach": [_vp, C.c_int, C.c_int, _u32p, _f64p, C.c_int, _u32p, _u32p, _u32p, _u32p,
                         _i64p, _u32p, _i64p, _u32p, C.POINTER(_vp)],
        "rs_bh_refit": [_vp, _f64p],
        "rs_bh_refit_device": [_vp, _vp],
        "rs_bh_energy": [_vp, C.c_double, C.c_double, _dp],
        "rs_bh_energy_and_differential": [_vp, C.c_double, C.c_double, _dp, _f64p],
        "rs_bh_energy_and_differential_device": [_vp, C.c_double, C.c_double, _vp, _vp],
        "rs_bh_face_partials": [_vp, C.c_double, C.c_double, _dp, _f64p],
        "rs_bh_sizes": [_vp, _i64p],
        "rs_bh_build_times": [_vp, _f64p],
        "rs_bh_export": [_vp, _u32p, _u32p, _u32p, _u32p, _i64p, _u32p, _i64p, _u32p],
        "rs_bh_culprit": [_vp, _i64p],
        "rs_bh_profile": [_vp, C.c_double, C.c_double, C.c_int, C.c_char_p, C.c_int, _f64p,
                          C.c_int, C.POINTER(C.c_int)],
        "rs_metric_build": [_vp, C.c_int, C.c_int, _u32p, _f64p, C.c_double, C.c_double, C.c_double,
                            C.c_int, C.c_int, C.POINTER(_vp)],
        "rs_metric_apply": [_vp, C.c_double, C.c_double, C.c_int, _f64p, _f64p],
        "rs_metric_apply_device": [_vp, C.c_double, C.c_double, C.c_int, _vp, _vp],
        "rs_metric_stats": [_vp, _i64p],
        "rs_metric_build_times": [_vp, _f64p],
        "rs_metric_blocks": [_vp, _u32p, _u32p, _u32p, _u32p],
        "rs_metric_profile": [_vp, C.c_double, C.c_double, C.c_int, C.c_int, C.c_char_p, C.c_int,
                              _f64p, C.c_int, C.POINTER(C.c_int)],
        "rs_vfrac_build": [_vp, C.c_int, _f64p, _f64p, C.c_double, C.c_double, C.c_int, C.c_int,
                           C.POINTER(_vp)],
        "rs_vfrac_apply": [_vp, C.c_int, _f64p, _f64p],
        "rs_vfrac_apply_device": [_vp, C.c_int, _vp, _vp],
        "rs_vfrac_stats": [_vp, _i64p],
        "rs_solver_build": [_vp, C.c_int, C.c_int, _u32p, _f64p, C.c_double, C.c_double, C.c_void_p,
                            C.POINTER(_vp)],
        "rs_solver_dims": [_vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)],
        "rs_solver_apply": [_vp, C.c_int, _f64p, _f64p],
        "rs_solver_apply_device": [_vp, C.c_int, _vp, _vp],
        "rs_solver_precondition": [_vp, C.c_int, _f64p, _f64p],
        "rs_solver_precondition_device": [_vp, C.c_int, _vp, _vp],
        "rs_solver_solve_many": [_vp, C.c_int, _f64p, _f64p, _f64p],
        "rs_solver_solve_many_device": [_vp, C.c_int, _vp, _vp, _f64p],
        "rs_solver_dense_solve_many_device": [_vp, C.c_int, _vp, _vp, _f64p],
        "rs_solver_dense_pivot_ratio": [_vp, C.POINTER(C.c_double)],
        "rs_metric_apply_device_noalloc": [_vp, C.c_double, C.c_double, C.c_int, C.c_void_p, C.c_void_p],
        "rs_copy_counters": [C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)],
        "rs_solver_build_times": [_vp, _f64p],
        "rs_learned_create": [_vp, C.c_uint64, C.POINTER(_vp)],
        "rs_learned_parameter_count": [_vp, C.POINTER(C.c_int64)],
        "rs_learned_get_parameters": [_vp, np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")],
        "rs_learned_set_parameters": [_vp, np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")],
        "rs_learned_get_gradient": [_vp, np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")],
        "rs_lgraph_create": [_vp, C.c_int, C.c_int, _u32p, _f64p, C.POINTER(_vp)],
        "rs_learned_apply_device": [_vp, _vp, C.c_int, _vp, _vp, _vp],
        "rs_learned_loss_and_gradient_device": [_vp, _vp, _vp, _vp, _vp, C.POINTER(C.c_double)],
        "rs_learned_adam_step": [_vp, C.c_double, C.c_double],
        "rs_solver_set_learned": [_vp, _vp, _vp, C.c_int, C.c_int],
        "rs_solver_learned_counts": [_vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)],
        "rs_flow_set_learned": [_vp, _vp, C.c_int, C.c_int],
        "rs_solver_set_gmres": [_vp, C.c_int, C.c_int, C.c_double],
        "rs_solver_multigrid_levels": [_vp, _i64p, C.c_int, C.POINTER(C.c_int)],
        "rs_solver_profile": [_vp, C.c_int, _f64p, C.c_char_p, C.c_int, _f64p, C.c_int, C.POINTER(C.c_int)],
        "rs_solver_history": [_vp, C.c_int, _f64p, C.c_int, C.POINTER(C.c_int), _f64p, C.c_int,
                              C.POINTER(C.c_int)],
        "rs_flow_create": [_vp, C.c_int, C.c_int, _u32p, _f64p, C.c_void_p, C.POINTER(_vp)],
        "rs_flow_step": [_vp, _f64p],
        "rs_flow_direction": [_vp, _f64p],
        "rs_flow_last_direction": [_vp, _f64p, _f64p],
        "rs_flow_last_trials": [_vp, _f64p, C.c_int, C.POINTER(C.c_int)],
        "rs_flow_last_solutions": [_vp, C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int64)],
        "rs_flow_positions": [_vp, _f64p],
        "rs_flow_cancel": [_vp, C.c_int],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = C.c_int
    L.rs_ctx_free.argtypes = [_vp]
    L.rs_ctx_free.restype = None
    L.rs_solver_options_default.restype = SolverOptions
    L.rs_solver_options_default.argtypes = []
    L.rs_flow_options_default.restype = FlowOptions
    L.rs_flow_options_default.argtypes = []
    L.rs_flow_free.argtypes = [_vp]
    L.rs_flow_free.restype = None
    L.rs_ccd_options_default.restype = CcdOptions
    L.rs_ccd_options_default.argtypes = []
    L.rs_ccd_free.argtypes = [_vp]
    L.rs_ccd_free.restype = None
    for name in ("rs_learned_free", "rs_lgraph_free"):
        getattr(L, name).argtypes = [_vp]
        getattr(L, name).restype = None
    for name in ("rs_bh_free", "rs_metric_free", "rs_vfrac_free", "rs_solver_free"):
        getattr(L, name).argtypes = [_vp]
        getattr(L, name).restype = None
    _lib = L
    return L


def _check(code: int) -> None:
    if code != 0:
        L = load_library()
        raise RsError(code, L.rs_last_error_kind().decode(), L.rs_last_error_operation().decode(),
                      L.rs_last_error().decode())


def device_count() -> int:
    n = C.c_int()
    _check(load_library().rs_device_count(C.byref(n)))
    return n.value


def device_info(ordinal: int = 0) -> dict:
    """Name, compute capability and memory of one device, without creating a context
    (gpu::devices, RS/src/gpu/mod.rs:89-100)."""
    name = C.create_string_buffer(256)
    ma, mi, mem = C.c_int(), C.c_int(), C.c_uint64()
    _check(load_library().rs_device_info(int(ordinal), name, 256, C.byref(ma), C.byref(mi), C.byref(mem)))
    return {"ordinal": int(ordinal), "name": name.value.decode(), "compute_capability": f"{ma.value}.{mi.value}",
            "memory_bytes": int(mem.value)}


class Context:
    """A device and its stream (GpuContext, RS/src/gpu/mod.rs:36-127)."""

    def __init__(self, ordinal: int = 0):
        L = load_library()
        h = _vp()
        _check(L.rs_ctx_create(int(ordinal), C.byref(h)))
        self._h = h
        self.ordinal = ordinal

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.rs_ctx_free(self._h)
            self._h = None

    @property
    def handle(self):
        return self._h

    @property
    def stream(self) -> int:
        s = _vp()
        _check(_lib.rs_ctx_stream(self._h, C.byref(s)))
        return s.value or 0

    def synchronize(self) -> None:
        _check(_lib.rs_ctx_synchronize(self._h))

    def info(self) -> dict:
        name = C.create_string_buffer(256)
        sm, ma, mi = C.c_int(), C.c_int(), C.c_int()
        _check(_lib.rs_ctx_info(self._h, name, 256, C.byref(sm), C.byref(ma), C.byref(mi)))
        return {"name": name.value.decode(), "sm_count": sm.value, "cc": (ma.value, mi.value)}

    def fp32_peak_tflops(self) -> float:
        """Measured FP32 FMA throughput of the device (TFLOP/s), by the separate measurement
        library librsprobe.so (rsp_fp32_peak)."""
        probe = C.CDLL(str(Path(__file__).resolve().parent / "librsprobe.so"))
        probe.rsp_fp32_peak.argtypes = [C.c_int, C.POINTER(C.c_double)]
        probe.rsp_fp32_peak.restype = C.c_int
        t = C.c_double()
        err = probe.rsp_fp32_peak(self.ordinal, C.byref(t))
        if err:
            raise RsError(f"rsp_fp32_peak: CUDA error {err}")
        return t.value

    def launch_count(self) -> int:
        n = C.c_int64()
        _check(_lib.rs_ctx_launch_count(self._h, C.byref(n)))
        return n.value


_default_ctx = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


@dataclass(frozen=True)
class Exponents:
    """(alpha, beta) of the tangent-point kernel (RS/src/kernel.rs:26-76)."""

    alpha: float = 6.0
    beta: float = 12.0

    def __post_init__(self):
        a, b = self.alpha, self.beta
        if not (np.isfinite(a) and np.isfinite(b)):
            raise RsError(1, "InvalidExponents", "energy", "both exponents must be finite")
        if a <= 1.0:
            raise RsError(1, "InvalidExponents", "energy", "alpha must be greater than 1")
        if b <= a + 2.0:
            raise RsError(1, "InvalidExponents", "energy",
                          "beta must be greater than alpha + 2 (s = (beta - 2)/alpha > 1)")
        if b >= 2.0 * a + 2.0:
            raise RsError(1, "InvalidExponents", "energy",
                          "beta must be smaller than 2 alpha + 2 (s = (beta - 2)/alpha < 2)")

    @property
    def s(self) -> float:
        return (self.beta - 2.0) / self.alpha


@dataclass(frozen=True)
class BhOptions:
    """Barnes-Hut parameters (RS/src/energy/mod.rs:62-102): theta 0.5, leaf size 8."""

    theta: float = 0.5
    leaf_size: int = 8


def _mesh(faces, positions):
    faces = np.ascontiguousarray(faces, dtype=np.uint32).reshape(-1, 3)
    positions = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
    return faces, positions


def validate_surface(faces, positions) -> None:
    """Surface::new + validate_positions (RS/src/surface.rs:132-541); raises RsError."""
    faces, positions = _mesh(faces, positions)
    _check(load_library().rs_surface_validate(len(positions), len(faces), faces.ravel(),
                                              positions.ravel()))


def face_tree(faces, positions, leaf_size: int = 8) -> dict:
    """The face BVH as the library builds it on the host (no device work)."""
    faces, positions = _mesh(faces, positions)
    cap = max(2 * len(faces), 1)
    start, end, right = (np.empty(cap, np.uint32) for _ in range(3))
    order = np.empty(len(faces), np.uint32)
    box, radius = np.empty(6 * cap), np.empty(cap)
    n = C.c_int()
    _check(load_library().rs_face_tree_build(len(positions), len(faces), faces.ravel(),
                                             positions.ravel(), int(leaf_size), cap, start, end,
                                             right, order, box, radius, C.byref(n)))
    k = n.value
    return dict(start=start[:k], end=end[:k], right=right[:k], order=order,
                box=box[: 6 * k].reshape(k, 6), radius=radius[:k])


class BhTree:
    """The Barnes-Hut evaluator of one step on the GPU (BhTree + DeviceBh,
    RS/src/energy/barnes_hut.rs:114-471). Build once per step, refit for line-search trials."""

    def __init__(self, handle, ctx: Context, n_vertices: int, n_faces: int):
        self._h, self.ctx, self.n_vertices, self.n_faces = handle, ctx, n_vertices, n_faces

    @classmethod
    def build(cls, faces, positions, opts: BhOptions = BhOptions(), ctx: Context | None = None):
        ctx = ctx or default_context()
        faces, positions = _mesh(faces, positions)
        h = _vp()
        _check(_lib.rs_bh_build(ctx.handle, len(positions), len(faces), faces.ravel(),
                                positions.ravel(), float(opts.theta), int(opts.leaf_size),
                                C.byref(h)))
        t = cls(h, ctx, len(positions), len(faces))
        t.options = opts
        return t

    @classmethod
    def attach(cls, faces, positions, tree: dict, lists: dict, ctx: Context | None = None):
        """attach_gpu with a tree and lists built by the caller (dicts as the oracle exports)."""
        ctx = ctx or default_context()
        faces, positions = _mesh(faces, positions)
        u = lambda a: np.ascontiguousarray(a, dtype=np.uint32)  # noqa: E731
        i = lambda a: np.ascontiguousarray(a, dtype=np.int64)  # noqa: E731
        h = _vp()
        _check(_lib.rs_bh_attach(ctx.handle, len(positions), len(faces), faces.ravel(),
                                 positions.ravel(), len(tree["start"]), u(tree["start"]),
                                 u(tree["end"]), u(tree["right"]), u(tree["order"]),
                                 i(lists["lumped_off"]), u(lists["lumped"]),
                                 i(lists["exact_off"]), u(lists["exact"]), C.byref(h)))
        return cls(h, ctx, len(positions), len(faces))

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.rs_bh_free(self._h)
            self._h = None

    def refit(self, positions) -> None:
        p = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1)
        if p.size != 3 * self.n_vertices:
            raise RsError(3, "PositionCountMismatch", "energy",
                          f"expected {self.n_vertices} positions, found {p.size // 3}")
        _check(_lib.rs_bh_refit(self._h, p))

    def refit_device(self, positions_dev_ptr: int) -> None:
        _check(_lib.rs_bh_refit_device(self._h, _vp(positions_dev_ptr)))

    def try_energy(self, e: Exponents = Exponents()) -> float:
        out = C.c_double()
        _check(_lib.rs_bh_energy(self._h, e.alpha, e.beta, C.byref(out)))
        return out.value

    def energy_and_differential(self, e: Exponents = Exponents()):
        out = C.c_double()
        d = np.empty((self.n_vertices, 3))
        _check(_lib.rs_bh_energy_and_differential(self._h, e.alpha, e.beta, C.byref(out), d.ravel()))
        return out.value, d

    def energy_and_differential_device(self, e: Exponents, energy_dev_ptr: int, dE_dev_ptr: int):
        _check(_lib.rs_bh_energy_and_differential_device(self._h, e.alpha, e.beta,
                                                         _vp(energy_dev_ptr), _vp(dE_dev_ptr)))

    def try_face_partials(self, e: Exponents = Exponents()):
        out = C.c_double()
        p = np.empty((self.n_faces, 7))
        _check(_lib.rs_bh_face_partials(self._h, e.alpha, e.beta, C.byref(out), p.ravel()))
        return out.value, p

    def build_times(self) -> dict:
        """Seconds spent in the phases of the build."""
        o = np.zeros(7)
        _check(_lib.rs_bh_build_times(self._h, o))
        return dict(zip(["geometry", "tree", "topology", "list_counts", "list_fill", "list_finish", "refit"],
                        map(float, o)))

    def sizes(self) -> dict:
        o = np.zeros(7, np.int64)
        _check(_lib.rs_bh_sizes(self._h, o))
        keys = ["n_nodes", "n_leaves", "n_lumped", "n_exact", "n_partner", "pairs_exact",
                "lumped_interactions"]
        return dict(zip(keys, (int(x) for x in o)))

    def export(self) -> tuple[dict, dict]:
        s = self.sizes()
        nn, nl = s["n_nodes"], s["n_leaves"]
        start, end, right = (np.empty(nn, np.uint32) for _ in range(3))
        order = np.empty(self.n_faces, np.uint32)
        lo, eo = np.empty(nl + 1, np.int64), np.empty(nl + 1, np.int64)
        lum, ex = np.empty(max(s["n_lumped"], 1), np.uint32), np.empty(max(s["n_exact"], 1), np.uint32)
        _check(_lib.rs_bh_export(self._h, start, end, right, order, lo, lum, eo, ex))
        return (dict(start=start, end=end, right=right, order=order),
                dict(lumped_off=lo, lumped=lum[: s["n_lumped"]], exact_off=eo, exact=ex[: s["n_exact"]]))

    def culprit(self) -> tuple[int, int]:
        o = np.zeros(2, np.int64)
        _check(_lib.rs_bh_culprit(self._h, o))
        return int(o[0]), int(o[1])

    def profile(self, e: Exponents = Exponents(), reps: int = 5) -> dict:
        """Average ms per kernel of one energy+differential evaluation (CUDA events)."""
        names = C.create_string_buffer(4096)
        ms = np.zeros(32)
        n = C.c_int()
        _check(_lib.rs_bh_profile(self._h, e.alpha, e.beta, int(reps), names, 4096, ms, 32, C.byref(n)))
        raw = names.raw.split(b"\0")[: n.value]
        return {k.decode(): float(v) for k, v in zip(raw, ms[: n.value])}


@dataclass
class EnergyReport:
    """Result of energy() (RS/src/energy/mod.rs:130-146)."""

    energy: float
    differential: np.ndarray
    penalties: list = field(default_factory=list)
    subcritical: bool = False
    pairs_exact: int = 0
    nodes_lumped: int = 0
    seconds: float = 0.0

    def total(self) -> float:
        return self.energy + sum(self.penalties)


def energy(faces, positions, exponents: Exponents = Exponents(), eval=None,
           ctx: Context | None = None) -> EnergyReport:
    """The crate's energy entry (RS/src/energy/mod.rs:168-219) on the GPU.

    ``eval`` is ``"exact"`` (all ordered pairs; on the device this is Barnes-Hut with theta 0,
    which admits no far field) or a ``BhOptions``. Penalties are not part of this path."""
    t0 = time.perf_counter()
    opts = BhOptions(theta=0.0) if eval in (None, "exact") else eval
    tree = BhTree.build(faces, positions, opts, ctx)
    E, dE = tree.energy_and_differential(exponents)
    s = tree.sizes()
    return EnergyReport(energy=E, differential=dE, subcritical=exponents.beta - exponents.alpha <= 4.0,
                        pairs_exact=s["pairs_exact"], nodes_lumped=s["n_lumped"],
                        seconds=time.perf_counter() - t0)


@dataclass(frozen=True)
class ClusterTreeOptions:
    """Block cluster tree parameters (RS/src/metric/hierarchical.rs:63-108)."""

    chi: float = 0.5
    leaf_size: int = 8
    leaf_pairs: int = 64


def _profile_dict(names, ms, n):
    raw = names.raw.split(b"\0")[: n.value]
    return {k.decode(): float(v) for k, v in zip(raw, ms[: n.value])}


class FaceMetricTree:
    """The hierarchical Hs metric w_hi B~ + w_lo B~0 on the GPU (FaceMetricTree + GpuFaceMetric,
    RS/src/metric/hierarchical.rs:279-812)."""

    def __init__(self, faces, positions, exponents: Exponents = Exponents(),
                 opts: ClusterTreeOptions = ClusterTreeOptions(), ctx: Context | None = None):
        self.ctx = ctx or default_context()
        faces, positions = _mesh(faces, positions)
        self.n_vertices, self.n_faces = len(positions), len(faces)
        h = _vp()
        _check(_lib.rs_metric_build(self.ctx.handle, len(positions), len(faces), faces.ravel(),
                                    positions.ravel(), exponents.alpha, exponents.beta, opts.chi,
                                    opts.leaf_size, opts.leaf_pairs, C.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.rs_metric_free(self._h)
            self._h = None

    def apply(self, x, w_hi: float = 1.0, w_lo: float = 1.0):
        """y = (w_hi B~ + w_lo B~0) x for x of shape (3V,) or (nb, 3V) (interleaved 3 v + axis)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        xs = x.reshape(-1, 3 * self.n_vertices)
        ys = np.empty_like(xs)
        _check(_lib.rs_metric_apply(self._h, w_hi, w_lo, len(xs), xs.ravel(), ys.ravel()))
        return ys.reshape(x.shape)

    def apply_device(self, xs_ptr: int, ys_ptr: int, nb: int, w_hi=1.0, w_lo=1.0):
        _check(_lib.rs_metric_apply_device(self._h, w_hi, w_lo, nb, _vp(xs_ptr), _vp(ys_ptr)))

    def stats(self) -> dict:
        o = np.zeros(5, np.int64)
        _check(_lib.rs_metric_stats(self._h, o))
        return dict(zip(["far_blocks", "near_blocks", "near_entries", "depth", "nodes"], map(int, o)))

    def build_times(self) -> dict:
        """Seconds spent in the phases of the build."""
        o = np.zeros(8)
        _check(_lib.rs_metric_build_times(self._h, o))
        return dict(zip(["geometry", "tree", "projectors", "blocks", "face_records", "work_items",
                         "far_coefficients", "device"], map(float, o)))

    def blocks(self) -> dict:
        s = self.stats()
        nn = s["nodes"]
        fp, np_ = np.empty(nn + 1, np.uint32), np.empty(nn + 1, np.uint32)
        fc = np.empty(max(s["far_blocks"], 1), np.uint32)
        nc = np.empty(max(s["near_blocks"], 1), np.uint32)
        _check(_lib.rs_metric_blocks(self._h, fp, fc, np_, nc))
        return dict(far_ptr=fp, far_col=fc[: s["far_blocks"]], near_ptr=np_, near_col=nc[: s["near_blocks"]])

    def profile(self, nb: int = 3, reps: int = 5, w_hi=1.0, w_lo=1.0) -> dict:
        names = C.create_string_buffer(4096)
        ms = np.zeros(32)
        n = C.c_int()
        _check(_lib.rs_metric_profile(self._h, w_hi, w_lo, nb, reps, names, 4096, ms, 32, C.byref(n)))
        return _profile_dict(names, ms, n)


class VertexFractionalTree:
    """The vertex-pair fractional operator L^V_tau on the GPU (VertexFractionalTree +
    GpuVertexFractional, RS/src/metric/hierarchical.rs:998-1346)."""

    def __init__(self, positions, mass, tau: float, opts: ClusterTreeOptions = ClusterTreeOptions(),
                 ctx: Context | None = None):
        self.ctx = ctx or default_context()
        positions = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        mass = np.ascontiguousarray(mass, dtype=np.float64)
        self.n_vertices = len(positions)
        h = _vp()
        _check(_lib.rs_vfrac_build(self.ctx.handle, len(positions), positions.ravel(), mass, float(tau),
                                   opts.chi, opts.leaf_size, opts.leaf_pairs, C.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.rs_vfrac_free(self._h)
            self._h = None

    def apply(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        xs = x.reshape(-1, 3 * self.n_vertices)
        ys = np.empty_like(xs)
        _check(_lib.rs_vfrac_apply(self._h, len(xs), xs.ravel(), ys.ravel()))
        return ys.reshape(x.shape)

    def stats(self) -> dict:
        o = np.zeros(5, np.int64)
        _check(_lib.rs_vfrac_stats(self._h, o))
        return dict(zip(["far_blocks", "near_blocks", "near_entries", "depth", "nodes"], map(int, o)))


def solver_options(**kw) -> SolverOptions:
    """The library defaults (rs_solver_options_default) with the given fields replaced."""
    o = load_library().rs_solver_options_default()
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class SaddleSolver:
    """The hierarchical saddle solver of one step on the GPU (HierarchicalSaddle,
    RS/src/solve/iterative.rs:426-575): A' [x; l] = [a; b] by right-preconditioned GMRES."""

    def __init__(self, faces, positions, exponents: Exponents = Exponents(),
                 options: SolverOptions | None = None, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        faces, positions = _mesh(faces, positions)
        o = options or solver_options()
        h = _vp()
        _check(_lib.rs_solver_build(self.ctx.handle, len(positions), len(faces), faces.ravel(),
                                    positions.ravel(), exponents.alpha, exponents.beta, C.byref(o),
                                    C.byref(h)))
        self._h = h
        nd, nc = C.c_int64(), C.c_int64()
        _check(_lib.rs_solver_dims(h, C.byref(nd), C.byref(nc)))
        self.n_dofs, self.n_constraints = nd.value, nc.value
        self.n = self.n_dofs + self.n_constraints

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.rs_solver_free(self._h)
            self._h = None

    def _batch(self, fn, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        xs = x.reshape(-1, self.n)
        ys = np.empty_like(xs)
        _check(fn(self._h, len(xs), xs.ravel(), ys.ravel()))
        return ys.reshape(x.shape)

    def apply(self, x):
        """A' x for x of shape (n,) or (nb, n), n = 3V + k_Q."""
        return self._batch(_lib.rs_solver_apply, x)

    def precondition(self, r):
        """P^-1 r."""
        return self._batch(_lib.rs_solver_precondition, r)

    def solve_many(self, rhs):
        """Solves A' y = rhs for up to 4 stacked right-hand sides; returns (y, reports)."""
        rhs = np.ascontiguousarray(rhs, dtype=np.float64).reshape(-1, self.n)
        out = np.empty_like(rhs)
        rep = np.zeros(5 * len(rhs))
        _check(_lib.rs_solver_solve_many(self._h, len(rhs), rhs.ravel(), out.ravel(), rep))
        keys = ["iterations", "relative_residual", "converged", "seconds", "cycles"]
        reports = [dict(zip(keys, rep[5 * i: 5 * i + 5])) for i in range(len(rhs))]
        for r in reports:
            r["iterations"] = int(r["iterations"])
            r["converged"] = bool(r["converged"])
        return out, reports

    def dense_solve_many(self, rhs):
        """The dense last resort (rs_solver_dense_solve_many_device): A' with the exact metric
        factored by LU on the device, one refinement step; returns (y, reports)."""
        import torch

        rhs = np.ascontiguousarray(rhs, dtype=np.float64).reshape(-1, self.n)
        rd = torch.tensor(rhs, device=f"cuda:{self.ctx.ordinal}")
        sd = torch.empty_like(rd)
        rep = np.zeros(5 * len(rhs))
        torch.cuda.synchronize(rd.device)
        _check(_lib.rs_solver_dense_solve_many_device(self._h, len(rhs), _vp(rd.data_ptr()), _vp(sd.data_ptr()), rep))
        self.ctx.synchronize()
        keys = ["iterations", "relative_residual", "converged", "seconds", "cycles"]
        reports = [dict(zip(keys, rep[5 * i: 5 * i + 5])) for i in range(len(rhs))]
        return sd.cpu().numpy(), reports

    def dense_pivot_ratio(self) -> float:
        r = C.c_double()
        _check(_lib.rs_solver_dense_pivot_ratio(self._h, C.byref(r)))
        return r.value

    def profile(self, rhs) -> dict:
        """Milliseconds per phase of one solve of the stacked right-hand sides."""
        rhs = np.ascontiguousarray(rhs, dtype=np.float64).reshape(-1, self.n)
        names = C.create_string_buffer(4096)
        ms = np.zeros(64)
        n = C.c_int()
        _check(_lib.rs_solver_profile(self._h, len(rhs), rhs.ravel(), names, 4096, ms, 64, C.byref(n)))
        return _profile_dict(names, ms, n)

    def multigrid_levels(self) -> list[tuple[int, int]]:
        """(rows, nonzeros) of every multigrid level, finest first."""
        out = np.zeros(64, np.int64)
        n = C.c_int()
        _check(_lib.rs_solver_multigrid_levels(self._h, out, 32, C.byref(n)))
        return [(int(out[2 * i]), int(out[2 * i + 1])) for i in range(min(n.value, 32))]

    def set_learned(self, model: "LearnedModel | None", graph: "SurfaceGraph | None" = None,
                    cheap_steps: int = 2, max_iterations: int = 0) -> None:
        """Uses the learned preconditioner (plain as the fallback), or the plain one again."""
        self._learned = (model, graph)  # keep both alive while the solver uses them
        _check(_lib.rs_solver_set_learned(self._h, model._h if model else None, graph._h if graph else None,
                                          cheap_steps, max_iterations))

    def learned_counts(self) -> tuple[int, int]:
        a, b = C.c_int64(), C.c_int64()
        _check(_lib.rs_solver_learned_counts(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def build_times(self) -> dict:
        """Host seconds of the solver's set-up by phase."""
        o = np.zeros(6)
        _check(_lib.rs_solver_build_times(self._h, o))
        return dict(zip(["metric", "vertex_fractional", "laplacian", "multigrid_setup", "multigrid_upload",
                         "total"], o.tolist()))

    def history(self, q: int = 0):
        """(per-iteration estimated relative residuals, explicit residual at every cycle start)
        of right-hand side q of the last solve."""
        ni, nc = C.c_int(), C.c_int()
        _check(_lib.rs_solver_history(self._h, q, np.zeros(1), 0, C.byref(ni), np.zeros(1), 0, C.byref(nc)))
        est, cyc = np.zeros(max(ni.value, 1)), np.zeros(max(nc.value, 1))
        _check(_lib.rs_solver_history(self._h, q, est, ni.value, C.byref(ni), cyc, nc.value, C.byref(nc)))
        return est[: ni.value], cyc[: nc.value]


def flow_options(**kw) -> FlowOptions:
    """The library defaults (rs_flow_options_default); keys of the solver options may be given
    with a ``solver_`` prefix."""
    o = load_library().rs_flow_options_default()
    for k, v in kw.items():
        if k.startswith("solver_"):
            setattr(o.solver, k[7:], v)
        else:
            setattr(o, k, v)
    return o


FLOW_REPORT_KEYS = ["energy_before", "energy_after", "tau", "halvings", "gmres_area", "gmres_volume",
                    "gmres_direction", "relative_residual", "seconds", "seconds_tree", "seconds_energy",
                    "seconds_solver_build", "seconds_solve", "seconds_line_search", "seconds_projection",
                    "accepted", "slope", "constraint_residual", "fallbacks", "learned_solves",
                    "learned_fallbacks", "gradient_norm", "tau0", "direction_max", "newton_steps",
                    "projection_status", "energy_trial", "tau_ccd", "seconds_ccd", "projection_blocked"]
PROJECTION_STATUS = ["converged", "maxrounds", "notimproving", "blocked"]
TRIAL_OUTCOMES = ["accepted", "armijo-failed", "non-finite", "projection-blocked"]


class Flow:
    """The repulsive-surface flow (Session, RS/src/step/session.rs): one Hs descent step per
    call of ``step()`` on the GPU (no remeshing, no collision detection)."""

    def __init__(self, faces, positions, options: FlowOptions | None = None, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        faces, positions = _mesh(faces, positions)
        self.n_vertices = len(positions)
        o = options or flow_options()
        h = _vp()
        _check(_lib.rs_flow_create(self.ctx.handle, len(positions), len(faces), faces.ravel(),
                                   positions.ravel(), C.byref(o), C.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.rs_flow_free(self._h)
            self._h = None

    def step(self) -> dict:
        rep = np.zeros(len(FLOW_REPORT_KEYS))
        _check(_lib.rs_flow_step(self._h, rep))
        return dict(zip(FLOW_REPORT_KEYS, rep.tolist()))

    def direction(self) -> dict:
        """Energy, differential and constrained direction at the current positions without a
        line search (the report's solve entries); ``last_direction()`` returns x and g."""
        rep = np.zeros(len(FLOW_REPORT_KEYS))
        _check(_lib.rs_flow_direction(self._h, rep))
        return dict(zip(FLOW_REPORT_KEYS, rep.tolist()))

    def last_direction(self) -> tuple[np.ndarray, np.ndarray]:
        """(x, g), V x 3 each, of the last step or direction: the step moves f <- f - tau x."""
        x, g = np.empty((self.n_vertices, 3)), np.empty((self.n_vertices, 3))
        _check(_lib.rs_flow_last_direction(self._h, x.ravel(), g.ravel()))
        return x, g

    def last_solutions(self) -> np.ndarray:
        """The last step's saddle solutions, (k + 1) x n: the Schur columns of the held rows
        (area, then volume), then y = A'^-1 [g; 0]."""
        k, n = C.c_int(), C.c_int64()
        _check(_lib.rs_flow_last_solutions(self._h, None, C.byref(k), C.byref(n)))
        out = np.empty((k.value + 1, n.value))
        _check(_lib.rs_flow_last_solutions(self._h, out.ctypes.data_as(C.c_void_p), C.byref(k), C.byref(n)))
        return out

    def last_trials(self) -> list[tuple[float, float, str]]:
        """(tau, energy, outcome) of every line-search trial of the last step."""
        n = C.c_int()
        _check(_lib.rs_flow_last_trials(self._h, np.zeros(3), 0, C.byref(n)))
        out = np.zeros(3 * max(n.value, 1))
        _check(_lib.rs_flow_last_trials(self._h, out, n.value, C.byref(n)))
        return [(out[3 * i], out[3 * i + 1], TRIAL_OUTCOMES[int(out[3 * i + 2])]) for i in range(n.value)]

    def set_learned(self, model: "LearnedModel | None", cheap_steps: int = 2, max_iterations: int = 0) -> None:
        self._learned = model
        _check(_lib.rs_flow_set_learned(self._h, model._h if model else None, cheap_steps, max_iterations))

    def positions(self) -> np.ndarray:
        out = np.empty((self.n_vertices, 3))
        _check(_lib.rs_flow_positions(self._h, out.ravel()))
        return out

    def cancel(self, on: bool = True) -> None:
        """Stops the running step between line-search trials, and later steps, with RsError
        kind "Cancelled"; the positions stay those of the last completed step."""
        _check(_lib.rs_flow_cancel(self._h, int(bool(on))))


def ccd_options(**kw) -> CcdOptions:
    """The library defaults (rs_ccd_options_default) with the given fields replaced."""
    o = load_library().rs_ccd_options_default()
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class CcdSurface:
    """Continuous collision detection of one surface against itself (first_contact,
    RS/src/ccd.rs:762-884, without obstacles and without the exempt band): the topology lives
    on the device, each ``first_contact`` call sweeps one linear motion."""

    REPORT_KEYS = ["contact", "windows", "pairs_tested", "close_pairs", "touching_pairs", "exempt_pairs",
                   "evaluations"]

    def __init__(self, faces, n_vertices: int, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        faces = np.ascontiguousarray(faces, dtype=np.uint32).reshape(-1, 3)
        self.n_vertices = int(n_vertices)
        h = _vp()
        _check(_lib.rs_ccd_create(self.ctx.handle, self.n_vertices, len(faces), faces.ravel(), C.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.rs_ccd_free(self._h)
            self._h = None

    def first_contact(self, start, velocity, tau_end: float, options: CcdOptions | None = None) -> dict:
        start = np.ascontiguousarray(start, dtype=np.float64).reshape(-1, 3)
        vel = np.ascontiguousarray(velocity, dtype=np.float64).reshape(-1, 3)
        if len(start) != self.n_vertices or len(vel) != self.n_vertices:
            raise RsError(1, "InvalidOption", "ccd", "start and velocity need one vector per vertex")
        o = options or ccd_options()
        tau = C.c_double()
        rep = np.zeros(7, np.int64)
        _check(_lib.rs_ccd_first_contact(self._h, start.ravel(), vel.ravel(), float(tau_end), C.byref(o),
                                         C.byref(tau), rep))
        return {"tau_max": tau.value, **{k: int(v) for k, v in zip(self.REPORT_KEYS, rep)}}

    def set_band(self, positions) -> tuple[int, int]:
        """The exempt band of `positions` for the following calls (IntersectionBand::new,
        RS/src/ccd.rs:1292-1319); None clears it. Returns (intersecting pairs, band vertices)."""
        npairs, nverts = C.c_int64(), C.c_int64()
        if positions is None:
            _check(_lib.rs_ccd_set_band(self._h, None, C.byref(npairs), C.byref(nverts)))
        else:
            p = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
            if len(p) != self.n_vertices:
                raise RsError(1, "InvalidOption", "ccd", "positions need one vector per vertex")
            _check(_lib.rs_ccd_set_band(self._h, p.ctypes.data_as(C.c_void_p), C.byref(npairs), C.byref(nverts)))
        return npairs.value, nverts.value

    def intersecting_pairs(self, positions) -> np.ndarray:
        """The intersecting face pairs (f < g), sorted (intersecting_pairs, RS/src/ccd.rs:1229-1279)."""
        p = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        if len(p) != self.n_vertices:
            raise RsError(1, "InvalidOption", "ccd", "positions need one vector per vertex")
        n = C.c_int64()
        out = np.zeros(2 * 1024, np.uint32)
        _check(_lib.rs_ccd_intersecting_pairs(self._h, p.ravel(), len(out) // 2, out, C.byref(n)))
        if n.value > len(out) // 2:
            out = np.zeros(2 * n.value, np.uint32)
            _check(_lib.rs_ccd_intersecting_pairs(self._h, p.ravel(), n.value, out, C.byref(n)))
        return out[: 2 * n.value].reshape(-1, 2)

    def last_seconds(self) -> float:
        t = C.c_double()
        _check(_lib.rs_ccd_last_seconds(self._h, C.byref(t)))
        return t.value


def copy_counters() -> tuple[int, int]:
    """(host->device, device->host) bytes the library has copied in this process."""
    a, b = C.c_uint64(), C.c_uint64()
    _check(load_library().rs_copy_counters(C.byref(a), C.byref(b)))
    return a.value, b.value


class SurfaceGraph:
    """A surface for the learned preconditioner: one-ring adjacency and static vertex features."""

    def __init__(self, faces, positions, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        faces, positions = _mesh(faces, positions)
        self.n_vertices = len(positions)
        h = _vp()
        _check(_lib.rs_lgraph_create(self.ctx.handle, len(positions), len(faces), faces.ravel(),
                                     positions.ravel(), C.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.rs_lgraph_free(self._h)
            self._h = None


class LearnedModel:
    """The learned preconditioner network (parameters, Adam state) on the device."""

    def __init__(self, seed: int = 0, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        h = _vp()
        _check(_lib.rs_learned_create(self.ctx.handle, seed, C.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.rs_learned_free(self._h)
            self._h = None

    @property
    def n_parameters(self) -> int:
        n = C.c_int64()
        _check(_lib.rs_learned_parameter_count(self._h, C.byref(n)))
        return n.value

    def get_parameters(self) -> np.ndarray:
        w = np.empty(self.n_parameters, np.float32)
        _check(_lib.rs_learned_get_parameters(self._h, w))
        return w

    def get_gradient(self) -> np.ndarray:
        g = np.empty(self.n_parameters, np.float32)
        _check(_lib.rs_learned_get_gradient(self._h, g))
        return g

    def set_parameters(self, w) -> None:
        w = np.ascontiguousarray(w, dtype=np.float32)
        if w.size != self.n_parameters:
            raise ValueError(f"expected {self.n_parameters} parameters, got {w.size}")
        _check(_lib.rs_learned_set_parameters(self._h, w))

    def apply_device(self, graph: SurfaceGraph, nb: int, r_ptr: int, y_ptr: int, z_ptr: int) -> None:
        _check(_lib.rs_learned_apply_device(self._h, graph._h, nb, _vp(r_ptr), _vp(y_ptr), _vp(z_ptr)))

    def loss_and_gradient_device(self, graph: SurfaceGraph, r_ptr: int, y_ptr: int, zt_ptr: int) -> float:
        out = C.c_double()
        _check(_lib.rs_learned_loss_and_gradient_device(self._h, graph._h, _vp(r_ptr), _vp(y_ptr), _vp(zt_ptr),
                                                        C.byref(out)))
        return out.value

    def adam_step(self, lr: float = 1e-3, clip: float = 1.0) -> None:
        _check(_lib.rs_learned_adam_step(self._h, lr, clip))
