"""ctypes wrapper of the FP64 CPU oracle (``oracle/_build/librs_oracle.so``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py``, as the checker. The product path (``rs_gb300``) never
imports this module.

The oracle restates the reference crate ``ddg-repulsive-surfaces`` in double precision;
each C entry point cites the reference file:line it follows (``oracle/rs_oracle.h``).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "librs_oracle.so"

_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")


class OracleError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code
        self.message = message


def build() -> Path:
    """Compiles the oracle with its Makefile (g++, a few seconds)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = C.CDLL(str(LIB_PATH))
        L.rso_last_error.restype = C.c_char_p
        L.rso_set_threads.argtypes = [C.c_int]
        L.rso_exponents_check.argtypes = [C.c_double, C.c_double]
        L.rso_face_geometry.argtypes = [C.c_int, _f64p, C.c_int, _u32p, _f64p, _f64p, _f64p]
        L.rso_exact_energy.argtypes = [C.c_int, _f64p, C.c_int, _u32p, C.c_double, C.c_double,
                                       C.POINTER(C.c_double), C.c_void_p, C.c_void_p]
        L.rso_bh_build.argtypes = [C.c_int, _f64p, C.c_int, _u32p, C.c_double, C.c_int,
                                   C.POINTER(C.c_void_p)]
        L.rso_bh_free.argtypes = [C.c_void_p]
        L.rso_bh_refit.argtypes = [C.c_void_p, _f64p]
        L.rso_bh_sizes.argtypes = [C.c_void_p, _i64p]
        L.rso_bh_tree.argtypes = [C.c_void_p, _u32p, _u32p, _u32p, _u32p, _u32p]
        L.rso_bh_clusters.argtypes = [C.c_void_p, _f64p, _f64p, _f64p, _f64p, _f64p]
        L.rso_bh_lists.argtypes = [C.c_void_p, _i64p, _u32p, _i64p, _u32p]
        L.rso_bh_energy.argtypes = [C.c_void_p, C.c_double, C.c_double, C.POINTER(C.c_double)]
        L.rso_bh_energy_and_differential.argtypes = [C.c_void_p, C.c_double, C.c_double,
                                                     C.POINTER(C.c_double), C.c_void_p, C.c_void_p]
        L.rso_pull_back.argtypes = [C.c_int, _f64p, C.c_int, _u32p, _f64p, _f64p]
        _lib = L
        threads = int(os.environ.get("RS_ORACLE_THREADS", "0")) or (os.cpu_count() or 1)
        L.rso_set_threads(threads)
    return _lib


def set_threads(n: int) -> None:
    lib().rso_set_threads(int(n))


def _check(code: int) -> None:
    if code != 0:
        raise OracleError(code, lib().rso_last_error().decode())


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _mesh(pos, faces):
    pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
    faces = np.ascontiguousarray(faces, dtype=np.uint32).reshape(-1, 3)
    return pos, faces


def exponents_check(alpha: float, beta: float) -> None:
    _check(lib().rso_exponents_check(alpha, beta))


def face_geometry(pos, faces):
    pos, faces = _mesh(pos, faces)
    nf = len(faces)
    a = np.empty(nf)
    n = np.empty((nf, 3))
    x = np.empty((nf, 3))
    _check(lib().rso_face_geometry(len(pos), pos.ravel(), nf, faces.ravel(), a, n.ravel(), x.ravel()))
    return a, n, x


def exact_energy(pos, faces, alpha=6.0, beta=12.0, gradient=True, partials=False):
    """Exact all-pairs energy; returns E, or (E, dE[V,3]) / (E, dE, partials[F,7])."""
    pos, faces = _mesh(pos, faces)
    e = C.c_double()
    dE = np.empty((len(pos), 3)) if gradient else None
    p7 = np.empty((len(faces), 7)) if partials else None
    _check(lib().rso_exact_energy(len(pos), pos.ravel(), len(faces), faces.ravel(), alpha, beta,
                                  C.byref(e), _ptr(dE), _ptr(p7)))
    if not gradient and not partials:
        return e.value
    if partials:
        return e.value, dE, p7
    return e.value, dE


def pull_back(pos, faces, partials7):
    pos, faces = _mesh(pos, faces)
    p7 = np.ascontiguousarray(partials7, dtype=np.float64)
    out = np.empty((len(pos), 3))
    _check(lib().rso_pull_back(len(pos), pos.ravel(), len(faces), faces.ravel(), p7.ravel(), out.ravel()))
    return out


class BhTree:
    """The oracle's Barnes-Hut evaluator (``BhTree`` of RS/src/energy/barnes_hut.rs:114-195)."""

    def __init__(self, pos, faces, theta=0.5, leaf_size=8):
        pos, faces = _mesh(pos, faces)
        self.nv, self.nf = len(pos), len(faces)
        self.faces = faces
        h = C.c_void_p()
        _check(lib().rso_bh_build(self.nv, pos.ravel(), self.nf, faces.ravel(), float(theta),
                                  int(leaf_size), C.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.rso_bh_free(self._h)
            self._h = None

    def refit(self, pos):
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        _check(lib().rso_bh_refit(self._h, pos.ravel()))

    def sizes(self) -> dict:
        o = np.zeros(6, dtype=np.int64)
        _check(lib().rso_bh_sizes(self._h, o))
        keys = ["n_nodes", "n_leaves", "n_lumped", "n_exact", "n_partner", "pairs_exact"]
        return dict(zip(keys, (int(x) for x in o)))

    def tree(self) -> dict:
        s = self.sizes()
        nn, nl = s["n_nodes"], s["n_leaves"]
        start, end, right = (np.empty(nn, np.uint32) for _ in range(3))
        order = np.empty(self.nf, np.uint32)
        leaves = np.empty(nl, np.uint32)
        _check(lib().rso_bh_tree(self._h, start, end, right, order, leaves))
        return dict(start=start, end=end, right=right, order=order, leaves=leaves)

    def clusters(self) -> dict:
        nn = self.sizes()["n_nodes"]
        bbox = np.empty((nn, 6))
        radius, area = np.empty(nn), np.empty(nn)
        centroid, proj = np.empty((nn, 3)), np.empty((nn, 6))
        _check(lib().rso_bh_clusters(self._h, bbox.ravel(), radius, area, centroid.ravel(), proj.ravel()))
        return dict(bbox=bbox, radius=radius, area=area, centroid=centroid, projector=proj)

    def lists(self) -> dict:
        s = self.sizes()
        nl = s["n_leaves"]
        lo = np.empty(nl + 1, np.int64)
        eo = np.empty(nl + 1, np.int64)
        lum = np.empty(s["n_lumped"], np.uint32)
        ex = np.empty(s["n_exact"], np.uint32)
        _check(lib().rso_bh_lists(self._h, lo, lum, eo, ex))
        return dict(lumped_off=lo, lumped=lum, exact_off=eo, exact=ex)

    def energy(self, alpha=6.0, beta=12.0) -> float:
        e = C.c_double()
        _check(lib().rso_bh_energy(self._h, alpha, beta, C.byref(e)))
        return e.value

    def energy_and_differential(self, alpha=6.0, beta=12.0, partials=False):
        e = C.c_double()
        dE = np.empty((self.nv, 3))
        p7 = np.empty((self.nf, 7)) if partials else None
        _check(lib().rso_bh_energy_and_differential(self._h, alpha, beta, C.byref(e), _ptr(dE), _ptr(p7)))
        return (e.value, dE, p7) if partials else (e.value, dE)


def _metric_lib():
    L = lib()
    if not getattr(L, "_metric_ready", False):
        L.rso_metric_build.argtypes = [C.c_int, _f64p, C.c_int, _u32p, C.c_double, C.c_double,
                                       C.c_double, C.c_int, C.c_int, C.POINTER(C.c_void_p)]
        L.rso_metric_free.argtypes = [C.c_void_p]
        L.rso_metric_last_error.restype = C.c_char_p
        L.rso_metric_stats.argtypes = [C.c_void_p, _i64p]
        L.rso_metric_blocks.argtypes = [C.c_void_p, _i64p, _u32p, _f64p, _i64p, _u32p]
        L.rso_metric_ha.argtypes = [C.c_void_p, _f64p]
        L.rso_metric_apply.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_int, _f64p, _f64p]
        L.rso_vfrac_build.argtypes = [C.c_int, _f64p, _f64p, C.c_double, C.c_double, C.c_int, C.c_int,
                                      C.POINTER(C.c_void_p)]
        L.rso_vfrac_free.argtypes = [C.c_void_p]
        L.rso_vfrac_stats.argtypes = [C.c_void_p, _i64p]
        L.rso_vfrac_apply.argtypes = [C.c_void_p, C.c_int, _f64p, _f64p]
        L._metric_ready = True
    return L


def _mcheck(code: int) -> None:
    if code != 0:
        raise OracleError(code, _metric_lib().rso_metric_last_error().decode())


class FaceMetricTree:
    """The oracle's hierarchical B~ + B~0 (FaceMetricTree, RS/src/metric/hierarchical.rs)."""

    def __init__(self, pos, faces, alpha=6.0, beta=12.0, chi=0.5, leaf_size=8, leaf_pairs=64):
        pos, faces = _mesh(pos, faces)
        self.nv, self.nf = len(pos), len(faces)
        h = C.c_void_p()
        _mcheck(_metric_lib().rso_metric_build(self.nv, pos.ravel(), self.nf, faces.ravel(), alpha, beta,
                                               chi, leaf_size, leaf_pairs, C.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.rso_metric_free(self._h)
            self._h = None

    def stats(self) -> dict:
        o = np.zeros(5, np.int64)
        _mcheck(_metric_lib().rso_metric_stats(self._h, o))
        return dict(zip(["far_blocks", "near_blocks", "near_entries", "depth", "nodes"], map(int, o)))

    def blocks(self) -> dict:
        s = self.stats()
        nn = s["nodes"]
        fp, np_ = np.empty(nn + 1, np.int64), np.empty(nn + 1, np.int64)
        fc = np.empty(max(s["far_blocks"], 1), np.uint32)
        coef = np.empty(2 * max(s["far_blocks"], 1))
        nc = np.empty(max(s["near_blocks"], 1), np.uint32)
        _mcheck(_metric_lib().rso_metric_blocks(self._h, fp, fc, coef, np_, nc))
        return dict(far_ptr=fp, far_col=fc[: s["far_blocks"]],
                    far_coef=coef[: 2 * s["far_blocks"]].reshape(-1, 2), near_ptr=np_,
                    near_col=nc[: s["near_blocks"]])

    def ha(self):
        out = np.empty((self.nf, 2))
        _mcheck(_metric_lib().rso_metric_ha(self._h, out.ravel()))
        return out

    def apply(self, x, w_hi=1.0, w_lo=1.0):
        """y = (w_hi B~ + w_lo B~0) x for x of shape (3V,) or (nb, 3V)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        xs = x.reshape(-1, 3 * self.nv)
        ys = np.empty_like(xs)
        _mcheck(_metric_lib().rso_metric_apply(self._h, w_hi, w_lo, len(xs), xs.ravel(), ys.ravel()))
        return ys.reshape(x.shape)


class VertexFractionalTree:
    """The oracle's vertex-pair L^V_tau (VertexFractionalTree, RS/src/metric/hierarchical.rs)."""

    def __init__(self, pos, mass, tau, chi=0.5, leaf_size=8, leaf_pairs=64):
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        mass = np.ascontiguousarray(mass, dtype=np.float64)
        self.nv = len(pos)
        h = C.c_void_p()
        _mcheck(_metric_lib().rso_vfrac_build(self.nv, pos.ravel(), mass, tau, chi, leaf_size, leaf_pairs,
                                              C.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.rso_vfrac_free(self._h)
            self._h = None

    def stats(self) -> dict:
        o = np.zeros(5, np.int64)
        _mcheck(_metric_lib().rso_vfrac_stats(self._h, o))
        return dict(zip(["far_blocks", "near_blocks", "near_entries", "depth", "nodes"], map(int, o)))

    def apply(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        xs = x.reshape(-1, 3 * self.nv)
        ys = np.empty_like(xs)
        _mcheck(_metric_lib().rso_vfrac_apply(self._h, len(xs), xs.ravel(), ys.ravel()))
        return ys.reshape(x.shape)


def ccd_first_contact(faces, start, velocity, tau_end, gap=0.05, reference_length=0.0, max_iterations=100,
                      close_factor=0.5, band=False) -> dict:
    """first_contact of the mesh moving as start + t velocity on [0, tau_end], against itself
    (RS/src/ccd.rs:762-884; no obstacles); with band, the exempt band of the start positions
    (first_contact_with_band). reference_length 0: the mean edge length of start."""
    start, faces = _mesh(start, faces)
    vel = np.ascontiguousarray(velocity, dtype=np.float64).reshape(-1, 3)
    L = lib()
    L.rso_ccd_first_contact.argtypes = [C.c_int, _f64p, C.c_int, _u32p, _f64p, C.c_double, C.c_double,
                                        C.c_double, C.c_int, C.c_double, C.c_int, C.POINTER(C.c_double), _i64p]
    L.rso_ccd_last_error.restype = C.c_char_p
    tau = C.c_double()
    out = np.zeros(7, np.int64)
    code = L.rso_ccd_first_contact(len(start), start.ravel(), len(faces), faces.ravel(), vel.ravel(),
                                   float(tau_end), float(gap), float(reference_length), int(max_iterations),
                                   float(close_factor), int(bool(band)), C.byref(tau), out)
    if code != 0:
        raise OracleError(code, L.rso_ccd_last_error().decode())
    keys = ["contact", "windows", "pairs_tested", "close_pairs", "touching_pairs", "exempt_pairs",
            "band_vertices"]
    return {"tau_max": tau.value, **{k: int(v) for k, v in zip(keys, out)}}


def ccd_min_distance(pos, faces) -> float:
    """The smallest distance over the vertex-triangle and edge-edge pairs CCD constrains."""
    pos, faces = _mesh(pos, faces)
    L = lib()
    L.rso_ccd_min_distance.argtypes = [C.c_int, _f64p, C.c_int, _u32p, C.POINTER(C.c_double)]
    d = C.c_double()
    code = L.rso_ccd_min_distance(len(pos), pos.ravel(), len(faces), faces.ravel(), C.byref(d))
    if code != 0:
        raise OracleError(code, L.rso_ccd_last_error().decode())
    return d.value


def ccd_intersecting_pairs(pos, faces) -> np.ndarray:
    """The intersecting face pairs (f < g), sorted (intersecting_pairs, RS/src/ccd.rs:1229-1279)."""
    pos, faces = _mesh(pos, faces)
    L = lib()
    L.rso_ccd_intersecting_pairs.argtypes = [C.c_int, _f64p, C.c_int, _u32p, C.c_int64, _u32p,
                                             C.POINTER(C.c_int64)]
    n = C.c_int64()
    out = np.zeros(2 * max(len(faces), 16), np.uint32)
    code = L.rso_ccd_intersecting_pairs(len(pos), pos.ravel(), len(faces), faces.ravel(), len(out) // 2, out,
                                        C.byref(n))
    if code != 0:
        raise OracleError(code, L.rso_ccd_last_error().decode())
    if n.value > len(out) // 2:
        out = np.zeros(2 * n.value, np.uint32)
        L.rso_ccd_intersecting_pairs(len(pos), pos.ravel(), len(faces), faces.ravel(), n.value, out, C.byref(n))
    return out[: 2 * n.value].reshape(-1, 2)


# ---------------------------------------------------------------- constraints, solves, the step


class _RsoConstraints(C.Structure):
    _fields_ = [("n", C.c_int), ("kind", C.c_void_p), ("comp", C.c_void_p), ("n_target", C.c_void_p),
                ("target", C.c_void_p), ("n_pin", C.c_void_p), ("pin", C.c_void_p), ("per_component", C.c_int)]


class SolverOptions(C.Structure):
    """rso_solver_options (HierarchicalOptions / PreconditionerOptions / GmresOptions)."""
    _fields_ = [("chi", C.c_double), ("leaf_size", C.c_int), ("leaf_pairs", C.c_int), ("tp_weight", C.c_double),
                ("low_order", C.c_int), ("eps_rel", C.c_double), ("eps_multi_rel", C.c_double),
                ("preconditioner", C.c_int), ("coarse", C.c_int), ("restart", C.c_int),
                ("max_iterations", C.c_int), ("tolerance", C.c_double)]


class StepOptions(C.Structure):
    """rso_step_options (FlowOptions of one step)."""
    _fields_ = [("energy_theta", C.c_double), ("leaf_size", C.c_int), ("backend", C.c_int),
                ("solver", SolverOptions), ("start_rule", C.c_int), ("start_value", C.c_double),
                ("first_rule", C.c_int), ("first_value", C.c_double), ("previous_tau", C.c_double),
                ("armijo_c", C.c_double), ("max_halvings", C.c_int), ("tau_min_rel", C.c_double),
                ("newton_fixed", C.c_int), ("newton_max", C.c_int), ("guard_projection", C.c_int),
                ("l0", C.c_double)]


def _solve_lib():
    L = lib()
    if not getattr(L, "_solve_ready", False):
        L.rso_solve_last_error.restype = C.c_char_p
        L.rso_solver_options_default.restype = SolverOptions
        L.rso_step_options_default.restype = StepOptions
        cp = C.POINTER(_RsoConstraints)
        L.rso_constraint_rows.argtypes = [C.c_int, _f64p, C.c_int, _u32p, cp, C.c_int, C.POINTER(C.c_int),
                                          C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.POINTER(C.c_int)]
        L.rso_dense_saddle.argtypes = [C.c_int, _f64p, C.c_int, _u32p, C.c_double, C.c_double, C.c_double,
                                       C.c_int, cp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), _f64p,
                                       _f64p, _f64p, _f64p, _f64p, C.POINTER(C.c_double)]
        L.rso_dense_precond.argtypes = [C.c_int, _f64p, C.c_int, _u32p, C.c_double, C.c_double, C.c_double,
                                        cp, _f64p, C.POINTER(C.c_double), _f64p, _f64p, _f64p,
                                        C.POINTER(C.c_int)]
        L.rso_step.argtypes = [C.c_int, _f64p, C.c_int, _u32p, C.c_double, C.c_double, cp,
                               C.POINTER(StepOptions), _f64p, _f64p, _f64p, _f64p, _f64p, C.c_int,
                               C.POINTER(C.c_int), _f64p, _f64p, C.c_int]
        L.rso_hsolver_build.argtypes = [C.c_int, _f64p, C.c_int, _u32p, C.c_double, C.c_double,
                                        C.POINTER(SolverOptions), cp, C.POINTER(C.c_void_p)]
        L.rso_hsolver_free.argtypes = [C.c_void_p]
        L.rso_hsolver_dims.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        L.rso_hsolver_set_gmres.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double]
        for f in ("rso_hsolver_apply", "rso_hsolver_precondition"):
            getattr(L, f).argtypes = [C.c_void_p, C.c_int, _f64p, _f64p]
        L.rso_hsolver_solve.argtypes = [C.c_void_p, C.c_int, _f64p, _f64p, _f64p]
        L.rso_hsolver_info.argtypes = [C.c_void_p, _f64p]
        L._solve_ready = True
    return L


def _scheck(code: int) -> None:
    if code != 0:
        raise OracleError(code, _solve_lib().rso_solve_last_error().decode())


KINDS = {"barycenter": 0, "pins": 1, "area": 2, "volume": 3}


class Constraints:
    """A constraint list (Constraint, RS/src/constraints/mod.rs:36-110), in order.

    ``barycenter(comp=None)`` with ``per_component`` holds every component's barycenter
    separately (BarycenterMode::PerComponent), else one global group."""

    def __init__(self, per_component: bool = False):
        self.items: list[tuple[int, int, list[float], list[int]]] = []
        self.per_component = per_component

    def barycenter(self, comp=None, target=None):
        self.items.append((0, -1 if comp is None else comp, [] if target is None else list(target), []))
        return self

    def pins(self, vertices, targets=None):
        t = [] if targets is None else list(np.asarray(targets, dtype=np.float64).ravel())
        self.items.append((1, -1, t, [int(v) for v in vertices]))
        return self

    def area(self, comp=None, target=None):
        self.items.append((2, -1 if comp is None else comp, [] if target is None else [float(target)], []))
        return self

    def volume(self, comp=None, target=None):
        self.items.append((3, -1 if comp is None else comp, [] if target is None else [float(target)], []))
        return self

    def _c(self):
        n = len(self.items)
        self._kind = np.array([i[0] for i in self.items] or [0], np.int32)
        self._comp = np.array([i[1] for i in self.items] or [0], np.int32)
        self._nt = np.array([len(i[2]) for i in self.items] or [0], np.int32)
        self._t = np.array([x for i in self.items for x in i[2]] or [0.0], np.float64)
        self._npin = np.array([len(i[3]) for i in self.items] or [0], np.int32)
        self._pin = np.array([x for i in self.items for x in i[3]] or [0], np.uint32)
        s = _RsoConstraints(n, self._kind.ctypes.data, self._comp.ctypes.data, self._nt.ctypes.data,
                            self._t.ctypes.data, self._npin.ctypes.data, self._pin.ctypes.data,
                            int(self.per_component))
        self._s = s
        return C.byref(s)


def solver_options(**kw) -> SolverOptions:
    o = _solve_lib().rso_solver_options_default()
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def step_options(**kw) -> StepOptions:
    o = _solve_lib().rso_step_options_default()
    for k, v in kw.items():
        if k == "solver":
            for kk, vv in v.items():
                setattr(o.solver, kk, vv)
        else:
            setattr(o, k, v)
    return o


def constraint_rows(pos, faces, cons: Constraints) -> dict:
    """Rows of the constraint set: kind, positional flag, Phi, dense Jacobian, components."""
    pos, faces = _mesh(pos, faces)
    L = _solve_lib()
    nv = len(pos)
    cap = 3 * nv + 64
    nr, ncomp = C.c_int(), C.c_int()
    kind, posi = np.zeros(cap, np.int32), np.zeros(cap, np.int32)
    phi, jac = np.zeros(cap), np.zeros(cap * 3 * nv)
    vcomp = np.zeros(nv, np.uint32)
    _scheck(L.rso_constraint_rows(nv, pos.ravel(), len(faces), faces.ravel(), cons._c(), cap, C.byref(nr),
                                  _ptr(kind), _ptr(posi), _ptr(phi), _ptr(jac), _ptr(vcomp), C.byref(ncomp)))
    n = nr.value
    return dict(kind=kind[:n], positional=posi[:n].astype(bool), phi=phi[:n], jac=jac[: n * 3 * nv].reshape(n, 3 * nv),
                vcomp=vcomp, n_components=ncomp.value)


def dense_saddle(pos, faces, cons: Constraints, alpha=6.0, beta=12.0, tp_weight=1.0, low_order=True) -> dict:
    """The dense nested saddle at the exact energy gradient: g, x, S, Phi_N, h, <g, x>."""
    pos, faces = _mesh(pos, faces)
    L = _solve_lib()
    nv = len(pos)
    kq, kn, gx = C.c_int(), C.c_int(), C.c_double()
    g, x, h = np.zeros(3 * nv), np.zeros(3 * nv), np.zeros(3 * nv)
    S, phin = np.zeros(64 * 64), np.zeros(64)
    _scheck(L.rso_dense_saddle(nv, pos.ravel(), len(faces), faces.ravel(), alpha, beta, tp_weight, int(low_order),
                               cons._c(), 64, C.byref(kq), C.byref(kn), g, x, S, phin, h, C.byref(gx)))
    k = kn.value
    return dict(kq=kq.value, kn=k, g=g.reshape(-1, 3), x=x.reshape(-1, 3), S=S[: k * k].reshape(k, k),
                phin=phin[:k], h=h.reshape(-1, 3), gx=gx.value)


def dense_precond(pos, faces, cons: Constraints, r, alpha=6.0, beta=12.0, eps_rel=1e-10) -> dict:
    """The dense face-pair preconditioner: eps, L_{2-s}, L', z = P^-1 [r; 0]."""
    pos, faces = _mesh(pos, faces)
    L = _solve_lib()
    nv = len(pos)
    cap = 3 * nv + 3 * nv
    eps, kq = C.c_double(), C.c_int()
    lfr, lp, z = np.zeros(nv * nv), np.zeros(cap * cap), np.zeros(3 * nv)
    r = np.ascontiguousarray(r, dtype=np.float64).ravel()
    _scheck(L.rso_dense_precond(nv, pos.ravel(), len(faces), faces.ravel(), alpha, beta, eps_rel, cons._c(), r,
                                C.byref(eps), lfr, lp, z, C.byref(kq)))
    n = 3 * nv + kq.value
    return dict(eps=eps.value, Lfr=lfr.reshape(nv, nv), Lp=lp[: n * n].reshape(n, n), z=z.reshape(-1, 3),
                kq=kq.value)


STEP_KEYS = ["energy_before", "energy_after", "energy_trial", "tau", "tau0", "accepted", "halvings", "slope",
             "xnorm", "xinf", "l0", "newton_rounds", "projection_status", "gradient_norm", "rows",
             "projection_blocked", "s_objective", "s_energy", "s_solver_build", "s_solve", "s_line_search",
             "s_projection", "s_total", "operator_products", "gmres_iterations", "worst_residual", "solves",
             "preconditioner_applications"]
OUTCOMES = ["accepted", "armijo-failed", "non-finite", "projection-blocked"]


def step(pos, faces, cons: Constraints, options: StepOptions | None = None, alpha=6.0, beta=12.0) -> dict:
    """One descent step (Session::step_inner): report, trials, positions, direction, gradient,
    Phi of every row after the line search and at the end."""
    pos, faces = _mesh(pos, faces)
    L = _solve_lib()
    nv = len(pos)
    o = options if options is not None else L.rso_step_options_default()
    rep = np.zeros(28)
    trials = np.zeros(3 * 256)
    nt = C.c_int()
    cap = 3 * nv + 64
    pb, pa = np.zeros(cap), np.zeros(cap)
    P, x, g = np.zeros(3 * nv), np.zeros(3 * nv), np.zeros(3 * nv)
    _scheck(L.rso_step(nv, pos.ravel(), len(faces), faces.ravel(), alpha, beta, cons._c(), C.byref(o), P, x, g,
                       rep, trials, 256, C.byref(nt), pb, pa, cap))
    out = dict(zip(STEP_KEYS, rep.tolist()))
    nr = int(out["rows"])
    out.update(positions=P.reshape(-1, 3), direction=x.reshape(-1, 3), gradient=g.reshape(-1, 3),
               trials=[(trials[3 * i], trials[3 * i + 1], OUTCOMES[int(trials[3 * i + 2])])
                       for i in range(min(nt.value, 256))],
               phi_before=pb[:nr], phi_after=pa[:nr])
    return out


class HSolver:
    """The hierarchical saddle solver (A', the augmented preconditioner, GMRES) of the oracle."""

    def __init__(self, pos, faces, cons: Constraints, options: SolverOptions | None = None, alpha=6.0, beta=12.0):
        pos, faces = _mesh(pos, faces)
        L = _solve_lib()
        h = C.c_void_p()
        o = options if options is not None else L.rso_solver_options_default()
        _scheck(L.rso_hsolver_build(len(pos), pos.ravel(), len(faces), faces.ravel(), alpha, beta, C.byref(o),
                                    cons._c(), C.byref(h)))
        self._h = h
        nd, nq = C.c_int64(), C.c_int64()
        L.rso_hsolver_dims(h, C.byref(nd), C.byref(nq))
        self.n_dofs, self.n_constraints = nd.value, nq.value
        self.n = self.n_dofs + self.n_constraints

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.rso_hsolver_free(self._h)
            self._h = None

    def info(self) -> dict:
        o = np.zeros(8)
        _solve_lib().rso_hsolver_info(self._h, o)
        return dict(zip(["eps", "multi", "fractional_scale", "coarse_dim", "s_metric", "s_fractional",
                         "s_laplacian", "s_coarse"], o.tolist()))

    def set_gmres(self, restart=30, max_iterations=200, tolerance=1e-6):
        _solve_lib().rso_hsolver_set_gmres(self._h, restart, max_iterations, tolerance)

    def _batch(self, fn, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        xs = x.reshape(-1, self.n)
        ys = np.empty_like(xs)
        _scheck(fn(self._h, len(xs), xs.ravel(), ys.ravel()))
        return ys.reshape(x.shape)

    def apply(self, x):
        return self._batch(_solve_lib().rso_hsolver_apply, x)

    def precondition(self, r):
        return self._batch(_solve_lib().rso_hsolver_precondition, r)

    def solve(self, rhs):
        rhs = np.ascontiguousarray(rhs, dtype=np.float64)
        rs = rhs.reshape(-1, self.n)
        sol = np.empty_like(rs)
        rep = np.zeros(5 * len(rs))
        _scheck(_solve_lib().rso_hsolver_solve(self._h, len(rs), rs.ravel(), sol.ravel(), rep))
        reps = [dict(iterations=int(rep[5 * q]), relative_residual=rep[5 * q + 1], converged=bool(rep[5 * q + 2]),
                     seconds=rep[5 * q + 3], cycles=int(rep[5 * q + 4])) for q in range(len(rs))]
        return sol.reshape(rhs.shape), reps
