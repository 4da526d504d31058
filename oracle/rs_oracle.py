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
