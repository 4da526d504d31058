"""The Repulsive Surfaces functions of the ``ddg_tools`` Python module, on the GPU.

Same names, keyword options, array conventions and report dicts as the reference's glue
(crates/ddg-py/src/python/repulsive_surfaces.rs:400-710) and its option and report code
(crates/ddg-py/src/repulsive_surfaces.rs:684-1415, 1626-1995):

* ``surface_energy(positions, faces, **options) -> (energy, differential, report)``;
* ``RepulsiveSurfaceSession(positions, faces, **options)`` with ``step``, ``run``,
  ``snapshot``, ``cancel``, ``reset`` and the getters;
* ``repulsive_surface_flow(positions, faces, steps=None, progress=None, **options)``;
* ``repulsive_surface_defaults()``, ``gpu_info()`` and ``repulsive_surface_scene(path)`` (the
  statements of a scene file that are on this path).

Positions are any buffer or (nested) sequence of 3 reals per vertex, faces 3 indices per face;
results are ``array('d')`` / ``array('i')``. Every option name of the reference is known. The
values this library runs are the GPU hot path of one Hs step: the tangent-point energy
(Barnes-Hut or exact), the Sobolev metric with the hierarchical solver and right-preconditioned
GMRES, projected gradient descent with the standard Armijo line search and its continuous
collision detection cap, and the barycenter, total-area and total-volume constraints held at
their initial values. A value outside that path (remeshing, penalties, obstacles, pins,
schedules, the other energies,
metrics, back ends and methods, ``device="cpu"``) raises ``RepulsiveSurfaceInputError`` naming
the option, as the reference does for a value outside an option's domain. There is no CPU
fallback.
"""
from __future__ import annotations

import array
import math
import threading
import time
from collections import deque

import numpy as np

from . import (PROJECTION_STATUS, BhOptions, BhTree, Context, Exponents, Flow, RsError, device_count,
               device_info, flow_options, load_library)


class DdgError(Exception):
    """Base class of the errors raised by ddg_tools (crates/ddg-py/src/python.rs:36-41)."""


class InputError(DdgError):
    """An argument is malformed or an option is outside its domain; the message starts with the
    name of the parameter."""


class SolveError(DdgError):
    """The input was accepted but the computation failed (non-finite energy, diverged solve)."""


class RepulsiveSurfaceInputError(InputError, ValueError):
    """An argument or an option of the repulsive-surfaces functions is invalid. Both an
    InputError and a ValueError; the message is the library's."""


def _bad(name: str, message) -> RepulsiveSurfaceInputError:
    return RepulsiveSurfaceInputError(f"{name}: {message}")


# The crate's error kinds that the reference reports as a failed computation
# (crates/ddg-py/src/repulsive_surfaces.rs:76-87); every other kind is an input error.
_SOLVE_KINDS = {"NonFiniteEnergy", "SingularSaddle", "SolverDiverged", "Internal", "Cancelled"}


def _lib_err(e: RsError) -> Exception:
    if e.kind in _SOLVE_KINDS:
        return SolveError(str(e))
    return RepulsiveSurfaceInputError(str(e))


# ----------------------------------------------------------------------------------------------
# Options
# ----------------------------------------------------------------------------------------------

REMESH_OPS = ["split", "collapse", "flip", "smooth"]

# Every option of the reference (OPTION_NAMES, crates/ddg-py/src/repulsive_surfaces.rs:684-753)
# with this library's default. The defaults equal the reference's except where the reference's
# default is outside the GPU path: device "cuda" (reference "cpu"), backend "hierarchical"
# (reference "auto", dense below 1000 faces) and remesh False (reference True).
_DEFAULTS = {
    "alpha": 6.0, "beta": 12.0, "energy": "tangent_point", "coulomb_alpha": None, "tp_weight": 1.0,
    "metric": "sobolev", "low_order": True, "l2_kind": "mass", "backend": "hierarchical",
    "dense_max_faces": 1000, "energy_eval": "barnes_hut", "theta": 0.5, "leaf_size": 8, "chi": 0.5,
    "cluster_leaf_size": 8, "gmres_restart": 60, "gmres_tolerance": 1e-3, "gmres_max_iterations": 200,
    "gmres_side": "right", "device": "cuda", "cuda_ordinal": 0, "gpu_determinism": "run_to_run",
    "method": "projected_gradient", "aqp_kappa": 100.0, "lbfgs_memory": 10, "lbfgs_variant": "standard",
    "constraints": None, "barycenter": None, "barycenter_mode": "auto", "barycenter_shift": False,
    "pins": None, "pin_targets": None, "pin_move": None, "pin_move_steps": None,
    "schedule_timing": "before_projection", "penalties": None, "ccd_obstacles": None,
    "armijo": "standard", "armijo_c": 1e-2, "start": "grow_previous", "start_lengths": 1.0,
    "start_factor": 2.0, "start_tau": None, "tau_min_rel": 1e-12, "max_halvings": None, "ccd": True,
    "ccd_gap": 0.05, "ccd_max_iterations": 100, "ccd_close_factor": 0.5, "newton_steps": None,
    "newton_max": 5, "remesh": False, "remesh_split": 1.5, "remesh_collapse": 0.5, "remesh_rounds": 5,
    "remesh_rho": 0.5, "remesh_flip_cap": 100, "remesh_order": "flip_then_smooth",
    "remesh_ops": list(REMESH_OPS), "stop": "energy_stall", "stop_relative": 1e-7, "stop_window": 10,
    "stop_eps": None, "max_iterations": 1000, "time_limit": None, "stuck_limit": 5, "threads": None,
    "reference_compat": False,
}
OPTION_NAMES = tuple(_DEFAULTS)

# Options whose only value on this path is the default: any other value raises.
_FIXED = {
    "energy": "tangent_point", "metric": "sobolev", "gmres_side": "right", "method": "projected_gradient",
    "barycenter_shift": False, "armijo": "standard", "start": "grow_previous", "start_lengths": 1.0,
    "start_factor": 2.0, "tau_min_rel": 1e-12, "remesh": False, "reference_compat": False,
}
_ABSENT = ("pins", "pin_targets", "pin_move", "pin_move_steps", "penalties", "ccd_obstacles",
           "newton_steps", "start_tau")
_ENUMS = {
    "energy": ("tangent_point", "coulomb", "willmore"), "metric": ("sobolev", "l2", "h1", "h2"),
    "l2_kind": ("mass", "identity"), "backend": ("auto", "dense", "hierarchical"),
    "energy_eval": ("barnes_hut", "exact"), "gmres_side": ("right", "left"),
    "device": ("cpu", "cuda", "auto"), "gpu_determinism": ("run_to_run", "match_cpu"),
    "method": ("projected_gradient", "aqp", "h1_lbfgs", "bcqn"), "lbfgs_variant": ("standard", "reference"),
    "barycenter_mode": ("auto", "global", "per_component"),
    "schedule_timing": ("before_projection", "after_projection"), "armijo": ("standard", "reference"),
    "start": ("grow_previous", "max_displacement", "reference", "absolute"),
    "remesh_order": ("flip_then_smooth", "smooth_then_flip"), "stop": ("energy_stall", "sobolev", "off"),
}
_REALS = ("alpha", "beta", "coulomb_alpha", "tp_weight", "theta", "chi", "gmres_tolerance", "aqp_kappa",
          "armijo_c", "start_lengths", "start_factor", "start_tau", "tau_min_rel", "ccd_gap",
          "ccd_close_factor", "remesh_split", "remesh_collapse", "remesh_rho", "stop_relative", "stop_eps",
          "time_limit")
_COUNTS = ("dense_max_faces", "leaf_size", "cluster_leaf_size", "gmres_restart", "gmres_max_iterations",
           "cuda_ordinal", "lbfgs_memory", "pin_move_steps", "max_halvings", "ccd_max_iterations",
           "newton_steps", "newton_max", "remesh_rounds", "remesh_flip_cap", "stop_window",
           "max_iterations", "stuck_limit", "threads")
_BOOLS = ("low_order", "barycenter", "barycenter_shift", "ccd", "remesh", "reference_compat")
_OFF_PATH = "is outside this library's GPU path"


def repulsive_surface_defaults() -> dict:
    """Every option with its default, as a dict; passing it back as keywords gives the default
    flow (repulsive_surface_defaults, crates/ddg-py/src/python/repulsive_surfaces.rs:678-685)."""
    d = dict(_DEFAULTS)
    d["remesh_ops"] = list(REMESH_OPS)
    return d


def _real(name, v):
    if isinstance(v, bool) or not isinstance(v, (int, float, np.integer, np.floating)):
        raise _bad(name, f"expected a number, got {type(v).__name__}")
    return float(v)


def _count(name, v):
    if isinstance(v, bool) or not isinstance(v, (int, np.integer)):
        raise _bad(name, f"expected an integer, got {type(v).__name__}")
    if v < 0:
        raise _bad(name, f"{v} must be >= 0")
    return int(v)


class _Options:
    """The options of one flow, checked (flow_options, crates/ddg-py/src/repulsive_surfaces.rs:766-1161)."""

    def __init__(self, options: dict, flow: bool = True):
        for k in options:
            if k not in _DEFAULTS:
                raise RepulsiveSurfaceInputError(
                    f"unknown option '{k}'; repulsive_surface_defaults() lists the options")
        o = dict(_DEFAULTS)
        for k, v in options.items():
            if v is None:
                if _DEFAULTS[k] is not None:
                    raise _bad(k, "None is not a valid value")
                continue
            if k in _REALS:
                v = _real(k, v)
                if not math.isfinite(v):
                    raise _bad(k, f"{v} must be finite")
            elif k in _COUNTS:
                v = _count(k, v)
            elif k in _BOOLS:
                if not isinstance(v, (bool, np.bool_)):
                    raise _bad(k, f"expected a bool, got {type(v).__name__}")
                v = bool(v)
            elif k in _ENUMS:
                if v not in _ENUMS[k]:
                    raise _bad(k, f"'{v}' is not valid; use {', '.join(_ENUMS[k])}")
            o[k] = v
        if o["remesh_ops"] is not None:
            if not isinstance(o["remesh_ops"], (list, tuple)):
                raise _bad("remesh_ops", f"expected a list of names, got {type(o['remesh_ops']).__name__}")
            for op in o["remesh_ops"]:
                if op not in REMESH_OPS:
                    raise _bad("remesh_ops", f"'{op}' is not valid; use split, collapse, flip, smooth")
        self.hold_area = self.hold_volume = False
        self.o = o
        if o["penalties"] is not None:
            raise _bad("penalties", f"{_OFF_PATH}: give None")
        if o["stop"] == "sobolev" and o["stop_eps"] is None:
            raise _bad("stop_eps", "required with stop='sobolev'")
        if o["energy"] == "coulomb" and o["coulomb_alpha"] is None:
            raise _bad("coulomb_alpha", "required with energy='coulomb'")
        try:
            Exponents(o["alpha"], o["beta"])
        except RsError as e:
            raise RepulsiveSurfaceInputError(f"alpha, beta: {e.detail}") from None
        if flow:
            self._flow_path()

    def _flow_path(self):
        """The values a flow on this library's GPU path runs (surface_energy reads only the
        exponents, the evaluation and the penalties, as the reference does)."""
        o = self.o
        for k, want in _FIXED.items():
            if o[k] != want:
                raise _bad(k, f"{o[k]!r} {_OFF_PATH} (it runs {want!r})")
        for k in _ABSENT:
            if o[k] is not None:
                raise _bad(k, f"{_OFF_PATH}: give None")
        if o["backend"] == "dense":
            raise _bad("backend", f"'dense' {_OFF_PATH}: 'hierarchical' or 'auto' run the hierarchical solver")
        if o["device"] == "cpu":
            raise _bad("device", "'cpu' is not served: this library runs on the GPU only; use 'cuda' or 'auto'")
        if o["gpu_determinism"] == "match_cpu":
            raise _bad("gpu_determinism", "'match_cpu' is outside this library's GPU path: its results are "
                                          "run-to-run deterministic ('run_to_run') but computed in compensated "
                                          "FP32, not bitwise the reference's FP64 CPU path")
        if o["barycenter_mode"] == "auto" and not o["low_order"]:
            # resolved_barycenter_mode (RS/src/step/options.rs:580-588): "auto" is per component
            # unless the metric is the Sobolev metric with its low-order term
            raise _bad("barycenter_mode", "'auto' with low_order=False resolves to per-component barycenters, "
                                          "which are outside this library's GPU path; give barycenter_mode='global'")
        if o["barycenter_mode"] == "per_component":
            raise _bad("barycenter_mode", f"'per_component' {_OFF_PATH}: the global barycenter is held")
        if o["barycenter"] is False:
            raise _bad("barycenter", f"False {_OFF_PATH}: the global barycenter is always held")
        if o["ccd"]:
            if not (o["ccd_gap"] > 0):
                raise _bad("ccd_gap", f"{o['ccd_gap']} must be finite and positive")
            if o["ccd_max_iterations"] < 1:
                raise _bad("ccd_max_iterations", "must be at least 1")
            if not (0.0 <= o["ccd_close_factor"] < 1.0):
                raise _bad("ccd_close_factor", f"{o['ccd_close_factor']} must be in [0, 1)")
        if o["time_limit"] is not None and o["time_limit"] < 0:
            raise _bad("time_limit", f"{o['time_limit']} must be finite and >= 0 seconds")
        if not (o["tp_weight"] > 0):
            raise _bad("tp_weight", f"{o['tp_weight']} must be finite and positive")
        if o["constraints"] is not None:
            self._constraints(o["constraints"])

    def _constraints(self, items):
        if not isinstance(items, (list, tuple)):
            raise _bad("constraints", f"expected a list of dicts, got {type(items).__name__}")
        has_bary = False
        for i, c in enumerate(items):
            what = f"constraints[{i}]"
            if not isinstance(c, dict):
                raise _bad(what, f"expected a dict, got {type(c).__name__}")
            kind = c.get("type", "")
            if kind not in ("barycenter", "pins", "area", "volume"):
                raise _bad(f"{what}.type", f"'{kind}' is not valid; use barycenter, pins, area, volume")
            allowed = {"type", "component", "target"} | ({"factor", "offset", "steps"} if kind in ("area", "volume") else set())
            if kind == "pins":
                raise _bad(what, f"pins {_OFF_PATH}")
            for k in c:
                if k not in allowed:
                    raise _bad(what, f"unknown key '{k}'")
            for k in ("component", "target", "factor", "offset", "steps"):
                if c.get(k) is not None:
                    raise _bad(f"{what}.{k}", f"{_OFF_PATH}: the constraint is held at its initial value over "
                                              "the whole surface")
            if kind == "barycenter":
                has_bary = True
            elif kind == "area":
                self.hold_area = True
            else:
                self.hold_volume = True
        if not has_bary:
            raise _bad("constraints", f"a list without the barycenter {_OFF_PATH}: the global barycenter is "
                                      "always held")

    def flow_options(self):
        o = self.o
        exact = o["energy_eval"] == "exact"
        fo = flow_options(alpha=o["alpha"], beta=o["beta"], theta=0.0 if exact else o["theta"],
                          leaf_size=o["leaf_size"], hold_area=int(self.hold_area),
                          hold_volume=int(self.hold_volume), armijo_c=o["armijo_c"],
                          max_halvings=10_000 if o["max_halvings"] is None else o["max_halvings"],
                          newton_max=o["newton_max"], ccd=int(o["ccd"]), ccd_gap=o["ccd_gap"],
                          ccd_max_iterations=o["ccd_max_iterations"], ccd_close_factor=o["ccd_close_factor"])
        s = fo.solver
        s.chi, s.leaf_size = o["chi"], o["cluster_leaf_size"]
        s.restart, s.tolerance, s.max_iterations = o["gmres_restart"], o["gmres_tolerance"], o["gmres_max_iterations"]
        s.tp_weight, s.low_order = o["tp_weight"], int(o["low_order"])
        return fo

    def bh(self) -> BhOptions:
        return BhOptions(theta=0.0 if self.o["energy_eval"] == "exact" else self.o["theta"],
                         leaf_size=self.o["leaf_size"])


def _mesh(positions, faces):
    """Positions (3 reals per vertex) and faces (3 indices per face) from a buffer or a nested
    sequence (mesh, crates/ddg-py/src/python/repulsive_surfaces.rs:88-176)."""
    try:
        p = np.asarray(positions, dtype=np.float64).ravel()
    except (TypeError, ValueError):
        raise _bad("positions", "expected an object with the buffer protocol or a sequence of numbers") from None
    if p.size % 3:
        raise _bad("positions", f"{p.size} numbers are not a whole number of vertexs of 3")
    bad = np.flatnonzero(~np.isfinite(p))
    if bad.size:
        raise _bad("positions", f"entry {int(bad[0])} is not finite")
    try:
        f = np.asarray(faces)
        if f.size and not np.issubdtype(f.dtype, np.integer):
            raise TypeError
        f = f.astype(np.int64).ravel()
    except (TypeError, ValueError):
        raise _bad("faces", "expected an object with the buffer protocol or a sequence of integers") from None
    if f.size % 3:
        raise _bad("faces", f"{f.size} indices are not a whole number of faces of 3")
    bad = np.flatnonzero((f < 0) | (f > 0xFFFFFFFF))
    if bad.size:
        raise _bad("faces", f"entry {int(bad[0])} = {int(f[bad[0]])} is not a valid index")
    return p.reshape(-1, 3).copy(), f.astype(np.uint32).reshape(-1, 3)


def _context(o: dict) -> Context:
    try:
        n = device_count()
    except RsError as e:
        raise _lib_err(e) from None
    if n == 0 or o["cuda_ordinal"] >= n:
        raise _bad("cuda_ordinal", f"{o['cuda_ordinal']}: the CUDA driver reports {n} device(s)")
    try:
        return Context(o["cuda_ordinal"])
    except RsError as e:
        raise _lib_err(e) from None


def _flat_points(p) -> array.array:
    return array.array("d", np.ascontiguousarray(p, dtype=np.float64).ravel().tobytes())


def _flat_faces(f) -> array.array:
    return array.array("i", np.ascontiguousarray(f, dtype=np.int32).ravel().tobytes())


# ----------------------------------------------------------------------------------------------
# Energy
# ----------------------------------------------------------------------------------------------

def surface_energy(positions, faces, **options):
    """The tangent-point energy of a mesh and its differential: ``(energy, differential,
    report)``; ``differential`` is an ``array('d')`` of 3 per vertex, ``report`` a dict with
    energy, total, penalties, subcritical, pairs_exact, nodes_lumped, seconds
    (surface_energy, crates/ddg-py/src/repulsive_surfaces.rs:1936-1978). Reads ``alpha``,
    ``beta``, ``energy_eval`` (``theta``, ``leaf_size``) and ``cuda_ordinal``; every other option
    is checked as the flow checks it and otherwise ignored."""
    p, f = _mesh(positions, faces)
    opts = _Options(options, flow=False)
    ctx = _context(opts.o)
    t0 = time.perf_counter()
    e = Exponents(opts.o["alpha"], opts.o["beta"])
    try:
        tree = BhTree.build(f, p, opts.bh(), ctx)
        E, dE = tree.energy_and_differential(e)
        s = tree.sizes()
    except RsError as err:
        raise _lib_err(err) from None
    report = {"energy": E, "total": E, "penalties": [], "subcritical": e.beta - e.alpha <= 4.0,
              "pairs_exact": int(s["pairs_exact"]), "nodes_lumped": int(s["n_lumped"]),
              "seconds": time.perf_counter() - t0}
    return E, _flat_points(dE), report


def gpu_info() -> dict:
    """What this library and machine offer for the ``device`` option: cuda_compiled,
    available, devices (ordinal, name, compute_capability, memory_bytes) and reason
    (gpu_info, crates/ddg-py/src/repulsive_surfaces.rs:1895-1938). Never raises."""
    try:
        load_library()
    except Exception as e:  # the library is the CUDA build; without it nothing runs
        return {"cuda_compiled": False, "available": False, "devices": [], "reason": str(e)}
    try:
        n = device_count()
        devices = [device_info(i) for i in range(n)]
        reason = None if n else "the CUDA driver reports no device"
    except Exception as e:
        devices, reason = [], str(e)
    return {"cuda_compiled": True, "available": bool(devices), "devices": devices, "reason": reason}


# ----------------------------------------------------------------------------------------------
# The session
# ----------------------------------------------------------------------------------------------

def _mean_edge_length(p, f) -> float:
    e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
    e = np.unique(np.sort(e, axis=1), axis=0)
    return float(np.linalg.norm(p[e[:, 0]] - p[e[:, 1]], axis=1).mean()) if len(e) else 0.0


class RepulsiveSurfaceSession:
    """The repulsive-surface flow of a triangle mesh, one step at a time
    (RepulsiveSurfaceSession, crates/ddg-py/src/python/repulsive_surfaces.rs:404-604; the engine
    crates/ddg-py/src/repulsive_surfaces.rs:1633-1810).

    Each step is ``rs_flow_step`` on the GPU: Barnes-Hut energy and differential, the
    hierarchical Hs solve, the Armijo line search on frozen lists and the projection. The
    session adds the reference's outer loop: stop rules, ``stuck_limit``, ``max_iterations``,
    ``time_limit``, ``cancel`` and ``reset``. With ``ccd`` (the default) the first trial of the
    line search is capped at two thirds of the first contact time of the motion
    (RS/src/ccd.rs:762-884, on the GPU). ``step`` and ``run`` release the GIL inside the
    library; ``snapshot`` and the getters never wait for a running step; ``cancel`` is safe from
    any thread and stops a running step between line-search trials (the mesh stays that of the
    last completed step). There is
    no remeshing: the faces, ``face_origin`` (the identity) and ``pinned`` (empty) never change.
    """

    def __init__(self, positions, faces, **options):
        p, f = _mesh(positions, faces)
        self._opts = _Options(options)
        self._start = (p, f)
        self._ctx = _context(self._opts.o)
        try:
            name = self._ctx.info()["name"]
        except RsError:
            name = None
        self._device = name
        self._lock = threading.Lock()      # held while a step runs
        self._snap_lock = threading.Lock()  # guards the snapshot
        self._cancel = False
        self._begin()

    def _begin(self):
        p, f = self._start
        try:
            self._flow = Flow(f, p, self._opts.flow_options(), self._ctx)
            tree = BhTree.build(f, p, self._opts.bh(), self._ctx)
            e0 = tree.try_energy(Exponents(self._opts.o["alpha"], self._opts.o["beta"]))
        except RsError as e:
            raise _lib_err(e) from None
        self._iteration = 0
        self._stuck = 0
        self._accepted = deque()
        self._first_sobolev = None
        self._snap = {"positions": p.copy(), "iteration": 0, "energy": e0, "status": "running",
                      "error": None, "mean_edge_length0": _mean_edge_length(p, f), "report": None}

    # ---- state -------------------------------------------------------------------------------
    def snapshot(self) -> dict:
        """The last completed state: positions, faces, pinned, face_origin, iteration, energy,
        status, error, mean_edge_length0, report. Does not wait for a running step."""
        with self._snap_lock:
            s = dict(self._snap)
        f = self._start[1]
        return {"positions": _flat_points(s["positions"]), "faces": _flat_faces(f),
                "pinned": array.array("i"), "face_origin": array.array("i", range(len(f))),
                "iteration": s["iteration"], "energy": s["energy"], "status": s["status"],
                "error": s["error"], "mean_edge_length0": s["mean_edge_length0"], "report": s["report"]}

    def _get(self, key):
        with self._snap_lock:
            return self._snap[key]

    positions = property(lambda self: _flat_points(self._get("positions")),
                         doc="array('d'), 3 per vertex: the positions of the last completed step.")
    faces = property(lambda self: _flat_faces(self._start[1]), doc="array('i'), 3 per face.")
    energy = property(lambda self: self._get("energy"), doc="The energy of the last completed step.")
    iteration = property(lambda self: self._get("iteration"), doc="Steps taken.")
    status = property(lambda self: self._get("status"),
                      doc='"running", "converged", "max_iterations", "time_limit", "stuck", "cancelled" or "error".')
    error = property(lambda self: self._get("error"), doc="The message of the error when status is \"error\".")
    n_vertices = property(lambda self: len(self._start[0]), doc="Number of vertices.")
    n_faces = property(lambda self: len(self._start[1]), doc="Number of faces.")
    report = property(lambda self: self._get("report"), doc="The dict of the last step, or None.")

    def __repr__(self):
        s = self.snapshot()
        return (f"RepulsiveSurfaceSession(vertices={self.n_vertices}, faces={self.n_faces}, "
                f"iteration={s['iteration']}, energy={s['energy']:.6e}, status={s['status']!r})")

    # ---- control -----------------------------------------------------------------------------
    def cancel(self) -> None:
        """Stops a running step between line-search trials, and every later step; the snapshot
        reads "cancelled" at once (Engine::cancel, crates/ddg-py/src/repulsive_surfaces.rs:1688-1695)."""
        self._cancel = True
        try:
            self._flow.cancel(True)
        except RsError:
            pass
        with self._snap_lock:
            self._snap["status"] = "cancelled"

    def reset(self) -> None:
        """Back to the initial mesh with the same options (clears cancel). Waits for a running step."""
        with self._lock:
            self._cancel = False
            self._begin()

    def _cancelled_report(self) -> dict:
        s = self._snap
        return {"iteration": s["iteration"], "status": "cancelled", "session_status": "cancelled",
                "n_vertices": self.n_vertices, "n_faces": self.n_faces,
                "energy_before": s["energy"], "energy_after": s["energy"]}

    def step(self) -> dict:
        """One step; returns its report dict (step_val, crates/ddg-py/src/repulsive_surfaces.rs:1433-1516).
        A cancelled session does not step and reports status "cancelled"."""
        with self._lock:
            if self._cancel:
                with self._snap_lock:
                    self._snap["status"] = "cancelled"
                    return self._cancelled_report()
            try:
                r = self._flow.step()
            except RsError as e:
                if e.kind == "Cancelled":  # the step stopped between trials: nothing moved
                    with self._snap_lock:
                        self._snap["status"] = "cancelled"
                        return self._cancelled_report()
                with self._snap_lock:
                    self._snap["status"], self._snap["error"] = "error", str(e)
                raise _lib_err(e) from None
            positions = self._flow.positions()
            return self._finish(r, positions)

    def _finish(self, r: dict, positions) -> dict:
        o = self._opts.o
        self._iteration += 1
        accepted = r["accepted"] > 0
        self._stuck = 0 if accepted else self._stuck + 1
        slope = r["slope"]
        if self._first_sobolev is None:
            self._first_sobolev = slope
        converged = False
        if o["stop"] == "energy_stall":
            if accepted:
                self._accepted.append(r["energy_after"])
                while len(self._accepted) > o["stop_window"] + 1:
                    self._accepted.popleft()
            w = o["stop_window"]
            converged = (len(self._accepted) == w + 1 and
                         self._accepted[0] - self._accepted[w] <= o["stop_relative"] * abs(self._accepted[w]))
        elif o["stop"] == "sobolev":
            s0 = self._first_sobolev
            converged = s0 > 0.0 and math.sqrt(max(slope / s0, 0.0)) < o["stop_eps"]
        if self._stuck >= o["stuck_limit"]:
            status = "stuck"
        elif converged:
            status = "converged"
        elif self._iteration >= o["max_iterations"]:
            status = "max_iterations"
        else:
            status = "running"
        holds = int(self._opts.hold_area) + int(self._opts.hold_volume)
        iters = int(r["gmres_direction"] + (r["gmres_area"] if self._opts.hold_area else 0)
                    + (r["gmres_volume"] if self._opts.hold_volume else 0))
        rep = {
            "iteration": self._iteration,
            "status": "accepted" if accepted else "stuck",
            "session_status": status,
            "device": "cuda", "device_name": self._device, "metric_device": "cuda",
            "n_vertices": self.n_vertices, "n_faces": self.n_faces,
            "energy_before": r["energy_before"], "energy_after": r["energy_after"],
            "tangent_point_after": r["energy_after"], "penalties_after": [],
            "gradient_norm": r["gradient_norm"], "sobolev_norm_sq": slope,
            "tau": r["tau"], "tau0": r["tau0"], "tau_ccd": None if math.isnan(r["tau_ccd"]) else r["tau_ccd"],
            "halvings": int(r["halvings"]), "newton_steps": int(r["newton_steps"]),
            "projection": PROJECTION_STATUS[int(r["projection_status"])],
            "max_violation": r["constraint_residual"], "dropped_rows": [],
            "linear": {"solver": "gmres", "dimension": 3 * self.n_vertices + 3, "solves": holds + 1,
                       "iterations": iters, "relative_residual": r["relative_residual"]},
            "remesh": None,
            "seconds": {"bvh": r["seconds_tree"], "energy": r["seconds_energy"],
                        "factor": r["seconds_solver_build"], "solve": r["seconds_solve"],
                        "line_search": r["seconds_line_search"], "ccd": r["seconds_ccd"],
                        "projection": r["seconds_projection"], "remesh": 0.0, "total": r["seconds"]},
        }
        with self._snap_lock:
            self._snap.update(positions=positions, iteration=self._iteration, energy=r["energy_after"],
                              status="cancelled" if self._cancel else status, report=rep)
        return rep

    def run(self, max_steps=None, progress=None, time_limit=None) -> dict:
        """Steps until the session is final, ``max_steps`` steps of this call were taken,
        ``cancel()`` was called, ``time_limit`` seconds passed (default: the option), or
        ``progress(report)`` returned False (Engine::run, crates/ddg-py/src/repulsive_surfaces.rs:1762-1806).
        Returns end, status, steps_taken, iteration, energy_before, energy_after, seconds, steps."""
        if max_steps is not None:
            max_steps = _count("max_steps", max_steps)
        if time_limit is None:
            time_limit = self._opts.o["time_limit"]
        t0 = time.perf_counter()
        energy_before = self.energy
        steps = []
        while True:
            if max_steps is not None and len(steps) >= max_steps:
                end = "max_steps"
                break
            if time_limit is not None and time.perf_counter() - t0 >= time_limit:
                end = "time_limit"
                break
            if self._cancel:
                end = "cancelled"
                break
            with self._snap_lock:
                if self._snap["status"] != "running":
                    end = "final"
                    break
                if self._snap["iteration"] >= self._opts.o["max_iterations"]:
                    self._snap["status"] = "max_iterations"
                    end = "final"
                    break
            rep = self.step()
            if rep["status"] == "cancelled":
                end = "cancelled"
                break
            go = True if progress is None else progress(rep)
            steps.append(rep)
            if go is False:
                end = "callback"
                break
        s = self.snapshot()
        return {"end": end, "status": s["status"], "steps_taken": len(steps), "iteration": s["iteration"],
                "energy_before": energy_before, "energy_after": s["energy"],
                "seconds": time.perf_counter() - t0, "steps": steps}


def repulsive_surface_flow(positions, faces, steps=None, progress=None, **options):
    """The flow in one call: ``(positions, faces, report)`` (repulsive_surface_flow,
    crates/ddg-py/src/python/repulsive_surfaces.rs:596-652). ``report`` has status, iterations,
    energy_initial, energy_final, seconds, pinned, face_origin and steps; ``progress`` returning
    False stops the flow with status "cancelled". A session stepped the same number of times
    gives bitwise the same mesh."""
    if steps is not None:
        options = dict(options, max_iterations=_count("steps", steps))
    s = RepulsiveSurfaceSession(positions, faces, **options)
    t0 = time.perf_counter()
    out = []
    status = s.status
    while True:
        if s.iteration >= s._opts.o["max_iterations"]:
            status = "max_iterations"
            break
        tl = s._opts.o["time_limit"]
        if tl is not None and time.perf_counter() - t0 >= tl:
            status = "time_limit"
            break
        rep = s.step()
        out.append(rep)
        status = rep["session_status"]
        if progress is not None and progress(rep) is False:
            status = "cancelled"
            break
        if status != "running":
            break
    snap = s.snapshot()
    report = {"status": status, "iterations": snap["iteration"],
              "energy_initial": out[0]["energy_before"] if out else None,
              "energy_final": snap["energy"], "seconds": time.perf_counter() - t0,
              "steps": [dict(r, session_status=status) for r in out],
              "pinned": snap["pinned"], "face_origin": snap["face_origin"]}
    return snap["positions"], snap["faces"], report


# ----------------------------------------------------------------------------------------------
# Scene files
# ----------------------------------------------------------------------------------------------

_SCENE_OFF_PATH = {"minimize", "obstacle", "point_cloud_obstacle", "implicit", "allow_barycenter_shift",
                   "autotarget_volume"}
_SCENE_METHODS = {"hs", "aqp", "bqn", "h1", "h1-lbfgs", "h2", "willmore", "l2"}


def repulsive_surface_scene(path):
    """A scene file of the reference program as ``(positions, faces, options)``
    (repulsive_surface_scene, crates/ddg-py/src/python/repulsive_surfaces.rs:693-710; the format
    of RS/src/scene.rs:466-700 and its options, RS/src/step/scene_run.rs:34-104).

    The statements on this library's path are read: ``repel_mesh <obj> <alpha> <beta>`` (the
    OBJ path relative to the scene's directory), ``constrain barycenter|area|volume`` without a
    growth schedule, ``iteration_limit``, ``time_limit`` (milliseconds), ``method hs``,
    ``disable_near_field`` and ``log`` (ignored). The options are this library's defaults with
    the scene's exponents, constraints and limits (no remeshing, as everywhere here). Any other
    statement or value, such as a potential, an obstacle, an implicit surface, a growth
    schedule, vertex pins or another method, raises ``RepulsiveSurfaceInputError`` naming it
    and its line."""
    from pathlib import Path

    from . import obj

    path = Path(path)
    try:
        text = path.read_text()
    except OSError as e:
        raise _bad("path", f"{path}: {e}") from None
    mesh, alpha, beta, constraints, seen = None, None, None, [], {}
    limits, low_order = {}, True

    def err(line, msg):
        return RepulsiveSurfaceInputError(f"{path}:{line}: {msg}")

    for i, raw in enumerate(text.splitlines(), 1):
        t = raw.strip()
        if not t or t.startswith("#"):
            continue
        words = t.split()
        kw, rest = words[0], words[1:]
        if kw in ("repel_mesh", "iteration_limit", "time_limit", "method", "log"):
            if kw in seen:
                raise err(i, f"`{kw}` is given twice (first on line {seen[kw]})")
            seen[kw] = i
        if kw == "repel_mesh":
            if len(rest) != 3:
                raise err(i, "`repel_mesh` needs an OBJ path and the exponents `alpha beta`")
            mesh = rest[0]
            try:
                alpha, beta = float(rest[1]), float(rest[2])
            except ValueError:
                raise err(i, "the exponents must be numbers") from None
        elif kw == "constrain":
            if not rest:
                raise err(i, "`constrain` needs a constraint type")
            kind = rest[0]
            if kind not in ("barycenter", "area", "volume"):
                raise err(i, f"`constrain {kind}` {_OFF_PATH}")
            if len(rest) > 1:
                raise err(i, f"a growth schedule (`constrain {kind} {' '.join(rest[1:])}`) {_OFF_PATH}")
            constraints.append({"type": kind})
        elif kw in ("iteration_limit", "time_limit"):
            if len(rest) != 1 or not rest[0].isdigit():
                raise err(i, f"`{kw}` needs one non-negative integer")
            n = int(rest[0])
            if n > 0:
                limits[kw] = n
        elif kw == "method":
            if len(rest) != 1 or rest[0] not in _SCENE_METHODS:
                raise err(i, f"unknown method `{' '.join(rest)}`")
            if rest[0] != "hs":
                raise err(i, f"method `{rest[0]}` {_OFF_PATH}")
        elif kw == "disable_near_field":
            low_order = False
        elif kw == "log":
            pass
        elif kw in _SCENE_OFF_PATH:
            raise err(i, f"`{kw}` {_OFF_PATH}")
        else:
            raise err(i, f"unknown keyword `{kw}`")
    if mesh is None:
        raise err(0, "the scene has no `repel_mesh` statement")
    try:
        P, F = obj.read_obj(path.parent / mesh)
    except RsError as e:
        raise _lib_err(e) from None
    options = repulsive_surface_defaults()
    options.update(alpha=alpha, beta=beta, constraints=constraints, low_order=low_order)
    if not low_order:
        options["barycenter_mode"] = "global"
    if "iteration_limit" in limits:
        options["max_iterations"] = limits["iteration_limit"]
    if "time_limit" in limits:
        options["time_limit"] = limits["time_limit"] / 1000.0
    _Options(options)  # the same checks as a session (exponents, constraints)
    return _flat_points(P), _flat_faces(F), options
