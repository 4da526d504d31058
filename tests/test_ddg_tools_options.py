"""The ddg_tools-compatible options and mesh decoding on the CPU: every option name of the
reference is known, bad values and values off the GPU path are errors naming the option, and
the accepted values map onto rs_flow_options (crates/ddg-py/src/repulsive_surfaces.rs:684-1161;
the reference's tests crates/ddg-py/python-tests/test_repulsive_surfaces.py:359-420, 602-730)."""
import array
import math

import numpy as np
import pytest

from rs_gb300 import ddg_tools as D

# the option names of the reference's glue, in its order (OPTION_NAMES)
REFERENCE_OPTIONS = (
    "alpha beta energy coulomb_alpha tp_weight metric low_order l2_kind backend dense_max_faces "
    "energy_eval theta leaf_size chi cluster_leaf_size gmres_restart gmres_tolerance "
    "gmres_max_iterations gmres_side device cuda_ordinal gpu_determinism method aqp_kappa "
    "lbfgs_memory lbfgs_variant constraints barycenter barycenter_mode barycenter_shift pins "
    "pin_targets pin_move pin_move_steps schedule_timing penalties ccd_obstacles armijo armijo_c "
    "start start_lengths start_factor start_tau tau_min_rel max_halvings ccd ccd_gap "
    "ccd_max_iterations ccd_close_factor newton_steps newton_max remesh remesh_split "
    "remesh_collapse remesh_rounds remesh_rho remesh_flip_cap remesh_order remesh_ops stop "
    "stop_relative stop_window stop_eps max_iterations time_limit stuck_limit threads "
    "reference_compat").split()


def test_every_reference_option_is_known():
    d = D.repulsive_surface_defaults()
    assert list(d) == REFERENCE_OPTIONS
    assert D.OPTION_NAMES == tuple(REFERENCE_OPTIONS)


def test_defaults_are_the_references_on_the_path():
    d = D.repulsive_surface_defaults()
    # the paper's exponents and the library's numerical defaults
    assert (d["alpha"], d["beta"], d["theta"], d["leaf_size"], d["chi"], d["cluster_leaf_size"]) == (
        6.0, 12.0, 0.5, 8, 0.5, 8)
    assert (d["gmres_restart"], d["gmres_tolerance"], d["gmres_max_iterations"]) == (60, 1e-3, 200)
    assert (d["armijo_c"], d["newton_max"], d["stop_relative"], d["stop_window"]) == (1e-2, 5, 1e-7, 10)
    assert (d["max_iterations"], d["stuck_limit"], d["tau_min_rel"]) == (1000, 5, 1e-12)
    # the defaults that differ: the GPU path has no CPU device and no remeshing
    assert (d["device"], d["backend"], d["remesh"]) == ("cuda", "hierarchical", False)
    assert (d["ccd"], d["ccd_gap"], d["ccd_max_iterations"], d["ccd_close_factor"]) == (True, 0.05, 100, 0.5)


def _fields(st):
    """A ctypes structure as nested tuples of its fields (its padding bytes are unset); NaN
    fields (unset targets) as a string so that equal structures compare equal."""
    return tuple(_fields(v) if hasattr(v, "_fields_") else ("nan" if v != v else v)
                 for v in (getattr(st, n) for n, _ in st._fields_))


def test_passing_the_defaults_back_changes_nothing():
    a = D._Options(D.repulsive_surface_defaults()).flow_options()
    b = D._Options({}).flow_options()
    assert _fields(a) == _fields(b)


def test_options_map_onto_the_flow():
    o = D._Options(dict(alpha=4.0, beta=9.0, theta=0.3, leaf_size=6, chi=0.25, cluster_leaf_size=12,
                        gmres_restart=30, gmres_tolerance=1e-6, gmres_max_iterations=77, tp_weight=2.0,
                        low_order=False, barycenter_mode="global", armijo_c=0.1, max_halvings=9, newton_max=3,
                        constraints=[{"type": "barycenter"}, {"type": "area"}, {"type": "volume"}]))
    f = o.flow_options()
    assert (f.alpha, f.beta, f.theta, f.leaf_size) == (4.0, 9.0, 0.3, 6)
    assert (f.hold_area, f.hold_volume, f.armijo_c, f.max_halvings, f.newton_max) == (1, 1, 0.1, 9, 3)
    s = f.solver
    assert (s.chi, s.leaf_size, s.restart, s.tolerance, s.max_iterations) == (0.25, 12, 30, 1e-6, 77)
    assert (s.tp_weight, s.low_order) == (2.0, 0)
    assert (f.ccd, f.ccd_gap, f.ccd_max_iterations, f.ccd_close_factor) == (1, 0.05, 100, 0.5)
    f = D._Options(dict(low_order=False, barycenter_mode="global")).flow_options()
    assert f.solver.low_order == 0
    f = D._Options(dict(ccd=False)).flow_options()
    assert f.ccd == 0
    f = D._Options(dict(ccd_gap=0.1, ccd_max_iterations=7, ccd_close_factor=0.25)).flow_options()
    assert (f.ccd_gap, f.ccd_max_iterations, f.ccd_close_factor) == (0.1, 7, 0.25)
    # exact evaluation is Barnes-Hut with theta 0 (no node is admissible)
    assert D._Options({"energy_eval": "exact", "theta": 0.7}).flow_options().theta == 0.0
    # no halving cap by default: the search stops at tau_min
    assert D._Options({}).flow_options().max_halvings >= 1000


@pytest.mark.parametrize("kw, name", [
    ({"alhpa": 6.0}, "alhpa"),
    ({"alpha": 1.0}, "alpha"),
    ({"beta": 30.0}, "alpha, beta"),
    ({"theta": "big"}, "theta"),
    ({"theta": math.inf}, "theta"),
    ({"leaf_size": -1}, "leaf_size"),
    ({"leaf_size": 2.5}, "leaf_size"),
    ({"low_order": 1}, "low_order"),
    ({"device": "gpu"}, "device"),
    ({"stop": "sobolev"}, "stop_eps"),
    ({"remesh_ops": ["split", "twist"]}, "remesh_ops"),
    ({"time_limit": -1.0}, "time_limit"),
    ({"tp_weight": 0.0}, "tp_weight"),
    ({"ccd_gap": 0.0}, "ccd_gap"),
    ({"ccd_max_iterations": 0}, "ccd_max_iterations"),
    ({"ccd_close_factor": 1.0}, "ccd_close_factor"),
    ({"theta": None}, "theta"),
])
def test_bad_values_are_named(kw, name):
    with pytest.raises(D.RepulsiveSurfaceInputError) as e:
        D._Options(kw)
    assert name in str(e.value)
    assert isinstance(e.value, ValueError) and isinstance(e.value, D.InputError)


@pytest.mark.parametrize("kw, name", [
    ({"remesh": True}, "remesh"),
    ({"device": "cpu"}, "device"),
    ({"backend": "dense"}, "backend"),
    ({"method": "aqp"}, "method"),
    ({"metric": "h1"}, "metric"),
    ({"energy": "willmore"}, "energy"),
    ({"gmres_side": "left"}, "gmres_side"),
    ({"armijo": "reference"}, "armijo"),
    ({"pins": [0, 1]}, "pins"),
    ({"penalties": [{"type": "area"}]}, "penalties"),
    ({"barycenter": False}, "barycenter"),
    ({"barycenter_mode": "per_component"}, "barycenter_mode"),
    ({"gpu_determinism": "match_cpu"}, "gpu_determinism"),
    ({"low_order": False}, "barycenter_mode"),
    ({"constraints": [{"type": "volume"}]}, "constraints"),
    ({"constraints": [{"type": "barycenter"}, {"type": "area", "target": 3.0}]}, "constraints[1].target"),
    ({"constraints": [{"type": "barycenter"}, {"type": "volume", "factor": 1.1, "steps": 3}]},
     "constraints[1].factor"),
    ({"constraints": [{"type": "barycenter"}, {"type": "pins", "vertices": [0]}]}, "constraints[1]"),
    ({"constraints": [{"type": "barycenter", "colour": 1}]}, "constraints[0]"),
    ({"constraints": {"type": "barycenter"}}, "constraints"),
])
def test_values_off_the_gpu_path_are_named(kw, name):
    with pytest.raises(D.RepulsiveSurfaceInputError) as e:
        D._Options(kw)
    assert str(e.value).startswith(name)


def test_energy_options_ignore_the_flow_settings():
    # surface_energy reads the exponents, the evaluation and the penalties only
    o = D._Options({"remesh": True, "ccd": True, "device": "cpu", "method": "bcqn"}, flow=False)
    assert o.bh().theta == 0.5
    with pytest.raises(D.RepulsiveSurfaceInputError, match="^penalties"):
        D._Options({"penalties": [{"type": "area"}]}, flow=False)


def test_mesh_inputs():
    p = [[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]]
    for pos in (p, np.array(p), array.array("d", np.ravel(p)), np.ravel(p).tolist()):
        for fac in ([[0, 1, 2]], [0, 1, 2], array.array("i", [0, 1, 2]), np.array([[0, 1, 2]], np.int64)):
            P, F = D._mesh(pos, fac)
            assert P.shape == (3, 3) and P.dtype == np.float64
            assert F.shape == (1, 3) and F.dtype == np.uint32
    with pytest.raises(D.RepulsiveSurfaceInputError, match="^positions"):
        D._mesh([0.0, 1.0], [0, 1, 2])
    with pytest.raises(D.RepulsiveSurfaceInputError, match="^positions: entry 4"):
        D._mesh([0, 0, 0, 1, math.nan, 0, 0, 1, 0], [0, 1, 2])
    with pytest.raises(D.RepulsiveSurfaceInputError, match="^faces"):
        D._mesh(p, [0, 1])
    with pytest.raises(D.RepulsiveSurfaceInputError, match="^faces: entry 1 = -1"):
        D._mesh(p, [0, -1, 2])
    with pytest.raises(D.RepulsiveSurfaceInputError, match="^faces"):
        D._mesh(p, [0.0, 1.5, 2.0])


def test_error_kinds_map_as_the_reference():
    from rs_gb300 import RsError
    assert isinstance(D._lib_err(RsError(5, "NonFiniteEnergy", "flow", "x")), D.SolveError)
    assert isinstance(D._lib_err(RsError(3, "SolverDiverged", "solve", "x")), D.SolveError)
    assert isinstance(D._lib_err(RsError(2, "DegenerateFace", "surface", "x")), D.RepulsiveSurfaceInputError)


def _scene(tmp_path, body):
    from rs_gb300 import generators as gen
    from rs_gb300 import obj

    P, F = gen.icosphere(1)
    obj.write_obj(tmp_path / "s.obj", P, F)
    (tmp_path / "a.scene").write_text(body)
    return tmp_path / "a.scene", P, F


def test_scene_files_on_the_path(tmp_path):
    path, P, F = _scene(tmp_path, "# a scene\nrepel_mesh s.obj 6 12\nconstrain barycenter\n"
                                  "constrain volume\niteration_limit 50\ntime_limit 2500\nmethod hs\nlog out.csv\n")
    p, f, o = D.repulsive_surface_scene(path)
    assert np.frombuffer(p, np.float64).tobytes() == np.ascontiguousarray(P, np.float64).tobytes()
    assert np.frombuffer(f, np.int32).tolist() == np.asarray(F).ravel().tolist()
    assert o["constraints"] == [{"type": "barycenter"}, {"type": "volume"}]
    assert (o["alpha"], o["beta"], o["max_iterations"], o["time_limit"]) == (6.0, 12.0, 50, 2.5)
    D._Options(o)


@pytest.mark.parametrize("body, what", [
    ("repel_mesh s.obj 6 12\nminimize area 1\n", "minimize"),
    ("repel_mesh s.obj 6 12\nobstacle o.obj 1\n", "obstacle"),
    ("repel_mesh s.obj 6 12\nconstrain area 2 100\n", "growth"),
    ("repel_mesh s.obj 6 12\nconstrain vertices 1 2\n", "constrain vertices"),
    ("repel_mesh s.obj 6 12\nmethod aqp\n", "aqp"),
    ("repel_mesh s.obj 6 12\nbogus\n", "unknown keyword"),
    ("constrain barycenter\n", "repel_mesh"),
    ("repel_mesh s.obj 6 12\nrepel_mesh s.obj 6 12\n", "twice"),
    ("repel_mesh s.obj 1 3\nconstrain barycenter\n", "alpha"),
    ("repel_mesh s.obj 6 12\nconstrain volume\n", "constraints"),
])
def test_scene_statements_off_the_path_are_named(tmp_path, body, what):
    path, _, _ = _scene(tmp_path, body)
    with pytest.raises(D.RepulsiveSurfaceInputError) as e:
        D.repulsive_surface_scene(path)
    assert what in str(e.value)
