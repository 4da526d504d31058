"""The ddg_tools-compatible functions on the GPU, tested the way the reference tests its Python
module (crates/ddg-py/python-tests/test_repulsive_surfaces.py:113-130, 225-357, 547-615):
surface_energy equals the library's energy bitwise, a session stepped N times equals the
one-call flow bitwise, run/cancel/reset follow the reference's outer loop, and the held volume
and barycenter stay put."""
import array
import threading
import time

import numpy as np
import pytest

import rs_gb300 as R
from rs_gb300 import ddg_tools as D
from rs_gb300 import generators as gen

pytestmark = pytest.mark.gpu


def _torus(nu=24, nv=12, seed=11):
    return gen.noisy_torus(nu, nv, 1.0, 0.35, 0.002, seed)


def _volume(P, F):
    p0, p1, p2 = P[F[:, 0]], P[F[:, 1]], P[F[:, 2]]
    return np.sum(np.einsum("ij,ij->i", p0, np.cross(p1, p2))) / 6.0


def _barycenter(P, F):
    p0, p1, p2 = P[F[:, 0]], P[F[:, 1]], P[F[:, 2]]
    a = 0.5 * np.linalg.norm(np.cross(p1 - p0, p2 - p0), axis=1)
    return (a[:, None] * (p0 + p1 + p2) / 3.0).sum(0) / a.sum()


def test_gpu_info():
    g = D.gpu_info()
    assert g["cuda_compiled"] and g["available"] and g["reason"] is None
    d = g["devices"][0]
    assert d["ordinal"] == 0 and d["memory_bytes"] > 0 and d["name"]
    assert d["compute_capability"].count(".") == 1


def test_surface_energy_is_the_librarys():
    P, F = _torus()
    E, dE, rep = D.surface_energy(P, F, theta=0.25)
    tree = R.BhTree.build(F, P, R.BhOptions(theta=0.25))
    E2, dE2 = tree.energy_and_differential(R.Exponents())
    assert E == E2 and rep["energy"] == E and rep["total"] == E
    assert isinstance(dE, array.array) and dE.typecode == "d"
    assert np.frombuffer(dE, np.float64).tobytes() == dE2.ravel().tobytes()
    assert set(rep) == {"energy", "total", "penalties", "subcritical", "pairs_exact", "nodes_lumped", "seconds"}
    assert rep["penalties"] == [] and rep["nodes_lumped"] > 0
    # exact evaluation: every ordered pair (theta 0 admits no node)
    Ex, _, rx = D.surface_energy(P, F, energy_eval="exact")
    assert rx["nodes_lumped"] == 0 and rx["pairs_exact"] == len(F) * (len(F) - 1)
    assert abs(Ex - E) <= 2e-2 * abs(Ex)
    # the flow's options are accepted and ignored, as the reference does
    E3, _, _ = D.surface_energy(P, F, theta=0.25, remesh=True, ccd=True, method="bcqn")
    assert E3 == E


def test_session_state_report_and_getters():
    P, F = _torus()
    s = D.RepulsiveSurfaceSession(P, F)
    assert (s.iteration, s.status, s.report, s.error) == (0, "running", None, None)
    assert s.n_vertices == len(P) and s.n_faces == len(F)
    r = s.step()
    for key in ("iteration", "status", "session_status", "n_vertices", "n_faces", "energy_before",
                "energy_after", "penalties_after", "gradient_norm", "tau", "halvings", "max_violation",
                "linear", "remesh", "seconds", "device", "device_name", "metric_device", "sobolev_norm_sq",
                "tau0", "newton_steps", "projection", "dropped_rows", "tangent_point_after"):
        assert key in r
    assert (r["iteration"], r["status"], r["device"], r["metric_device"]) == (1, "accepted", "cuda", "cuda")
    assert r["energy_after"] < r["energy_before"]
    assert r["gradient_norm"] > 0 and r["sobolev_norm_sq"] > 0 and r["tau0"] >= r["tau"] > 0
    assert r["linear"]["solver"] == "gmres" and r["linear"]["relative_residual"] <= 1.5e-3
    assert s.iteration == 1 and s.energy == r["energy_after"] and s.report["iteration"] == 1
    assert "RepulsiveSurfaceSession(" in repr(s)
    snap = s.snapshot()
    assert set(snap) == {"positions", "faces", "pinned", "face_origin", "iteration", "energy", "status",
                         "error", "mean_edge_length0", "report"}
    assert snap["positions"].typecode == "d" and snap["faces"].typecode == "i"
    assert len(snap["face_origin"]) == len(F) and len(snap["pinned"]) == 0
    assert np.frombuffer(snap["faces"], np.int32).tolist() == F.ravel().tolist()
    # energy_after is F at the new positions (on the step's lists): a fresh tree agrees closely
    Q = np.frombuffer(snap["positions"], np.float64).reshape(-1, 3)
    E1, _, _ = D.surface_energy(Q, F)
    assert abs(E1 - r["energy_after"]) <= 1e-2 * E1


def test_stepping_equals_the_one_call_flow_bitwise():
    P, F = _torus()
    for options in ({}, {"constraints": [{"type": "barycenter"}, {"type": "volume"}]}):
        q, g, report = D.repulsive_surface_flow(P, F, steps=3, **options)
        s = D.RepulsiveSurfaceSession(P, F, max_iterations=3, **options)
        for _ in range(3):
            s.step()
        assert s.positions.tobytes() == q.tobytes()
        assert s.faces.tobytes() == g.tobytes()
        assert report["iterations"] == 3 and len(report["steps"]) == 3 and report["status"] == "max_iterations"
        s2 = D.RepulsiveSurfaceSession(P, F, max_iterations=3, **options)
        end = s2.run()
        assert end["steps_taken"] == 3 and end["end"] == "final" and end["status"] == "max_iterations"
        assert s2.positions.tobytes() == q.tobytes()


def test_flow_keeps_volume_and_barycenter():
    P, F = _torus()
    e0, _, _ = D.surface_energy(P, F)
    v0, b0 = _volume(P, F), _barycenter(P, F)
    q, g, report = D.repulsive_surface_flow(P, F, steps=6, constraints=[{"type": "barycenter"}, {"type": "volume"}])
    Q = np.frombuffer(q, np.float64).reshape(-1, 3)
    e1, _, _ = D.surface_energy(Q, F)
    assert e1 < e0
    assert abs(report["energy_initial"] - e0) <= 1e-12 * e0
    assert abs(_volume(Q, F) - v0) <= 1e-6 * abs(v0)
    assert np.abs(_barycenter(Q, F) - b0).max() <= 1e-9
    for st in report["steps"]:
        assert st["energy_after"] <= st["energy_before"] * (1 + 1e-9)


def test_run_with_progress_and_limits():
    P, F = _torus()
    s = D.RepulsiveSurfaceSession(P, F)
    seen = []
    end = s.run(max_steps=5, progress=lambda r: seen.append(r["iteration"]) or len(seen) < 3)
    assert end["end"] == "callback" and seen == [1, 2, 3]
    end = s.run(max_steps=2)
    assert (end["end"], end["steps_taken"], len(end["steps"])) == ("max_steps", 2, 2)
    assert s.iteration == 5
    s2 = D.RepulsiveSurfaceSession(P, F, max_iterations=2)
    end = s2.run()
    assert (end["end"], end["status"], end["steps_taken"]) == ("final", "max_iterations", 2)
    assert s2.run()["steps_taken"] == 0
    with pytest.raises(KeyError):  # an exception in progress() propagates
        D.repulsive_surface_flow(P, F, steps=3, progress=lambda r: {}["boom"])
    _, _, rep = D.repulsive_surface_flow(P, F, steps=3, progress=lambda r: False)
    assert rep["status"] == "cancelled" and rep["iterations"] == 1


def test_cancel_and_reset():
    P, F = _torus()
    s = D.RepulsiveSurfaceSession(P, F)
    s.step()
    s.cancel()
    assert s.status == "cancelled"
    r = s.step()
    assert r["status"] == "cancelled" and s.iteration == 1
    assert s.run()["end"] == "cancelled"
    s.reset()
    assert (s.iteration, s.status) == (0, "running")
    assert s.positions.tobytes() == np.ascontiguousarray(P, np.float64).tobytes()
    s.step()
    assert s.iteration == 1


def test_cancel_from_another_thread_while_running():
    P, F = _torus(48, 24)
    s = D.RepulsiveSurfaceSession(P, F, max_iterations=100000)
    result = {}
    worker = threading.Thread(target=lambda: result.update(s.run()))
    worker.start()
    deadline = time.time() + 120
    ticks = 0
    while s.iteration < 2 and time.time() < deadline:
        ticks += 1  # the library releases the GIL: this thread polls while a step runs
        snap = s.snapshot()
        assert len(snap["faces"]) // 3 == len(snap["face_origin"])
        time.sleep(0.01)
    assert s.iteration >= 2 and ticks > 0
    s.cancel()
    assert s.status == "cancelled"
    worker.join(60)
    assert not worker.is_alive()
    assert result["end"] == "cancelled"


def test_stop_rules():
    P, F = _torus()
    # the Sobolev rule with a ratio above 1 stops after the first step
    s = D.RepulsiveSurfaceSession(P, F, stop="sobolev", stop_eps=2.0)
    assert s.step()["session_status"] == "converged"
    assert s.run()["end"] == "final"
    # the energy-stall rule with a huge tolerance stops once the window is full
    s = D.RepulsiveSurfaceSession(P, F, stop_window=2, stop_relative=1e9)
    statuses = [s.step()["session_status"] for _ in range(3)]
    assert statuses == ["running", "running", "converged"]


def test_bad_inputs_and_device_errors():
    P, F = _torus()
    with pytest.raises(D.RepulsiveSurfaceInputError, match="^cuda_ordinal"):
        D.RepulsiveSurfaceSession(P, F, cuda_ordinal=64)
    bad = np.array(F, copy=True)
    bad[0, 0] = len(P) + 5
    with pytest.raises(D.RepulsiveSurfaceInputError):
        D.RepulsiveSurfaceSession(P, bad)
    with pytest.raises(D.RepulsiveSurfaceInputError):
        D.surface_energy(P, bad)


def test_collision_cap_in_the_flow():
    """With ccd the first trial is min(tau0, 2/3 tau_max) when the motion meets a contact before
    tau0, and unchanged otherwise (session.rs:927-955)."""
    P, F = _torus()
    a = D.RepulsiveSurfaceSession(P, F, ccd=False).step()
    assert a["tau_ccd"] is None and a["seconds"]["ccd"] == 0.0
    t0 = a["tau0"]
    for gap in (0.05, 1.0, 3.0):
        b = D.RepulsiveSurfaceSession(P, F, ccd=True, ccd_gap=gap).step()
        assert b["tau_ccd"] is not None and b["tau_ccd"] <= t0
        assert b["seconds"]["ccd"] > 0.0
        if b["tau_ccd"] == t0:  # no contact before the first trial: nothing changes
            assert b["tau0"] == t0 and b["energy_after"] == a["energy_after"]
        else:
            assert b["tau0"] == min(t0, 2.0 / 3.0 * b["tau_ccd"])
        assert b["energy_after"] < b["energy_before"]


def test_a_scene_file_runs(tmp_path):
    """A scene of the reference program's format runs through the session
    (crates/ddg-py/python-tests/test_repulsive_surfaces.py:739-772 does the same)."""
    from rs_gb300 import obj

    P, F = _torus()
    obj.write_obj(tmp_path / "t.obj", P, F)
    (tmp_path / "t.scene").write_text("repel_mesh t.obj 6 12\nconstrain barycenter\nconstrain volume\n"
                                      "iteration_limit 3\n")
    p, f, o = D.repulsive_surface_scene(tmp_path / "t.scene")
    s = D.RepulsiveSurfaceSession(p, f, **o)
    end = s.run()
    assert (end["end"], end["status"], end["steps_taken"]) == ("final", "max_iterations", 3)
    Q = np.frombuffer(s.positions, np.float64).reshape(-1, 3)
    assert abs(_volume(Q, F) - _volume(P, F)) <= 1e-6 * abs(_volume(P, F))
    assert end["energy_after"] < end["energy_before"]
