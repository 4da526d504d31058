"""The outer loop of RepulsiveSurfaceSession on the CPU, over a scripted stand-in for the GPU
flow step: the stop rules, stuck_limit, max_iterations, the ends of run(), cancel, reset and the
error mapping (Engine::step / run, crates/ddg-py/src/repulsive_surfaces.rs:1712-1806;
Session::step, RS/src/step/session.rs:1210-1245)."""
import math

import numpy as np
import pytest

from rs_gb300 import RsError
from rs_gb300 import ddg_tools as D

P = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])
F = np.array([[0, 2, 1], [0, 1, 3], [0, 3, 2], [1, 2, 3]], np.uint32)


def _report(accepted=True, e0=10.0, e1=9.0, slope=1.0):
    return dict(energy_before=e0, energy_after=e1, tau=0.1 if accepted else 0.0, halvings=0.0, gmres_area=0.0,
             gmres_volume=0.0, gmres_direction=5.0, relative_residual=1e-4, seconds=0.01, seconds_tree=0.0,
             seconds_energy=0.0, seconds_solver_build=0.0, seconds_solve=0.0, seconds_line_search=0.0,
             seconds_projection=0.0, accepted=1.0 if accepted else 0.0, slope=slope, constraint_residual=0.0,
             fallbacks=0.0, learned_solves=0.0, learned_fallbacks=0.0, gradient_norm=1.0, tau0=0.1,
             direction_max=1.0, newton_steps=0.0, projection_status=0.0, energy_trial=e1,
             tau_ccd=math.nan, seconds_ccd=0.0)


class FakeFlow:
    """Replays a script of step reports; raises RsError for an entry that is an exception."""

    script = []

    def __init__(self, faces, positions, options, ctx):
        self.i = 0
        self.pos = np.asarray(positions, np.float64).copy()

    def step(self):
        item = FakeFlow.script[min(self.i, len(FakeFlow.script) - 1)]
        self.i += 1
        if isinstance(item, Exception):
            raise item
        if item["accepted"]:
            self.pos = self.pos * 0.99
        return dict(item)

    def positions(self):
        return self.pos.copy()

    def cancel(self, on=True):
        self.cancelled = on


class FakeTree:
    @classmethod
    def build(cls, faces, positions, opts, ctx):
        return cls()

    def try_energy(self, e):
        return 10.0


class FakeCtx:
    def info(self):
        return {"name": "fake"}


@pytest.fixture(autouse=True)
def fake_gpu(monkeypatch):
    monkeypatch.setattr(D, "Flow", FakeFlow)
    monkeypatch.setattr(D, "BhTree", FakeTree)
    monkeypatch.setattr(D, "_context", lambda o: FakeCtx())
    FakeFlow.script = [_report()]
    yield


def test_energy_stall_rule():
    # energies 9, 8, 8, 8: with window 2 the third accepted step compares 9 with 8 (not stalled),
    # the fourth 8 with 8 (stalled)
    FakeFlow.script = [_report(e1=9.0), _report(e1=8.0), _report(e1=8.0), _report(e1=8.0)]
    s = D.RepulsiveSurfaceSession(P, F, stop_window=2, stop_relative=1e-7)
    st = [s.step()["session_status"] for _ in range(4)]
    assert st == ["running", "running", "running", "converged"]
    assert s.status == "converged" and s.iteration == 4 and s.energy == 8.0
    assert s.run()["end"] == "final"


def test_sobolev_rule_and_off():
    FakeFlow.script = [_report(slope=4.0), _report(slope=1.0), _report(slope=0.01)]
    s = D.RepulsiveSurfaceSession(P, F, stop="sobolev", stop_eps=0.2)
    assert [s.step()["session_status"] for _ in range(3)] == ["running", "running", "converged"]
    FakeFlow.script = [_report(e1=8.0)]
    s = D.RepulsiveSurfaceSession(P, F, stop="off", max_iterations=6)
    assert s.run()["steps_taken"] == 6 and s.status == "max_iterations"


def test_stuck_limit():
    FakeFlow.script = [_report(accepted=False)]
    s = D.RepulsiveSurfaceSession(P, F, stuck_limit=3)
    reps = [s.step() for _ in range(3)]
    assert [r["status"] for r in reps] == ["stuck"] * 3
    assert reps[-1]["session_status"] == "stuck" and s.status == "stuck"
    # an accepted step resets the count
    FakeFlow.script = [_report(accepted=False), _report(), _report(accepted=False), _report(accepted=False)]
    s = D.RepulsiveSurfaceSession(P, F, stuck_limit=2)
    assert [s.step()["session_status"] for _ in range(4)] == ["running", "running", "running", "stuck"]


def test_run_ends():
    s = D.RepulsiveSurfaceSession(P, F, stop="off")
    assert s.run(max_steps=3)["end"] == "max_steps"
    seen = []
    assert s.run(max_steps=10, progress=lambda r: seen.append(1) or len(seen) < 2)["end"] == "callback"
    assert s.iteration == 5
    assert s.run(time_limit=0.0)["end"] == "time_limit"
    s.cancel()
    assert s.run()["end"] == "cancelled" and s.step()["status"] == "cancelled" and s.iteration == 5
    s.reset()
    assert (s.iteration, s.status) == (0, "running")
    assert s.positions.tobytes() == P.tobytes()
    s2 = D.RepulsiveSurfaceSession(P, F, stop="off", max_iterations=2)
    end = s2.run()
    assert (end["end"], end["status"], end["steps_taken"]) == ("final", "max_iterations", 2)
    assert s2.run()["steps_taken"] == 0


def test_one_call_flow_reports():
    FakeFlow.script = [_report(e1=9.0), _report(e1=8.0), _report(e1=7.0)]
    q, g, rep = D.repulsive_surface_flow(P, F, steps=3, stop="off")
    assert rep["status"] == "max_iterations" and rep["iterations"] == 3 and len(rep["steps"]) == 3
    assert all(r["session_status"] == "max_iterations" for r in rep["steps"])
    assert rep["energy_initial"] == 10.0 and rep["energy_final"] == 7.0
    assert q.typecode == "d" and g.typecode == "i" and len(rep["face_origin"]) == len(F)
    _, _, rep = D.repulsive_surface_flow(P, F, steps=3, progress=lambda r: False)
    assert rep["status"] == "cancelled" and rep["iterations"] == 1


def test_errors_map_and_set_the_status():
    FakeFlow.script = [_report(), RsError(5, "NonFiniteEnergy", "flow", "non-finite energy")]
    s = D.RepulsiveSurfaceSession(P, F)
    s.step()
    with pytest.raises(D.SolveError):
        s.step()
    assert s.status == "error" and "non-finite" in s.error and s.iteration == 1
    FakeFlow.script = [RsError(1, "InvalidOption", "flow", "bad")]
    s = D.RepulsiveSurfaceSession(P, F)
    with pytest.raises(D.RepulsiveSurfaceInputError):
        s.step()


def test_step_report_keys_follow_the_reference():
    FakeFlow.script = [_report()]
    r = D.RepulsiveSurfaceSession(P, F, constraints=[{"type": "barycenter"}, {"type": "volume"}]).step()
    for k in ("iteration", "status", "session_status", "device", "device_name", "metric_device", "n_vertices",
              "n_faces", "energy_before", "energy_after", "tangent_point_after", "penalties_after",
              "gradient_norm", "sobolev_norm_sq", "tau", "tau0", "tau_ccd", "halvings", "newton_steps",
              "projection", "max_violation", "dropped_rows", "linear", "remesh", "seconds"):
        assert k in r, k
    assert r["linear"]["solves"] == 2 and r["linear"]["dimension"] == 3 * len(P) + 3
    assert r["tau_ccd"] is None and r["remesh"] is None
    assert set(r["seconds"]) == {"bvh", "energy", "factor", "solve", "line_search", "ccd", "projection",
                                 "remesh", "total"}


def test_a_step_stopped_between_trials_is_a_cancelled_step():
    FakeFlow.script = [_report(e1=9.0), RsError(11, "Cancelled", "flow", "the step was cancelled")]
    s = D.RepulsiveSurfaceSession(P, F)
    s.step()
    before = s.positions.tobytes()
    r = s.step()
    assert r["status"] == "cancelled" and s.status == "cancelled" and s.iteration == 1
    assert s.positions.tobytes() == before and s.energy == 9.0
    s.cancel()
    assert s._flow.cancelled and s.run()["end"] == "cancelled"
