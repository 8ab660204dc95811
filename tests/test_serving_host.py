"""Host logic of the serving loop (vmc_jax_gb300.serving.Server) on the CPU:
admission against the slot count and the HBM budget, per-job failure,
cancellation and the report, with the device side (slot buffers, the shared
sampling graph, the FP64 solve) replaced by a stand-in that sleeps.  The
GPU path itself is covered by tests/test_gpu_serving.py."""

import threading
import time

import pytest
import torch

from vmc_jax_gb300 import serving


class FakeSlot:
    """A job's step: sleeps, records an energy, calls on_step; a job whose
    seed is 13 raises in its second step."""

    def __init__(self, job_id, spec, arrival_wall):
        self.id = job_id
        self.spec = spec
        self.arrival_wall = arrival_wall
        self.steps_done = 0
        self.step_latencies = []
        self.energies = []
        self.theta = torch.zeros(4, dtype=torch.float64)

    def solve(self, ready_event, t_launch):
        time.sleep(0.002)
        if self.spec.seed == 13 and self.steps_done == 1:
            raise RuntimeError("planted failure")
        self.energies.append(torch.tensor(-float(self.steps_done)))
        self.theta = self.theta + 1.0
        self.steps_done += 1
        self.step_latencies.append(time.perf_counter() - t_launch)
        if self.spec.on_step is not None:
            self.spec.on_step(self.id, self.steps_done, float(self.energies[-1]))

    @property
    def finished(self):
        return self.steps_done >= self.spec.steps


class HostServer(serving.Server):
    def __init__(self, **kw):
        self.launched = []
        self.resident_seen = []
        super().__init__(**kw)

    def _open_device(self):
        return None

    def _new_slot(self, job_id, spec, arrival_wall):
        return FakeSlot(job_id, spec, arrival_wall)

    def _launch(self, ids):
        self.launched.append(tuple(ids))
        self.resident_seen.append(len(self.active))
        return None, time.perf_counter()


def _spec(steps=3, **kw):
    return serving.JobSpec(L=8, h=1.0, M=8, num_samples=256, steps=steps, **kw)


def _run(server, timeout=60.0):
    out = {}
    th = threading.Thread(target=lambda: out.setdefault("report", server.run()), daemon=True)
    th.start()
    th.join(timeout)
    assert not th.is_alive(), "serving loop did not finish"
    return out["report"]


def test_all_jobs_complete_in_order():
    srv = HostServer(hbm_budget=1 << 40, max_slots=4, batch_window=0.0)
    seen = {}
    cb = lambda jid, step, e: seen.setdefault(jid, []).append(step)
    ids = [srv.submit(_spec(steps=3 + i % 2, arrival=0.001 * i, on_step=cb)) for i in range(6)]
    rep = _run(srv)
    assert rep["jobs"] == 6 and rep["not_completed"] == {}
    assert rep["steps"] == sum(3 + i % 2 for i in range(6))
    assert all(srv.status(i) == "done" for i in ids)
    for i in ids:
        assert seen[i] == list(range(1, srv.done[i].spec.steps + 1))
        theta, energies = srv.result(i)
        assert energies.shape[0] == srv.done[i].spec.steps
    assert max(srv.resident_seen) <= 4 and rep["max_resident_jobs"] <= 4
    assert rep["graph_launches"] == len(srv.launched)


def test_budget_rejects_and_defers():
    one = serving.footprint_bytes(_spec())
    srv = HostServer(hbm_budget=2 * one + 1, max_slots=8, batch_window=0.0)
    big = serving.JobSpec(L=64, h=1.0, M=256, num_samples=16384, steps=1)
    assert serving.footprint_bytes(big) > srv.hbm_budget
    jb = srv.submit(big)
    small = [srv.submit(_spec()) for _ in range(5)]
    rep = _run(srv)
    assert srv.status(jb) == "rejected" and "HBM budget" in srv.errors[jb]
    assert all(srv.status(i) == "done" for i in small)
    assert rep["max_resident_jobs"] == 2  # two footprints fit the budget at a time
    assert rep["not_completed"] == {jb: "rejected"}
    with pytest.raises(KeyError, match="rejected"):
        srv.result(jb)


def test_failure_stays_with_its_job():
    srv = HostServer(hbm_budget=1 << 40, max_slots=4, batch_window=0.0)
    bad = srv.submit(_spec(steps=4, seed=13))
    good = [srv.submit(_spec(steps=4, seed=s)) for s in range(3)]
    rep = _run(srv)
    assert srv.status(bad) == "failed" and "planted failure" in srv.errors[bad]
    assert all(srv.status(i) == "done" for i in good)
    assert rep["jobs"] == 3 and rep["steps"] == 12
    assert "planted failure" in rep["errors"][bad] and set(rep["errors"]) == {bad}


class LaunchFailServer(HostServer):
    """The sampling launch of a job whose seed is 7 fails from its third step
    on (e.g. its graph cannot be captured), alone or together with others."""

    def _launch(self, ids):
        if any(self.active[i].spec.seed == 7 and self.active[i].steps_done >= 2 for i in ids):
            raise RuntimeError("capture failed")
        return super()._launch(ids)


def test_failed_launch_stays_with_its_job():
    srv = LaunchFailServer(hbm_budget=1 << 40, max_slots=4, batch_window=0.0)
    bad = srv.submit(_spec(steps=5, seed=7))
    good = [srv.submit(_spec(steps=5, seed=s)) for s in (1, 2, 3)]
    rep = _run(srv)
    assert srv.status(bad) == "failed" and "capture failed" in srv.errors[bad]
    assert srv.done.get(bad) is None and bad not in srv.active
    assert all(srv.status(i) == "done" for i in good)
    assert rep["steps"] == 15 and rep["not_completed"] == {bad: "failed"}
    # after the failure the other jobs were launched on their own
    assert any(len(k) == 1 for k in srv.launched)


class ReplayFailServer(HostServer):
    """The replay of any launch that contains the job with seed 9 fails at
    its second step, after it may have enqueued other jobs' work."""

    def _launch(self, ids):
        if any(self.active[i].spec.seed == 9 and self.active[i].steps_done == 1 for i in ids):
            self.launched.append(("replay-failed",) + tuple(ids))
            raise serving.ReplayError("illegal address")
        return super()._launch(ids)


def test_failed_replay_is_not_run_again():
    """Jobs of a replay that failed are failed, not re-launched on their own:
    their chains may already have advanced in this step."""
    srv = ReplayFailServer(hbm_budget=1 << 40, max_slots=4, batch_window=0.0)
    bad = srv.submit(_spec(steps=3, seed=9))
    rep = _run(srv)
    assert srv.status(bad) == "failed" and "replay" in srv.errors[bad]
    failed_launch = [k for k in srv.launched if k[0] == "replay-failed"]
    assert len(failed_launch) == 1
    # nothing of that launch was retried job by job
    others = set(failed_launch[0][1:])
    assert all(srv.status(i) == "failed" for i in others)
    assert srv.done.get(bad) is None and rep["not_completed"][bad] == "failed"


def test_cancel_queued_and_active():
    srv = HostServer(hbm_budget=1 << 40, max_slots=2, batch_window=0.0)

    def stop_after_two(jid, step, e):
        if step == 2:
            srv.cancel(jid)

    active = srv.submit(_spec(steps=10, on_step=stop_after_two))
    late = srv.submit(_spec(steps=2, arrival=30.0))  # not yet arrived: still queued
    other = srv.submit(_spec(steps=3))
    srv.cancel(late)
    assert srv.status(late) == "cancelled"
    rep = _run(srv)
    assert srv.status(active) == "cancelled"
    assert srv.status(other) == "done"
    assert rep["not_completed"] == {active: "cancelled", late: "cancelled"}


def test_invalid_specs_are_refused_at_submit():
    srv = HostServer(hbm_budget=1 << 30)
    for bad in (serving.JobSpec(L=1, h=1.0, M=4, num_samples=64),
                serving.JobSpec(L=8, h=1.0, M=4, num_samples=64, kind="annealing"),
                serving.JobSpec(L=8, h=1.0, M=4, num_samples=64, precision="fp16")):
        with pytest.raises(ValueError):
            srv.submit(bad)
    assert srv.states == {}


def test_launch_plan_shares_recurring_sets():
    """A set of ready jobs gets a shared graph from its second launch on;
    a new set and a single job replay the jobs' own graphs; a set is
    forgotten with its jobs."""
    srv = HostServer(hbm_budget=1 << 40)
    assert srv._launch_plan([2, 1]) == (False, (1, 2))
    assert srv._launch_plan([1, 2]) == (True, (1, 2))
    assert srv._launch_plan([3]) == (False, (3,))
    assert srv._launch_plan([3]) == (False, (3,))
    assert srv._launch_plan([1, 3]) == (False, (1, 3))
    srv.graphs[(1, 2)] = object()
    assert srv._launch_plan([1, 2]) == (True, (1, 2))
