"""Serving loop: jobs admitted by HBM footprint, sampling + E_loc of the
ready jobs launched as one shared CUDA graph, solves overlapping on their own
streams; every job's result equals its result alone (tolerance 1e-9 relative
on the final parameters and the energies; every reduction adds in a fixed
order); failures injected on the host stay with their job."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _specs():
    from vmc_jax_gb300.serving import JobSpec
    return [JobSpec(L=8, h=0.8, M=8, num_samples=512, steps=4, seed=1),
            JobSpec(L=12, h=1.2, M=24, num_samples=1024, steps=3, seed=2, arrival=0.02),
            JobSpec(L=10, h=0.5, M=10, num_samples=512, steps=5, seed=3, kind="quench", dt=0.005),
            JobSpec(L=16, h=1.0, M=16, num_samples=2048, steps=2, seed=4, arrival=0.05)]


def _rel(a, b):
    a, b = a.double(), b.double()
    return float((a - b).abs().max() / b.abs().max())


def test_results_alone_equal_results_in_the_mix(cuda):
    from vmc_jax_gb300.serving import Server
    specs = _specs()
    alone = []
    for sp in specs:
        srv = Server(max_slots=1)
        jid = srv.submit(sp)
        srv.run()
        alone.append(srv.result(jid))
    srv = Server(max_slots=4)
    ids = [srv.submit(sp) for sp in specs]
    rep = srv.run()
    assert rep["jobs"] == len(specs)
    assert rep["steps"] == sum(sp.steps for sp in specs)
    assert rep["step_latency_s"]["p99"] >= rep["step_latency_s"]["p50"] > 0
    assert rep["graph_launches"] < rep["steps"]  # several jobs share launches
    for jid, (th, en) in zip(ids, alone):
        th2, en2 = srv.result(jid)
        assert _rel(th2, th) < 1e-9
        assert _rel(en2, en) < 1e-9


def test_admission_by_footprint(cuda):
    from vmc_jax_gb300.serving import Server, footprint_bytes
    specs = _specs()
    budget = sorted(footprint_bytes(s) for s in specs)
    srv = Server(hbm_budget=budget[-1] + budget[-2], max_slots=8)
    for sp in specs:
        srv.submit(sp)
    rep = srv.run()
    assert rep["jobs"] == len(specs)
    assert rep["max_resident_jobs"] <= 2


def test_failures_stay_with_their_job(cuda):
    """Host-side fault injection (nothing faults on the GPU): an invalid spec
    is refused, a job larger than the whole budget is rejected, a job whose
    step callback raises fails alone, a queued job is cancelled; the other
    jobs finish with the results they have alone."""
    from vmc_jax_gb300.serving import JobSpec, Server, footprint_bytes
    specs = _specs()
    srv = Server(max_slots=4)
    with pytest.raises(ValueError):
        srv.submit(JobSpec(L=8, h=1.0, M=8, num_samples=256, kind="annealing"))

    def boom(job_id, step, energy):
        if step == 2:
            raise RuntimeError("client callback failed")
    import dataclasses
    bad = dataclasses.replace(specs[2], on_step=boom)
    huge = JobSpec(L=64, h=1.0, M=256, num_samples=16384, steps=1)
    budget = 2 * max(footprint_bytes(s) for s in specs)
    assert footprint_bytes(huge) > budget
    srv = Server(hbm_budget=budget, max_slots=4)
    ok0 = srv.submit(specs[0])
    failing = srv.submit(bad)
    too_big = srv.submit(huge)
    withdrawn = srv.submit(dataclasses.replace(specs[1], arrival=5.0))
    srv.cancel(withdrawn)
    ok3 = srv.submit(specs[3])
    rep = srv.run()
    assert srv.status(ok0) == "done" and srv.status(ok3) == "done"
    assert srv.status(failing) == "failed" and "client callback failed" in srv.errors[failing]
    assert srv.status(too_big) == "rejected"
    assert srv.status(withdrawn) == "cancelled"
    assert rep["not_completed"] == {failing: "failed", too_big: "rejected", withdrawn: "cancelled"}
    with pytest.raises(KeyError):
        srv.result(failing)
    # the surviving jobs are unaffected
    for jid, sp in ((ok0, specs[0]), (ok3, specs[3])):
        alone = Server(max_slots=1)
        a = alone.submit(sp)
        alone.run()
        th, en = alone.result(a)
        th2, en2 = srv.result(jid)
        assert _rel(th2, th) < 1e-9 and _rel(en2, en) < 1e-9
