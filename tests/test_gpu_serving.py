"""Serving loop: jobs admitted by HBM footprint, sampling + E_loc of the
ready jobs launched as one shared CUDA graph, solves overlapping on their own
streams; every job's result equals its result alone (tolerance 1e-9 relative
on the final parameters and the energies: only the FP32 atomic column sums of
the SNR contraction may round differently between runs)."""

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
