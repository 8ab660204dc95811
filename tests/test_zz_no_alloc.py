"""The allocation-free entry point vmc_rbm_grad_stats_noalloc.

Callers that cannot allocate device memory where they need the statistics
(an XLA FFI handler, a runtime with a fixed memory budget, code inside a
stream capture) call this variant: it takes its scratch from a static
32 MiB device array inside the library.  These tests call it through the C
ABI and compare it with vmc_rbm_grad_stats (caller workspace) on two calls
in a row; this file is collected last on purpose."""

import ctypes

import numpy as np
import pytest
import torch


def _inputs(N, L, M, seed, dev):
    g = torch.Generator().manual_seed(seed)
    cfg = torch.randint(0, 2, (N, L), generator=g, dtype=torch.int32).to(dev)
    W = (0.1 * torch.randn(L, M, dtype=torch.complex128, generator=g)).to(dev)
    b = (0.1 * torch.randn(M, dtype=torch.complex128, generator=g)).to(dev)
    w = torch.rand(N, dtype=torch.float64, generator=g).to(dev)
    w = w / w.sum()
    E = torch.randn(N, dtype=torch.complex128, generator=g).to(dev)
    emean = (w.to(torch.complex128) * E).sum().reshape(1)
    return cfg, W, b, w, E, emean


def test_noalloc_rejects_oversized_problem_without_a_gpu():
    import vmc_jax_gb300._lib as L
    lib = L.load()
    p = ctypes.c_void_p(256)
    rc = lib.vmc_rbm_grad_stats_noalloc(0, p, 16384, 64, 256, p, p, p, p, p, p, p, None)
    assert rc == 2
    assert b"static scratch" in lib.vmc_last_error_string()


@pytest.mark.gpu
def test_noalloc_matches_workspace_entry_point(cuda):
    import vmc_jax_gb300._lib as L
    for call, (N, L_, M, prec) in enumerate([(1024, 10, 20, 0), (3000, 16, 48, 1)]):
        cfg, W, b, w, E, emean = _inputs(N, L_, M, seed=call, dev=cuda)
        if prec == 1:
            W, b = W.to(torch.complex64), b.to(torch.complex64)
        P = L_ * M + M
        ref_m = torch.empty(P, dtype=torch.complex128, device=cuda)
        ref_f = torch.empty(P, dtype=torch.complex128, device=cuda)
        ws = torch.empty(L.query("vmc_rbm_grad_stats_workspace_bytes", N, L_, M), dtype=torch.uint8, device=cuda)
        L.call("vmc_rbm_grad_stats", prec, L.ptr(cfg), N, L_, M, L.ptr(W), L.ptr(b), L.ptr(w), L.ptr(E),
               L.ptr(emean), L.ptr(ref_m), L.ptr(ref_f), L.ptr(ws), ws.numel(), L.stream())
        got_m = torch.full((P,), float("nan"), dtype=torch.complex128, device=cuda)
        got_f = torch.full((P,), float("nan"), dtype=torch.complex128, device=cuda)
        L.call("vmc_rbm_grad_stats_noalloc", prec, L.ptr(cfg), N, L_, M, L.ptr(W), L.ptr(b), L.ptr(w), L.ptr(E),
               L.ptr(emean), L.ptr(got_m), L.ptr(got_f), L.stream())
        torch.cuda.synchronize()
        scale = max(float(ref_m.abs().max()), float(ref_f.abs().max()))
        assert float((got_m - ref_m).abs().max()) <= 1e-12 * scale
        assert float((got_f - ref_f).abs().max()) <= 1e-12 * scale
