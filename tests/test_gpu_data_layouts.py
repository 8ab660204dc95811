"""The centred-data producers of the S/F build and the SNR transform
(vmc_rbm_centered_gradients, vmc_rbm_snr_data; stats.py:197-205, 255-292):
BF16 hi/lo planes against the complex128 output of the same call, and the
paired-store path (even leading dimension) against the per-element path (odd
leading dimension), which must give bitwise the same planes."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _case(L, M, N, dev, seed=0):
    rng = np.random.default_rng(seed)
    # theta stays well inside |Im theta| < pi/2, away from the poles of tanh
    # where FP32 and FP64 evaluations of the same input part by more than the
    # format's rounding
    sd = 0.3 / np.sqrt(L)
    W = torch.as_tensor(rng.normal(0, sd, (L, M)) + 1j * rng.normal(0, sd, (L, M)), device=dev).contiguous()
    b = torch.as_tensor(rng.normal(0, 0.1, M) + 1j * rng.normal(0, 0.1, M), device=dev).contiguous()
    s = torch.as_tensor(rng.integers(0, 2, (N, L)).astype(np.int32), device=dev)
    w = torch.as_tensor(rng.uniform(0.5, 1.5, N), device=dev)
    w /= w.sum()
    P = L * M + M
    om = torch.as_tensor(rng.normal(0, 0.05, P) + 1j * rng.normal(0, 0.05, P), device=dev)
    E = torch.as_tensor(rng.normal(0, 1, N) + 1j * rng.normal(0, 0.1, N), device=dev)
    Em = torch.as_tensor(np.array([0.3 - 0.1j]), device=dev)
    f = torch.as_tensor(rng.normal(0, 0.01, P) + 1j * rng.normal(0, 0.01, P), device=dev)
    return W, b, s, w, om, E, Em, f, P


def _planes(hi, lo):
    return hi.double() + lo.double()


# (64, 256, 300): the 64-site shapes, even P; (6, 3, 33): odd P and odd N
@pytest.mark.parametrize("L,M,N", [(64, 256, 300), (6, 3, 33), (10, 20, 1000)])
def test_centered_gradient_planes(cuda, L, M, N):
    import vmc_jax_gb300._lib as Lb
    W, b, s, w, om, E, Em, f, P = _case(L, M, N, cuda)
    st = Lb.stream()
    X = torch.empty((N, P), dtype=torch.complex128, device=cuda)
    Lb.call("vmc_rbm_centered_gradients", 0, Lb.ptr(s), N, L, M, Lb.ptr(W), Lb.ptr(b), Lb.ptr(w), Lb.ptr(om), 0,
            Lb.ptr(X), None, P, st)
    W32, b32 = W.to(torch.complex64), b.to(torch.complex64)
    out = {}
    for ld in ((N + 63) // 64 * 64, (N + 63) // 64 * 64 + 1):  # paired stores / per-element stores
        hi = torch.zeros((2 * P, ld), dtype=torch.bfloat16, device=cuda)
        lo = torch.zeros_like(hi)
        Lb.call("vmc_rbm_centered_gradients", 1, Lb.ptr(s), N, L, M, Lb.ptr(W32), Lb.ptr(b32), Lb.ptr(w),
                Lb.ptr(om), 2, Lb.ptr(hi), Lb.ptr(lo), ld, st)
        torch.cuda.synchronize()
        assert not hi[:, N:].any() and not lo[:, N:].any()  # padding columns untouched
        out[ld] = (hi[:, :N].clone(), lo[:, :N].clone())
    (h0, l0), (h1, l1) = out.values()
    assert torch.equal(h0, h1) and torch.equal(l0, l1)
    got = _planes(h0, l0)
    want = torch.cat([X.real.T, X.imag.T], 0)
    scale = want.abs().max()
    assert ((got - want).abs().max() / scale) < 3e-5


@pytest.mark.parametrize("L,M,N", [(64, 256, 300), (6, 3, 33), (10, 20, 1000)])
def test_snr_data_planes(cuda, L, M, N):
    import vmc_jax_gb300._lib as Lb
    W, b, s, w, om, E, Em, f, P = _case(L, M, N, cuda, seed=1)
    st = Lb.stream()
    H = torch.empty((N, P), dtype=torch.complex128, device=cuda)
    Lb.call("vmc_rbm_snr_data", 0, Lb.ptr(s), N, L, M, Lb.ptr(W), Lb.ptr(b), Lb.ptr(w), Lb.ptr(om), Lb.ptr(E),
            Lb.ptr(Em), 1.0, 0.0, Lb.ptr(f), 0, Lb.ptr(H), None, P, st)
    W32, b32 = W.to(torch.complex64), b.to(torch.complex64)
    out = {}
    for ld in (2 * P + 2, 2 * P + 1):  # paired stores when P is even / per-element stores
        hi = torch.zeros((N, ld), dtype=torch.bfloat16, device=cuda)
        lo = torch.zeros_like(hi)
        Lb.call("vmc_rbm_snr_data", 1, Lb.ptr(s), N, L, M, Lb.ptr(W32), Lb.ptr(b32), Lb.ptr(w), Lb.ptr(om),
                Lb.ptr(E), Lb.ptr(Em), 1.0, 0.0, Lb.ptr(f), 2, Lb.ptr(hi), Lb.ptr(lo), ld, st)
        torch.cuda.synchronize()
        assert not hi[:, 2 * P:].any() and not lo[:, 2 * P:].any()
        out[ld] = (hi[:, :2 * P].clone(), lo[:, :2 * P].clone())
    (h0, l0), (h1, l1) = out.values()
    assert torch.equal(h0, h1) and torch.equal(l0, l1)
    got = _planes(h0, l0)
    want = torch.cat([H.real, H.imag], 1)
    scale = want.abs().max()
    assert ((got - want).abs().max() / scale) < 3e-5
