"""initcheck-style poisoning (no sanitizer on this pool): output buffers are
filled with NaN before a call, and every element the call owns must be
overwritten with a finite value afterwards."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _nan(shape, dtype, device):
    t = torch.empty(shape, dtype=dtype, device=device)
    t.fill_(float("nan"))
    return t


def _rbm(L, M, dev, seed=0):
    rng = np.random.default_rng(seed)
    W = torch.as_tensor(rng.normal(0, 0.1, (L, M)) + 1j * rng.normal(0, 0.1, (L, M)), device=dev)
    b = torch.as_tensor(rng.normal(0, 0.1, M) + 1j * rng.normal(0, 0.1, M), device=dev)
    return W.contiguous(), b.contiguous()


@pytest.mark.parametrize("L,M,N", [(10, 20, 1000), (64, 256, 300), (7, 3, 33)])
def test_rbm_outputs_fully_written(cuda, L, M, N):
    import vmc_jax_gb300._lib as Lb
    W, b = _rbm(L, M, cuda)
    s = torch.as_tensor(np.random.default_rng(1).integers(0, 2, (N, L)).astype(np.int32), device=cuda)
    st = Lb.stream()
    P = L * M + M
    lp = _nan((N,), torch.complex128, cuda)
    Lb.call("vmc_rbm_logpsi", 0, Lb.ptr(s), N, L, M, Lb.ptr(W), Lb.ptr(b), Lb.ptr(lp), st)
    assert torch.isfinite(torch.view_as_real(lp)).all()
    for layout, width in ((0, 2 * P), (1, P)):
        g = _nan((N, width), torch.complex128, cuda)
        Lb.call("vmc_rbm_gradients", 0, Lb.ptr(s), N, L, M, Lb.ptr(W), Lb.ptr(b), layout, Lb.ptr(g), st)
        assert torch.isfinite(torch.view_as_real(g)).all()
    w = torch.full((N,), 1.0 / N, dtype=torch.float64, device=cuda)
    om = torch.zeros(P, dtype=torch.complex128, device=cuda)
    X = _nan((N, P), torch.complex128, cuda)
    Lb.call("vmc_rbm_centered_gradients", 0, Lb.ptr(s), N, L, M, Lb.ptr(W), Lb.ptr(b), Lb.ptr(w), Lb.ptr(om), 0,
            Lb.ptr(X), None, P, st)
    assert torch.isfinite(torch.view_as_real(X)).all()
    # transposed bf16 planes: the N valid columns of every one of the 2P rows
    ld = (N + 63) // 64 * 64
    hi = _nan((2 * P, ld), torch.bfloat16, cuda)
    lo = _nan((2 * P, ld), torch.bfloat16, cuda)
    W32, b32 = W.to(torch.complex64), b.to(torch.complex64)  # kept alive across the launch
    Lb.call("vmc_rbm_centered_gradients", 1, Lb.ptr(s), N, L, M, Lb.ptr(W32), Lb.ptr(b32), Lb.ptr(w), Lb.ptr(om), 2,
            Lb.ptr(hi), Lb.ptr(lo), ld, st)
    assert torch.isfinite(hi[:, :N].float()).all() and torch.isfinite(lo[:, :N].float()).all()


def test_symnet_and_cnn_outputs_fully_written(cuda):
    import vmc_jax_gb300 as V
    import vmc_jax_gb300._lib as Lb
    from vmc_jax_gb300.util import symmetries as S
    L, M, N = 12, 5, 257
    psi = V.vqs.NQS(V.nets.CpxRBM(M, True), orbit=S.get_orbit_1D(L, "translation", "reflection"))
    psi(np.zeros((1, 1, L), np.int32))
    s = torch.as_tensor(np.random.default_rng(2).integers(0, 2, (N, L)).astype(np.int32), device=cuda)
    pr = psi.params
    lp = _nan((N,), torch.complex128, cuda)
    Lb.call("vmc_sym_rbm_logpsi", 0, Lb.ptr(s), N, L, M, Lb.ptr(pr["kernel"]), Lb.ptr(pr["bias"]),
            Lb.ctypes_ref(psi.net.desc(cuda)), Lb.ptr(lp), Lb.stream())
    assert torch.isfinite(torch.view_as_real(lp)).all()
    P = L * M + M
    g = _nan((N, 2 * P), torch.complex128, cuda)
    Lb.call("vmc_sym_rbm_gradients", 0, Lb.ptr(s), N, L, M, Lb.ptr(pr["kernel"]), Lb.ptr(pr["bias"]),
            Lb.ctypes_ref(psi.net.desc(cuda)), 0, Lb.ptr(g), Lb.stream())
    assert torch.isfinite(torch.view_as_real(g)).all()
    net = V.nets.CNN(F=(3, 3), channels=(4, 3), strides=(1, 1))
    cpsi = V.vqs.NQS(net)
    cpsi(np.zeros((1, 1, 5, 5), np.int32))
    cs = torch.as_tensor(np.random.default_rng(3).integers(0, 2, (N, 25)).astype(np.int32), device=cuda)
    d = net.desc((5, 5))
    flat = net.flat(cpsi.params, "fp64")
    out = _nan((N,), torch.complex128, cuda)
    Lb.call("vmc_cnn_logpsi", 0, Lb.ctypes_ref(d), Lb.ptr(cs), N, Lb.ptr(flat), Lb.ptr(out), Lb.stream())
    assert torch.isfinite(torch.view_as_real(out)).all()
    Pc = flat.numel()
    gc = _nan((N, Pc), torch.complex128, cuda)
    Lb.call("vmc_cnn_gradients", 0, Lb.ctypes_ref(d), Lb.ptr(cs), N, Lb.ptr(flat), 0, Lb.ptr(gc), Lb.stream())
    assert torch.isfinite(torch.view_as_real(gc)).all()


def test_solve_outputs_fully_written(cuda):
    import vmc_jax_gb300._lib as Lb
    P, N = 300, 700
    rng = np.random.default_rng(4)
    X = torch.as_tensor(rng.normal(size=(N, P)) + 1j * rng.normal(size=(N, P)), device=cuda) / np.sqrt(N)
    A = X.mH @ X
    ev, U = torch.linalg.eigh(A)
    U = U.mT.contiguous().mT if U.stride(0) != 1 else U
    f = torch.as_tensor(rng.normal(size=P) + 1j * rng.normal(size=P), device=cuda)
    vtf = _nan((P,), torch.complex128, cuda)
    Lb.call("vmc_zgemv", 1, Lb.ptr(U), U.stride(1), P, Lb.ptr(f), Lb.ptr(vtf), None, 0, Lb.stream())
    assert torch.isfinite(torch.view_as_real(vtf)).all()
    pinv = _nan((P,), torch.float64, cuda)
    res = _nan((3,), torch.float64, cuda)
    ws = torch.empty(Lb.query("vmc_tdvp_regularize_workspace_bytes", P, 1e-8), dtype=torch.uint8, device=cuda)
    Lb.call("vmc_tdvp_regularize", Lb.ptr(ev), Lb.ptr(vtf), None, P, 1e-8, 1e-14, 2.0, Lb.ptr(pinv), Lb.ptr(res),
            Lb.ptr(ws), ws.numel(), Lb.stream())
    assert torch.isfinite(pinv).all() and torch.isfinite(res).all()
    z = _nan((P,), torch.complex128, cuda)
    wz = torch.empty(Lb.query("vmc_zgemv_workspace_bytes", P), dtype=torch.uint8, device=cuda)
    Lb.call("vmc_zgemv", 0, Lb.ptr(U), U.stride(1), P, Lb.ptr(vtf), Lb.ptr(z), Lb.ptr(wz), wz.numel(), Lb.stream())
    assert torch.isfinite(torch.view_as_real(z)).all()
