"""torch.autograd.Function over log psi: the O_k backward kernels against
central finite differences (torch.autograd.gradcheck, FP64) and against the
oracle's Jacobian."""

import numpy as np
import pytest
import torch

from oracle import jvmc_oracle as O

pytestmark = pytest.mark.gpu


def test_rbm_autograd_gradcheck(cuda):
    import vmc_jax_gb300 as V
    from vmc_jax_gb300.autograd import log_psi
    psi = V.vqs.NQS(V.nets.CpxRBM(numHidden=5, bias=True))
    s = np.random.default_rng(0).integers(0, 2, (1, 12, 6)).astype(np.int32)
    psi(s)
    theta = (0.2 * torch.randn(psi.get_parameters().numel(), dtype=torch.float64, device=cuda)).requires_grad_()
    assert torch.autograd.gradcheck(lambda t: log_psi(psi, t, s), (theta,), eps=1e-6, atol=1e-7, rtol=1e-6)


def test_rbm_vjp_matches_jacobian(cuda):
    import vmc_jax_gb300 as V
    from vmc_jax_gb300.autograd import log_psi
    rng = np.random.default_rng(1)
    L, M = 16, 24
    prm = O.init_cpx_rbm(L, M, True, rng, scale=0.2)
    opsi = O.NQS(O.CpxRBM(M, True), prm)
    psi = V.vqs.NQS(V.nets.CpxRBM(numHidden=M, bias=True))
    s = rng.integers(0, 2, (1, 500, L)).astype(np.int32)
    psi(s)
    theta = torch.as_tensor(opsi.get_parameters(), device=cuda).requires_grad_()
    out = log_psi(psi, theta, s)
    gr = torch.as_tensor(rng.normal(size=(500, 2)), device=cuda)
    (out * gr).sum().backward()
    # oracle: d log psi / d [Re theta; Im theta] from the 2P holomorphic layout
    J = opsi.gradients(s)[0]                       # (N, 2P) complex = d log psi / d theta_flat
    ref = (gr[:, 0].cpu().numpy() @ J.real + gr[:, 1].cpu().numpy() @ J.imag)
    assert np.max(np.abs(theta.grad.cpu().numpy() - ref)) / np.max(np.abs(ref)) < 1e-12


def test_cnn_autograd_chunked(cuda):
    import vmc_jax_gb300 as V
    from vmc_jax_gb300.autograd import log_psi
    net = V.nets.CNN(F=(3, 3), channels=(4, 4), strides=(1, 1), actFun=("poly4",))
    psi = V.vqs.NQS(net)
    s = np.random.default_rng(2).integers(0, 2, (1, 40, 5, 5)).astype(np.int32)
    psi(s)
    theta = (0.3 * torch.randn(psi.get_parameters().numel(), dtype=torch.float64, device=cuda)).requires_grad_()
    # a chunk of 7 configurations at a time: the Jacobian never exists in full
    f = lambda t: log_psi(psi, t, s, chunk_bytes=7 * 8 * theta.numel())
    assert torch.autograd.gradcheck(f, (theta,), eps=1e-6, atol=1e-7, rtol=1e-6)
