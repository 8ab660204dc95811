"""Properties at the 64-site workload's full dimensions (L=64, M=256,
P=16,640, 2P=33,280 Gram rows, N_s=16,384), where an element-by-element
oracle comparison of everything would take too long:

* Metropolis chains bit-exact against the oracle for a subset of chains;
* fused E_loc against the oracle on a subset of samples;
* the S-build Gram at 33,280 rows: every sampled upper entry against the
  FP64 product of the same BF16 planes, and the Hermitian assembly
  (A Hermitian, sampled entries);
* the SNR contraction at N_s x 2P x 2P with a signed permutation as the
  eigenvector matrix: every column sum of squares equals the squared norm of
  the permuted column (orthogonal invariance), to BF16x3 accuracy."""

import numpy as np
import pytest
import torch

from oracle import jvmc_oracle as O

pytestmark = pytest.mark.gpu

L, M = 64, 256


def _pair(seed=0, scale=0.05):
    import vmc_jax_gb300 as V
    rng = np.random.default_rng(seed)
    prm = O.init_cpx_rbm(L, M, True, rng, scale=scale)
    opsi = O.NQS(O.CpxRBM(M, True), prm)
    psi = V.vqs.NQS(V.nets.CpxRBM(numHidden=M, bias=True))
    psi(np.zeros((1, 1, L), np.int32))
    psi.set_parameters(opsi.get_parameters())
    return psi, opsi


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def test_metropolis_and_eloc_at_full_shape(cuda):
    import vmc_jax_gb300 as V
    psi, opsi = _pair()
    mc = V.sampler.MCSampler(psi, (L,), 2024, updateProposer=V.sampler.propose_spin_flip, numChains=8,
                             numSamples=16, thermalizationSweeps=2, sweepSteps=L)
    mco = O.MCSampler(opsi, (L,), 2024, numChains=8, numSamples=16, thermalizationSweeps=2, sweepSteps=L)
    s, lp, p = mc.sample()
    so, lpo, po = mco.sample()
    assert np.array_equal(s.cpu().numpy(), so)
    assert _rel(lp.cpu().numpy(), lpo) < 1e-12
    H = V.operator.BranchFreeOperator()
    for l in range(L):
        H.add(V.operator.scal_opstr(-1.0, (V.operator.Sz(l), V.operator.Sz((l + 1) % L))))
        H.add(V.operator.scal_opstr(-1.0, (V.operator.Sx(l),)))
    cfg = np.random.default_rng(5).integers(0, 2, (1, 64, L)).astype(np.int32)
    assert _rel(H.get_O_loc(cfg, psi).cpu().numpy(), O.tfim(L, 1.0, 1.0).get_O_loc(cfg, opsi)) < 1e-11


def _planes(x, ld):
    rows, k = x.shape
    hi = torch.zeros((rows, ld), dtype=torch.bfloat16, device=x.device)
    lo = torch.zeros((rows, ld), dtype=torch.bfloat16, device=x.device)
    h = x.to(torch.bfloat16)
    hi[:, :k] = h
    lo[:, :k] = (x - h.float()).to(torch.bfloat16)
    return hi, lo


def test_gram_and_hermitian_at_full_rows(cuda):
    import vmc_jax_gb300._lib as Lb
    P = L * M + M
    R, k = 2 * P, 256
    torch.manual_seed(7)
    x = torch.randn(R, k, device=cuda) / 16
    hi, lo = _planes(x, k)
    ldg = (R + 15) // 16 * 16
    G = torch.empty((R, ldg), dtype=torch.float32, device=cuda)
    Lb.call("vmc_gram_bf16x3", Lb.ptr(hi), Lb.ptr(lo), R, k, k, Lb.ptr(G), ldg, 3, None, Lb.stream())
    torch.cuda.synchronize()
    assert Lb.query("vmc_tc_error_flag", 1) == 0
    rng = np.random.default_rng(8)
    i = torch.as_tensor(rng.integers(0, R, 4096), device=cuda)
    j = torch.as_tensor(rng.integers(0, R, 4096), device=cuda)
    r, c = torch.minimum(i, j), torch.maximum(i, j)
    hh, ll = hi.double(), lo.double()
    want = (hh[r] * hh[c]).sum(1) + (hh[r] * ll[c]).sum(1) + (ll[r] * hh[c]).sum(1)
    got = G[r, c].double()
    assert torch.isfinite(got).all()
    scale = torch.sqrt((hh * hh).sum(1).max())
    assert float((got - want).abs().max() / scale ** 2) < 2e-5
    # Hermitian assembly of the complex P x P matrix from the real Gram
    A = torch.empty((P, P), dtype=torch.complex128, device=cuda)
    Lb.call("vmc_gram_to_hermitian", Lb.VMC_F32, Lb.ptr(G), ldg, P, 0.0, Lb.ptr(A), Lb.stream())
    a = torch.as_tensor(rng.integers(0, P, 2048), device=cuda)
    b = torch.as_tensor(rng.integers(0, P, 2048), device=cuda)
    assert torch.equal(A[a, b], torch.conj(A[b, a]))
    aa, bb = torch.minimum(a, b), torch.maximum(a, b)
    re = G[aa, bb].double() + G[P + aa, P + bb].double()
    im = G[aa, P + bb].double() - G[bb, P + aa].double()
    im = torch.where(aa == bb, torch.zeros_like(im), im)
    assert torch.equal(A[aa, bb], torch.complex(re, im))


def test_snr_contraction_at_full_shape(cuda):
    import vmc_jax_gb300._lib as Lb
    N, R = 16384, 2 * (L * M + M)
    torch.manual_seed(9)
    a = torch.randn(N, R, device=cuda) / 64
    ah, al = _planes(a, R)
    # eigenvector planes: a signed permutation (orthogonal, exact in BF16)
    perm = torch.randperm(R, device=cuda)
    sign = torch.where(torch.rand(R, device=cuda) < 0.5, -1.0, 1.0)
    bh = torch.zeros((R, R), dtype=torch.bfloat16, device=cuda)
    bh[torch.arange(R, device=cuda), perm] = sign.to(torch.bfloat16)
    bl = torch.zeros_like(bh)
    colsq = torch.empty(R, dtype=torch.float32, device=cuda)
    ws = torch.empty(Lb.query("vmc_gemm_bf16x3_colsq_workspace_bytes", N, R), dtype=torch.uint8, device=cuda)
    Lb.call("vmc_gemm_bf16x3_colsq", Lb.ptr(ah), Lb.ptr(al), N, R, Lb.ptr(bh), Lb.ptr(bl), R, R, R, Lb.ptr(colsq),
            Lb.ptr(ws), ws.numel(), 3, None, Lb.stream())
    torch.cuda.synchronize()
    assert Lb.query("vmc_tc_error_flag", 1) == 0
    v = ah.double() + al.double()
    want = (v[:, perm] ** 2).sum(0)
    assert float(((colsq.double() - want).abs() / want).max()) < 2e-5
