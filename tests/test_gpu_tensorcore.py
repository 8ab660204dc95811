"""tcgen05 split-precision (BF16 x3) contractions against FP64 products of
the same BF16 planes: the only difference allowed is FP32 accumulation
(tolerance 2e-5 relative to the largest entry)."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _planes(x, ld):
    """bf16 hi/lo planes (rows x ld) of a float32 matrix (rows x k)."""
    rows, k = x.shape
    hi = torch.zeros((rows, ld), dtype=torch.bfloat16, device=x.device)
    lo = torch.zeros((rows, ld), dtype=torch.bfloat16, device=x.device)
    h = x.to(torch.bfloat16)
    hi[:, :k] = h
    lo[:, :k] = (x - h.float()).to(torch.bfloat16)
    return hi, lo


def _split_product(ah, al, bh, bl, k):
    a_h, a_l = ah[:, :k].double(), al[:, :k].double()
    b_h, b_l = bh[:, :k].double(), bl[:, :k].double()
    return a_h @ b_h.T + a_h @ b_l.T + a_l @ b_h.T


# (2600, 256): 11 column tiles = a full and a ragged group of the tile order
@pytest.mark.parametrize("rows,k", [(200, 300), (600, 1000), (128, 64), (1000, 2048), (2600, 256)])
def test_gram_bf16x3(cuda, rows, k):
    import vmc_jax_gb300._lib as L
    torch.manual_seed(rows + k)
    ld = (k + 63) // 64 * 64
    x = torch.randn(rows, k, device=cuda)
    hi, lo = _planes(x, ld)
    ldg = (rows + 15) // 16 * 16
    G = torch.full((rows, ldg), float("nan"), dtype=torch.float32, device=cuda)
    L.call("vmc_gram_bf16x3", L.ptr(hi), L.ptr(lo), rows, k, ld, L.ptr(G), ldg, 3, None, L.stream())
    torch.cuda.synchronize()
    assert L.query("vmc_tc_error_flag", 1) == 0
    ref = _split_product(hi, lo, hi, lo, k)
    iu = torch.triu_indices(rows, rows, device=cuda)
    got = G[:, :rows].double()[iu[0], iu[1]]
    want = ref[iu[0], iu[1]]
    assert torch.isfinite(got).all()
    err = (got - want).abs().max() / want.abs().max()
    assert err < 2e-5, float(err)
    # split correction: much closer to the FP64 Gram than a plain BF16 product
    full = (x.double() @ x.double().T)[iu[0], iu[1]]
    assert (got - full).abs().max() / full.abs().max() < 1e-4


@pytest.mark.parametrize("m,n,k", [(300, 520, 200), (1024, 256, 512), (77, 1000, 130), (700, 2600, 192)])
def test_gemm_bf16x3_colsq(cuda, m, n, k):
    import vmc_jax_gb300._lib as L
    torch.manual_seed(m * n + k)
    ld = (k + 63) // 64 * 64
    a = torch.randn(m, k, device=cuda)
    b = torch.randn(n, k, device=cuda) / np.sqrt(k)
    ah, al = _planes(a, ld)
    bh, bl = _planes(b, ld)
    colsq = torch.full((n,), float("nan"), dtype=torch.float32, device=cuda)
    ws = torch.empty(L.query("vmc_gemm_bf16x3_colsq_workspace_bytes", m, n), dtype=torch.uint8, device=cuda)
    L.call("vmc_gemm_bf16x3_colsq", L.ptr(ah), L.ptr(al), m, ld, L.ptr(bh), L.ptr(bl), n, ld, k, L.ptr(colsq),
           L.ptr(ws), ws.numel(), 3, None, L.stream())
    first = colsq.clone()
    L.call("vmc_gemm_bf16x3_colsq", L.ptr(ah), L.ptr(al), m, ld, L.ptr(bh), L.ptr(bl), n, ld, k, L.ptr(colsq),
           L.ptr(ws), ws.numel(), 3, None, L.stream())
    torch.cuda.synchronize()
    assert torch.equal(first, colsq)  # fixed-order reduction: bitwise reproducible
    assert L.query("vmc_tc_error_flag", 1) == 0
    D = _split_product(ah, al, bh, bl, k)
    ref = (D ** 2).sum(0)
    err = (colsq.double() - ref).abs().max() / ref.abs().max()
    assert err < 2e-5, float(err)


@pytest.mark.parametrize("precision", ["mixed", "fp32"])
def test_tdvp_mixed_and_fp32_forms(cuda, precision):
    """The reduced-precision forms against the FP64 form on the same exact
    samples: energies identical to FP32 kernel accuracy, updates close."""
    import vmc_jax_gb300 as V
    from oracle import jvmc_oracle as O
    L_, M = 10, 20
    rng = np.random.default_rng(0)
    prm = {"bias": rng.normal(0, 0.1, M) + 1j * rng.normal(0, 0.1, M),
           "kernel": rng.normal(0, 0.1, (L_, M)) + 1j * rng.normal(0, 0.1, (L_, M))}
    opsi = O.NQS(O.CpxRBM(M, True), prm)
    res = {}
    for prec in ["fp64", precision]:
        psi = V.vqs.NQS(V.nets.CpxRBM(numHidden=M, bias=True), precision="fp64" if prec == "fp64" else "fp32")
        psi(np.zeros((1, 1, L_), np.int32))
        psi.set_parameters(opsi.get_parameters())
        H = V.operator.BranchFreeOperator()
        for l in range(L_):
            H.add(V.operator.scal_opstr(-1.0, (V.operator.Sz(l), V.operator.Sz((l + 1) % L_))))
            H.add(V.operator.scal_opstr(-0.7, (V.operator.Sx(l),)))
        es = V.sampler.ExactSampler(psi, L_)
        td = V.util.TDVP(es, makeReal="real", rhsPrefactor=1., pinvCutoff=1e-8, precision=prec)
        u = td(psi.get_parameters(), 0., psi=psi, hamiltonian=H, intStep=0)
        res[prec] = (u.cpu().numpy(), complex(td.ElocMean0), td.get_spectrum().cpu().numpy())
    u64, e64, s64 = res["fp64"]
    u, e, s = res[precision]
    assert abs(e - e64) / abs(e64) < 1e-6
    assert np.max(np.abs(s - s64)) / np.max(np.abs(s64)) < 1e-4
    assert np.max(np.abs(u - u64)) / np.max(np.abs(u64)) < 5e-2


def test_bounded_wait_runs_out_and_reports(cuda):
    """A wait on a barrier that nothing completes gives up after the limit
    and writes its code to the caller's status word; the context stays
    usable (a GEMM right after is exact), and a per-call status word leaves
    the library-wide flag untouched."""
    import vmc_jax_gb300._lib as L
    L.query("vmc_tc_error_flag", 1)
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    L.call("vmc_tc_wait_check", 20_000_000, L.ptr(status), L.stream())
    torch.cuda.synchronize()
    assert int(status.item()) == 6
    assert L.query("vmc_tc_error_flag", 0) == 0
    x = torch.randn(256, 128, device=cuda)
    hi, lo = _planes(x, 128)
    G = torch.full((256, 256), float("nan"), dtype=torch.float32, device=cuda)
    ok = torch.zeros(1, dtype=torch.int32, device=cuda)
    L.call("vmc_gram_bf16x3", L.ptr(hi), L.ptr(lo), 256, 128, 128, L.ptr(G), 256, 3, L.ptr(ok), L.stream())
    torch.cuda.synchronize()
    assert int(ok.item()) == 0
    ref = _split_product(hi, lo, hi, lo, 128)
    iu = torch.triu_indices(256, 256, device=cuda)
    assert torch.allclose(G.double()[iu[0], iu[1]], ref[iu[0], iu[1]], rtol=0, atol=2e-5 * ref.abs().max().item())


def test_gram_plain_bf16(cuda):
    """products = 1: the hi planes alone (plain BF16), lo planes not read
    (here filled with NaN to show it)."""
    import vmc_jax_gb300._lib as L
    torch.manual_seed(4)
    rows, k = 600, 1000
    ld = (k + 63) // 64 * 64
    x = torch.randn(rows, k, device=cuda)
    hi, lo = _planes(x, ld)
    lo.fill_(float("nan"))
    ldg = (rows + 15) // 16 * 16
    G = torch.full((rows, ldg), float("nan"), dtype=torch.float32, device=cuda)
    L.call("vmc_gram_bf16x3", L.ptr(hi), L.ptr(lo), rows, k, ld, L.ptr(G), ldg, 1, None, L.stream())
    torch.cuda.synchronize()
    ref = hi[:, :k].double() @ hi[:, :k].double().T
    iu = torch.triu_indices(rows, rows, device=cuda)
    got = G[:, :rows].double()[iu[0], iu[1]]
    assert torch.isfinite(got).all()
    assert ((got - ref[iu[0], iu[1]]).abs().max() / ref.abs().max()).item() < 2e-5
