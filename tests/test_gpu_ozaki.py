"""FP64-accurate complex products on the BF16 tensor cores (Ozaki split,
vmc_zgemm_ozaki) against cuBLAS ZGEMM in FP64.

Bars: with 8 slices and levels <= 7 every entry is within 2^-48 of
||op(A) row|| ||B column|| (the products' own scale; the three lowest
levels are rounded to 2^-lsb of the row and column scales once per K range,
and an FP64 DGEMM's own bound, K 2^-53 of the same scale, is above 2^-48
for K >= 32); integer inputs whose products fit in 53 bits come out
exact."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _ozaki(L, trans, A, B, m, n, k, herm=False, slices=8, level=7, C=None, acc=False, trans_b="N"):
    dev = A.device
    nb = L.query("vmc_zgemm_ozaki_workspace_bytes", m, n, k, slices)
    ws = torch.empty(nb + 256, dtype=torch.uint8, device=dev)
    base = (256 - ws.data_ptr() % 256) % 256
    if C is None:
        C = torch.full((n, m), complex(float("nan"), 0.0), dtype=torch.complex128, device=dev)  # column-major m x n
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    L.call("vmc_zgemm_ozaki", ord(trans), ord(trans_b), m, n, k, L.ptr(A), A.shape[1], L.ptr(B), B.shape[1], L.ptr(C), m,
           1 if herm else 0, 1 if acc else 0, slices, level, ws.data_ptr() + base, nb, L.ptr(status), L.stream())
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    return C.T  # row-major view of the m x n result


def _colmajor(x):
    """Column-major storage of x (rows x cols) as a (cols, rows) tensor (a
    lazily conjugated view is materialised first)."""
    return x.resolve_conj().T.contiguous()


@pytest.mark.parametrize("m,n,k", [(130, 70, 50), (257, 300, 129), (512, 384, 1000), (64, 200, 2047)])
@pytest.mark.parametrize("trans", ["C", "N"])
def test_product_matches_fp64(cuda, m, n, k, trans):
    import vmc_jax_gb300._lib as L
    g = torch.Generator(device=cuda).manual_seed(m + n + k)
    opA = torch.randn(m, k, dtype=torch.complex128, device=cuda, generator=g)
    opA[:, :3] *= 1e3   # uneven magnitudes inside a row
    Bm = torch.randn(k, n, dtype=torch.complex128, device=cuda, generator=g)
    A = opA.conj().T if trans == "C" else opA          # stored matrix (k x m or m x k)
    got = _ozaki(L, trans, _colmajor(A), _colmajor(Bm), m, n, k)
    want = opA @ Bm
    scale = opA.abs().square().sum(1).sqrt()[:, None] * Bm.abs().square().sum(0).sqrt()[None, :]
    err = ((got - want).abs() / scale).max().item()
    assert err < 2.0 ** -48, err


def test_adjoint_b_operand(cuda):
    """trans_b 'C': op(B) = B^H with B stored n x k (the layout of a
    row-major samples x parameters matrix read as its transpose)."""
    import vmc_jax_gb300._lib as L
    g = torch.Generator(device=cuda).manual_seed(11)
    m, n, k = 300, 260, 900
    Mt = torch.randn(m, k, dtype=torch.complex128, device=cuda, generator=g)
    Bs = torch.randn(n, k, dtype=torch.complex128, device=cuda, generator=g)   # stored B (n x k)
    got = _ozaki(L, "N", _colmajor(Mt), _colmajor(Bs), m, n, k, trans_b="C")
    want = Mt @ Bs.conj().T
    scale = Mt.abs().square().sum(1).sqrt()[:, None] * Bs.abs().square().sum(1).sqrt()[None, :]
    assert ((got - want).abs() / scale).max().item() < 2.0 ** -48


def test_hermitian_and_accumulate(cuda):
    import vmc_jax_gb300._lib as L
    g = torch.Generator(device=cuda).manual_seed(3)
    k, m = 700, 300
    X = torch.randn(k, m, dtype=torch.complex128, device=cuda, generator=g)
    got = _ozaki(L, "C", _colmajor(X), _colmajor(X), m, m, k, herm=True)
    want = X.conj().T @ X
    err = ((got - want).abs().max() / want.abs().max()).item()
    asym = (got - got.conj().T).abs().max().item()
    assert err < 2.0 ** -48 and asym == 0.0, (err, asym)
    C0 = torch.randn(m, m, dtype=torch.complex128, device=cuda, generator=g)
    Cc = _colmajor(C0)
    got2 = _ozaki(L, "C", _colmajor(X), _colmajor(X), m, m, k, herm=True, C=Cc, acc=True)
    assert ((got2 - (want + C0)).abs().max() / want.abs().max()).item() < 2.0 ** -48


def test_integer_products_are_exact(cuda):
    """Entries with at most 20 significant bits: every product and sum is an
    integer below 2^53, so the split product must equal the exact one (this
    also checks that the tensor core sums each level's group exactly)."""
    import vmc_jax_gb300._lib as L
    g = torch.Generator(device=cuda).manual_seed(7)
    m, n, k = 200, 180, 1500
    re = torch.randint(-2 ** 19, 2 ** 19, (k, m), device=cuda, generator=g).double()
    im = torch.randint(-2 ** 19, 2 ** 19, (k, m), device=cuda, generator=g).double()
    A = torch.complex(re, im)
    re = torch.randint(-2 ** 10, 2 ** 10, (k, n), device=cuda, generator=g).double()
    im = torch.randint(-2 ** 10, 2 ** 10, (k, n), device=cuda, generator=g).double()
    B = torch.complex(re, im)
    got = _ozaki(L, "C", _colmajor(A), _colmajor(B), m, n, k)
    want = A.conj().T @ B   # |entries| < 2^(19+10+1+11) = 2^41: exact in FP64
    assert torch.equal(got, want)


def test_fewer_levels_bound(cuda):
    """maxLevel 4 (5 levels): entries within 2^-28 of the row / column scales."""
    import vmc_jax_gb300._lib as L
    g = torch.Generator(device=cuda).manual_seed(9)
    m = n = 256
    k = 512
    A = torch.randn(k, m, dtype=torch.complex128, device=cuda, generator=g)
    B = torch.randn(k, n, dtype=torch.complex128, device=cuda, generator=g)
    got = _ozaki(L, "C", _colmajor(A), _colmajor(B), m, n, k, slices=5, level=4)
    want = A.conj().T @ B
    scale = A.abs().square().sum(0).sqrt()[:, None] * B.abs().square().sum(0).sqrt()[None, :]
    err = ((got - want).abs() / scale).max().item()
    assert err < 2.0 ** -28, err


def test_minsr_fp64_tangent_kernel(cuda):
    """The FP64 MinSR tangent kernel X X^dagger (N = 1280 samples, P = 700)
    from the Hermitian Ozaki product: exactly Hermitian, entries within 2^-47
    of the row / column scales of cuBLAS ZGEMM's X X^dagger (the split
    product's 2^-48 plus the reference's own rounding, ~sqrt(P) u = 3e-15 of
    the scales on the diagonal, where every term is positive; measured
    3.9e-15)."""
    from vmc_jax_gb300.util.minsr import tangent_kernel_fp64
    g = torch.Generator(device=cuda).manual_seed(11)
    X = torch.randn(1280, 700, dtype=torch.complex128, device=cuda, generator=g)
    T = tangent_kernel_fp64(X)
    want = X @ X.mH
    nrm = X.abs().square().sum(1).sqrt()
    err = ((T - want).abs() / (nrm[:, None] * nrm[None, :])).max().item()
    assert err < 2.0 ** -47, err
    assert torch.equal(T, T.mH.resolve_conj())
