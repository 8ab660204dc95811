"""Mixed-precision (BF16 x3 split, FP32 accumulation, tcgen05) S build and
SNR contraction of the TDVP step for a holomorphic network."""

import torch

from .. import _lib
from .timing import TIMER

BF16X2 = 2


def _round_up(x, m):
    return (x + m - 1) // m * m


def mixed_hermitian(data, w, okMean, shift, status=None, products=3):
    """A = <O^dagger O>_c (P x P complex128) from the BF16x3 Gram matrix of the
    real representation of the centred data of ``data`` (a util.sr_data
    producer).  ``status``: device int32 word that a timed-out wait of the
    tensor-core kernel sets (the caller zeroes and checks it).  ``products``:
    3 (hi.hi + hi.lo + lo.hi) or 1 (hi.hi: plain BF16)."""
    dev = data.device
    st = _lib.stream()
    N, P = data.N, data.P
    ld = _round_up(N, 64)
    R = 2 * P
    hi = torch.empty((R, ld), dtype=torch.bfloat16, device=dev)
    lo = torch.empty((R, ld), dtype=torch.bfloat16, device=dev)
    data.centered(w, okMean, BF16X2, hi, lo, ld)
    ldg = _round_up(R, 16)
    G = torch.empty((R, ldg), dtype=torch.float32, device=dev)
    TIMER.mark("gram_kernel")
    _lib.call("vmc_gram_bf16x3", _lib.ptr(hi), _lib.ptr(lo), R, N, ld, _lib.ptr(G), ldg, products, _lib.ptr(status), st)
    TIMER.mark("hermitian")
    del hi, lo
    A = torch.empty((P, P), dtype=torch.complex128, device=dev)
    _lib.call("vmc_gram_to_hermitian", _lib.VMC_F32, _lib.ptr(G), ldg, P, float(shift), _lib.ptr(A), st)
    return A


def mixed_snr_colsq(data, w, okMean, E, emean, f, U, x, status=None, products=3):
    """Column sums of |H conj(U)|^2 in the real representation (2P floats);
    ``status`` as for ``mixed_hermitian``."""
    dev = data.device
    st = _lib.stream()
    N, P = data.N, data.P
    R = 2 * P
    ld = _round_up(R, 64)
    hh = torch.empty((N, ld), dtype=torch.bfloat16, device=dev)
    hl = torch.empty((N, ld), dtype=torch.bfloat16, device=dev)
    data.snr_data(w, okMean, E, emean, -complex(x), f, BF16X2, hh, hl, ld)
    bh = torch.empty((R, ld), dtype=torch.bfloat16, device=dev)
    bl = torch.empty((R, ld), dtype=torch.bfloat16, device=dev)
    _lib.call("vmc_eigvec_bf16x2", _lib.ptr(U), U.stride(1), P, _lib.ptr(bh), _lib.ptr(bl), ld, st)
    colsq = torch.empty(R, dtype=torch.float32, device=dev)
    ws = _lib.Workspace.get(_lib.query("vmc_gemm_bf16x3_colsq_workspace_bytes", N, R))
    TIMER.mark("snr_kernel")
    _lib.call("vmc_gemm_bf16x3_colsq", _lib.ptr(hh), _lib.ptr(hl), N, ld, _lib.ptr(bh), _lib.ptr(bl), R, ld, R,
              _lib.ptr(colsq), _lib.ptr(ws), ws.numel(), products, _lib.ptr(status), st)
    TIMER.mark("snr_tail")
    return colsq


OZAKI_MIN_DIM = 1024   # below this the FP64 product goes through cuBLAS
OZAKI_MAX_K = 30720    # longest complex reduction of vmc_zgemm_ozaki (int64 tile sums below 2^63)


def fp64_product(trans_a, A, lda, trans_b, B, ldb, m, n, k, hermitian=False, status=None):
    """C = op(A) op(B) as the FP64-accurate tensor-core product
    (vmc_zgemm_ozaki: 8 slices, levels <= 7, entries within ~2^-48 of the
    row and column scales).  A, B: complex128 device storage read with the
    given leading dimensions; returns the column-major m x n result as an
    (n, m) tensor (its .T is C)."""
    dev = A.device
    nb = _lib.query("vmc_zgemm_ozaki_workspace_bytes", m, n, k, 8)
    ws = _lib.Workspace.get(nb + 256)
    base = ws.data_ptr() + (256 - ws.data_ptr() % 256) % 256
    C = torch.empty((n, m), dtype=torch.complex128, device=dev)
    _lib.call("vmc_zgemm_ozaki", ord(trans_a), ord(trans_b), m, n, k, _lib.ptr(A), lda, _lib.ptr(B), ldb,
              _lib.ptr(C), m, 1 if hermitian else 0, 0, 8, 7, base, nb, _lib.ptr(status), _lib.stream())
    return C


def eigh_fp64(A):
    """FP64 eigendecomposition of the Hermitian (or real symmetric) A (a
    row-major torch tensor) by cuSOLVER through the C ABI (vmc_eigh_fp64):
    (ev ascending, U column-major with U[:, j] the eigenvectors), as
    torch.linalg.eigh(A) returns them."""
    n = A.shape[0]
    cplx = A.is_complex()
    dev = A.device
    # the C ABI reads column-major: the row-major storage of conj(A) (= A^T) is A
    V = (torch.conj_physical(A) if cplx else A.T).contiguous()
    ev = torch.empty(n, dtype=torch.float64, device=dev)
    info = torch.zeros(1, dtype=torch.int32, device=dev)
    ws = _lib.Workspace.get(_lib.query("vmc_eigh_fp64_workspace_bytes", n, 1 if cplx else 0))
    _lib.call("vmc_eigh_fp64", n, 1 if cplx else 0, _lib.ptr(V), n, _lib.ptr(ev), _lib.ptr(V), n, _lib.ptr(ws),
              ws.numel(), _lib.ptr(info), _lib.stream())
    if int(info.item()) != 0:
        raise _lib.VmcError("FP64 eigensolver did not converge (info %d)" % int(info.item()))
    return ev, V.mT   # V's storage is column-major: the tensor's transpose is the eigenvector matrix
