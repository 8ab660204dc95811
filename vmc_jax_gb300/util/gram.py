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
