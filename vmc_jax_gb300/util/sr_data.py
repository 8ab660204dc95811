"""Producers of the per-sample data that the complex S/F build and the SNR
transform contract (stats.py:50-58, 197-205, 255-292 via tdvp.py:134-181).

Two sources, one interface:

* ``RbmData``: a CpxRBM, from the configurations (tanh(theta) recomputed in
  the producing kernel; O is never stored).
* ``DenseData``: any holomorphic network whose log-derivatives O (N, P)
  complex128 are materialised by its gradient kernel (e.g. SymNet).

Each producer writes X = sqrt(w)(O - <O>) and H = sqrt(w)((-x) dE conj(O -
<O>) - f) in the storage formats of ``vmc_data_format`` and forms <O> and
covar(O, E) with fixed-order reductions.
"""

import torch

from .. import _lib


class RbmData:
    def __init__(self, psi, flat, precision):
        params = psi.params_for(precision)
        self.flat = flat
        self.prec = psi.net._prec(precision)
        self.N, self.L = flat.shape
        self.M = int(params["kernel"].shape[1])
        self.P = self.L * self.M + (self.M if "bias" in params else 0)
        self.Wk, self.bk = _lib.ptr(params["kernel"]), _lib.ptr(params.get("bias"))
        self._keep = params
        self.device = flat.device

    def stats(self, w, E, emean, okMean, covOE):
        ws = _lib.Workspace.get(_lib.query("vmc_rbm_grad_stats_workspace_bytes", self.N, self.L, self.M))
        _lib.call("vmc_rbm_grad_stats", self.prec, _lib.ptr(self.flat), self.N, self.L, self.M, self.Wk, self.bk,
                  _lib.ptr(w), _lib.ptr(E), _lib.ptr(emean), _lib.ptr(okMean), _lib.ptr(covOE), _lib.ptr(ws),
                  ws.numel(), _lib.stream())

    def centered(self, w, okMean, fmt, out, out_lo, ld):
        _lib.call("vmc_rbm_centered_gradients", self.prec, _lib.ptr(self.flat), self.N, self.L, self.M, self.Wk,
                  self.bk, _lib.ptr(w), _lib.ptr(okMean), fmt, _lib.ptr(out), _lib.ptr(out_lo), ld, _lib.stream())

    def snr_data(self, w, okMean, E, emean, negx, f, fmt, out, out_lo, ld):
        _lib.call("vmc_rbm_snr_data", self.prec, _lib.ptr(self.flat), self.N, self.L, self.M, self.Wk, self.bk,
                  _lib.ptr(w), _lib.ptr(okMean), _lib.ptr(E), _lib.ptr(emean), negx.real, negx.imag, _lib.ptr(f),
                  fmt, _lib.ptr(out), _lib.ptr(out_lo), ld, _lib.stream())


class DenseData:
    """``real=True``: a real-parameter net (O real, stored as complex128 with
    imaginary part 0; S and F are the real parts, makeReal = Re)."""

    def __init__(self, psi, flat, precision, real=False):
        params = psi.params_for(precision)
        layout = _lib.VMC_GRAD_REFERENCE if real else _lib.VMC_GRAD_COMPACT
        self.O = psi.net.gradients(params, flat, precision, layout)
        self.N, self.P = self.O.shape
        self.device = flat.device
        self.real = real

    def stats(self, w, E, emean, okMean, covOE):
        ws = _lib.Workspace.get(_lib.query("vmc_dense_grad_stats_workspace_bytes", self.N, self.P))
        _lib.call("vmc_dense_grad_stats", _lib.ptr(self.O), self.P, self.N, self.P, _lib.ptr(w), _lib.ptr(E),
                  _lib.ptr(emean), _lib.ptr(okMean), _lib.ptr(covOE), _lib.ptr(ws), ws.numel(), _lib.stream())

    def centered(self, w, okMean, fmt, out, out_lo, ld):
        _lib.call("vmc_dense_centered_gradients", _lib.ptr(self.O), self.P, self.N, self.P, _lib.ptr(w),
                  _lib.ptr(okMean), fmt, _lib.ptr(out), _lib.ptr(out_lo), ld, _lib.stream())

    def snr_data(self, w, okMean, E, emean, negx, f, fmt, out, out_lo, ld):
        _lib.call("vmc_dense_snr_data", _lib.ptr(self.O), self.P, self.N, self.P, _lib.ptr(w), _lib.ptr(okMean),
                  _lib.ptr(E), _lib.ptr(emean), negx.real, negx.imag, _lib.ptr(f), int(self.real), fmt,
                  _lib.ptr(out), _lib.ptr(out_lo), ld, _lib.stream())


def producer(psi, flat, precision):
    """The data producer for the network of ``psi`` (None: no complex path)."""
    from ..nets.cnn import CNN
    from ..nets.rbm import CpxRBM
    from ..nets.sym_wrapper import SymNet
    if isinstance(psi.net, CpxRBM):
        return RbmData(psi, flat, precision)
    if isinstance(psi.net, SymNet):
        return DenseData(psi, flat, precision)
    if isinstance(psi.net, CNN):
        return DenseData(psi, flat, precision, real=True)
    return None
