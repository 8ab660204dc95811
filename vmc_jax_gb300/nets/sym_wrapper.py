"""Symmetrised network (mirror of jVMC/nets/sym_wrapper.py:22-64).

``SymNet(orbit, net)`` evaluates a CpxRBM on every element tau of a lattice
symmetry orbit and averages,

    log psi(s) = avgFun_tau(log psi_net(tau(s)), factor),

in one kernel per call (csrc/sym_rbm.cu): the per-element networks are never
materialised as separate configurations.
"""

import ctypes

import numpy as np
import torch

from .. import _lib
from .rbm import CpxRBM


def avgFun_Coefficients_Exp(coeffs, sym_factor):
    """log sum_tau factor_tau exp(coeffs_tau) (sym_wrapper.py:7-9), in the
    form of jax's logsumexp with ``b = factor``.  Host form, for reference
    and tests; the kernels implement the same reduction."""
    c = torch.as_tensor(coeffs)
    b = torch.as_tensor(np.asarray(sym_factor), device=c.device).to(torch.complex128).reshape(
        (-1,) + (1,) * (c.dim() - 1))
    a = torch.where(b != 0, c.to(torch.complex128), torch.full_like(c, float("-inf"), dtype=torch.complex128))
    amax = torch.max(a.real, dim=0).values
    amax = torch.where(torch.isfinite(amax), amax, torch.zeros_like(amax))
    return torch.log(torch.sum(torch.exp(a - amax) * b, dim=0)) + amax


def avgFun_Coefficients_Log(coeffs, sym_factor):
    """Mean of the log-coefficients (sym_wrapper.py:12-13; factor unused)."""
    return torch.mean(torch.as_tensor(coeffs), dim=0)


def avgFun_Coefficients_Sep(coeffs, sym_factor):
    """Separate averages of modulus and phase (sym_wrapper.py:16-19); not
    holomorphic, so it has no CUDA path."""
    raise NotImplementedError("avgFun_Coefficients_Sep (non-holomorphic average) has no CUDA path")


class SymDesc(ctypes.Structure):
    """Mirror of ``vmc_sym_desc``."""
    _fields_ = [
        ("num_sym", ctypes.c_int32),
        ("average", ctypes.c_int32),
        ("orbit", ctypes.c_void_p),
        ("inverse", ctypes.c_void_p),
        ("factor", ctypes.c_void_p),
    ]


_AVG = {avgFun_Coefficients_Exp: 0, avgFun_Coefficients_Log: 1}


class SymNet:
    """Wrapper module for symmetrisation (sym_wrapper.py:22-64).

    Initialization arguments:
        * ``orbit``: ``util.symmetries.LatticeSymmetry``.
        * ``net``: the plain ansatz (``CpxRBM``).
        * ``avgFun``: ``avgFun_Coefficients_Exp`` (default) or
          ``avgFun_Coefficients_Log``.

    The parameters are those of ``net`` (same leaves and flat layout).
    """

    def __init__(self, orbit, net, avgFun=avgFun_Coefficients_Exp):
        from ..util.symmetries import orbit_codes
        if not isinstance(net, CpxRBM):
            raise NotImplementedError("SymNet has CUDA kernels for a CpxRBM")
        if avgFun not in _AVG:
            raise NotImplementedError("SymNet averages with a CUDA path: avgFun_Coefficients_Exp, "
                                      "avgFun_Coefficients_Log")
        self.orbit = orbit
        self.net = net
        self.avgFun = avgFun
        self.average = _AVG[avgFun]
        self.codes, self.inverse = orbit_codes(orbit)
        self.factor = np.asarray(orbit.factor, dtype=np.complex128).reshape(-1)
        self.numSym = int(self.codes.shape[0])
        self._dev = {}

    holomorphic = True
    realParams = False

    @property
    def numHidden(self):
        return self.net.numHidden

    @property
    def bias(self):
        return self.net.bias

    def leaf_shapes(self, sampleShape):
        return self.net.leaf_shapes(sampleShape)

    def init(self, seed, sampleShape, device):
        if int(np.prod(sampleShape)) != self.codes.shape[1]:
            raise ValueError("orbit acts on %d sites, configurations have %d" %
                             (self.codes.shape[1], int(np.prod(sampleShape))))
        return self.net.init(seed, sampleShape, device)

    _prec = staticmethod(CpxRBM._prec)

    def dims(self, params):
        return self.net.dims(params)

    def tables(self, params, precision="fp64"):
        return self.net.tables(params, precision)

    def desc(self, device):
        """Descriptor with the orbit tables on ``device`` (cached)."""
        key = str(device)
        if key not in self._dev:
            codes = torch.as_tensor(self.codes, device=device).contiguous()
            inv = torch.as_tensor(self.inverse, device=device).contiguous()
            fac = torch.as_tensor(self.factor, device=device).contiguous()
            d = SymDesc(self.numSym, self.average, codes.data_ptr(), inv.data_ptr(), fac.data_ptr())
            self._dev[key] = (d, codes, inv, fac)
        return self._dev[key][0]

    def logpsi(self, params, configs, precision="fp64"):
        L, M = self.dims(params)
        N = configs.shape[0]
        out = torch.empty(N, dtype=torch.complex128, device=configs.device)
        _lib.call("vmc_sym_rbm_logpsi", self._prec(precision), _lib.ptr(configs), N, L, M,
                  _lib.ptr(params["kernel"]), _lib.ptr(params.get("bias")),
                  _lib.ctypes_ref(self.desc(configs.device)), _lib.ptr(out), _lib.stream())
        return out

    def gradients(self, params, configs, precision="fp64", layout=_lib.VMC_GRAD_REFERENCE):
        L, M = self.dims(params)
        N = configs.shape[0]
        P = L * M + (M if "bias" in params else 0)
        width = 2 * P if layout == _lib.VMC_GRAD_REFERENCE else P
        out = torch.empty((N, width), dtype=torch.complex128, device=configs.device)
        _lib.call("vmc_sym_rbm_gradients", self._prec(precision), _lib.ptr(configs), N, L, M,
                  _lib.ptr(params["kernel"]), _lib.ptr(params.get("bias")),
                  _lib.ctypes_ref(self.desc(configs.device)), layout, _lib.ptr(out), _lib.stream())
        return out
