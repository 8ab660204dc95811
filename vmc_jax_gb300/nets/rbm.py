"""Complex RBM ansatz (mirror of jVMC/nets/rbm.py:17-38) dispatched to the
CUDA kernels of csrc/rbm.cu."""

import numpy as np
import torch

from .. import _lib


class CpxRBM:
    """Restricted Boltzmann machine with complex parameters,

        log psi(s) = sum_j log cosh( sum_i W_ij (2 s_i - 1) + b_j ).

    Initialization arguments:
        * ``numHidden``: Number of hidden units.
        * ``bias``: ``Boolean`` indicating whether to use bias.

    Parameter leaves in jVMC's flatten order: ``bias`` (M,) if present, then
    ``kernel`` (L, M).  Defaults follow the reference initialisers
    (initializers.py:17-20: kernel U[0,0.01) + i U[0,0.01); bias 0).
    """

    holomorphic = True
    realParams = False

    def __init__(self, numHidden=2, bias=False):
        self.numHidden = int(numHidden)
        self.bias = bool(bias)

    def leaf_shapes(self, sampleShape):
        L = int(np.prod(sampleShape))
        shapes = []
        if self.bias:
            shapes.append(("bias", (self.numHidden,)))
        shapes.append(("kernel", (L, self.numHidden)))
        return shapes

    def init(self, seed, sampleShape, device):
        rng = np.random.default_rng(seed)
        params = {}
        for name, shape in self.leaf_shapes(sampleShape):
            if name == "bias":
                v = np.zeros(shape, dtype=np.complex128)
            else:
                v = rng.uniform(0, 0.01, shape) + 1.j * rng.uniform(0, 0.01, shape)
            params[name] = torch.as_tensor(v, dtype=torch.complex128, device=device)
        return params

    # ------------------------------------------------------------ kernels
    @staticmethod
    def _prec(precision):
        return _lib.VMC_F32 if precision == "fp32" else _lib.VMC_F64

    def dims(self, params):
        L, M = params["kernel"].shape
        return int(L), int(M)

    def logpsi(self, params, configs, precision="fp64"):
        """log psi of configs (N, L) int32 -> (N,) complex128."""
        L, M = self.dims(params)
        N = configs.shape[0]
        out = torch.empty(N, dtype=torch.complex128, device=configs.device)
        _lib.call("vmc_rbm_logpsi", self._prec(precision), _lib.ptr(configs), N, L, M,
                  _lib.ptr(params["kernel"]), _lib.ptr(params.get("bias")), _lib.ptr(out), _lib.stream())
        return out

    def gradients(self, params, configs, precision="fp64", layout=_lib.VMC_GRAD_REFERENCE):
        L, M = self.dims(params)
        N = configs.shape[0]
        P = L * M + (M if "bias" in params else 0)
        width = 2 * P if layout == _lib.VMC_GRAD_REFERENCE else P
        out = torch.empty((N, width), dtype=torch.complex128, device=configs.device)
        _lib.call("vmc_rbm_gradients", self._prec(precision), _lib.ptr(configs), N, L, M,
                  _lib.ptr(params["kernel"]), _lib.ptr(params.get("bias")), layout, _lib.ptr(out),
                  _lib.stream())
        return out

    def tables(self, params, precision="fp64"):
        L, M = self.dims(params)
        nbytes = _lib.query("vmc_rbm_tables_bytes", self._prec(precision), L, M)
        dt = torch.complex64 if precision == "fp32" else torch.complex128
        tab = torch.empty(nbytes // (8 if precision == "fp32" else 16), dtype=dt, device=params["kernel"].device)
        _lib.call("vmc_rbm_prepare", self._prec(precision), L, M, _lib.ptr(params["kernel"]), _lib.ptr(tab),
                  _lib.stream())
        return tab
