"""Real CNN ansatz (mirror of jVMC/nets/cnn.py:18-83)."""

import numpy as np
import torch

from .. import _lib
from . import activation_functions as act_funs


class CNN:
    """Convolutional neural network with real parameters.

    Initialization arguments (cnn.py:21-39):
        * ``F``: Filter diameter
        * ``channels``: Number of channels
        * ``strides``: Number of pixels the filter shifts over (only 1)
        * ``actFun``: Non-linear activation function(s)
        * ``bias``: Whether to use biases
        * ``firstLayerBias``: Whether to use biases in the first layer
        * ``periodicBoundary``: Whether to use periodic boundary conditions (only True)
    """

    holomorphic = False
    realParams = True

    def __init__(self, F=(8,), channels=(10,), strides=(1,), actFun=(act_funs.poly6,), bias=True,
                 firstLayerBias=False, periodicBoundary=True):
        self.F = tuple(int(f) for f in F)
        self.channels = tuple(int(c) for c in channels)
        self.strides = tuple(int(s) for s in strides)
        if any(s != 1 for s in self.strides):
            raise NotImplementedError("CNN: only unit strides have CUDA kernels")
        if not periodicBoundary:
            raise NotImplementedError("CNN: only periodic boundaries have CUDA kernels")
        acts = list(actFun) if isinstance(actFun, (list, tuple)) else [actFun]
        while len(acts) < len(self.channels):
            acts.append(acts[-1])
        self.actFun = acts
        self.act_codes = [act_funs.kernel_code(a) for a in acts]
        self.bias = bool(bias)
        self.firstLayerBias = bool(firstLayerBias)
        self.periodicBoundary = True

    def layer_bias(self, l):
        return self.firstLayerBias if l == 0 else self.bias

    def leaf_shapes(self, sampleShape):
        shapes = []
        cin = 1
        for l, c in enumerate(self.channels):
            if self.layer_bias(l):
                shapes.append((f"Conv_{l}/bias", (c,)))
            shapes.append((f"Conv_{l}/kernel", self.F + (cin, c)))
            cin = c
        return shapes

    def init(self, seed, sampleShape, device):
        """variance_scaling(1, fan_avg, uniform) kernels, zero biases (cnn.py:42,63-64)."""
        self._shape = tuple(sampleShape)
        rng = np.random.default_rng(seed)
        params = {}
        for name, shape in self.leaf_shapes(sampleShape):
            if name.endswith("bias"):
                v = np.zeros(shape)
            else:
                rf = int(np.prod(shape[:-2]))
                fan_in, fan_out = shape[-2] * rf, shape[-1] * rf
                lim = np.sqrt(3.0 / ((fan_in + fan_out) / 2.0))
                v = rng.uniform(-lim, lim, shape)
            params[name] = torch.as_tensor(v, dtype=torch.float64, device=device)
        return params

    # ------------------------------------------------------------ kernels
    @staticmethod
    def _prec(precision):
        return _lib.VMC_F32 if precision == "fp32" else _lib.VMC_F64

    def desc(self, sampleShape):
        """vmc_cnn_desc of this network on a lattice of shape ``sampleShape``."""
        import ctypes
        sampleShape = tuple(sampleShape)
        if len(sampleShape) != len(self.F) or len(sampleShape) not in (1, 2):
            raise NotImplementedError("CNN kernels support 1-D and 2-D lattices with matching filters")
        if len(self.channels) > 4:
            raise NotImplementedError("CNN kernels support up to 4 layers")
        d = _CnnDesc()
        d.ndim = len(sampleShape)
        d.dims = (ctypes.c_int32 * 2)(*(list(sampleShape) + [1])[:2])
        d.filter = (ctypes.c_int32 * 2)(*(list(self.F) + [1])[:2])
        d.num_layers = len(self.channels)
        d.channels = (ctypes.c_int32 * 4)(*(list(self.channels) + [0] * 4)[:4])
        d.activation = (ctypes.c_int32 * 4)(*(self.act_codes + [0] * 4)[:4])
        d.has_bias = (ctypes.c_int32 * 4)(*([int(self.layer_bias(l)) for l in range(len(self.channels))] + [0] * 4)[:4])
        return d

    def flat(self, params, precision):
        dt = torch.float32 if precision == "fp32" else torch.float64
        return torch.cat([p.reshape(-1) for p in params.values()]).to(dt).contiguous()

    def logpsi(self, params, configs, precision="fp64", sampleShape=None):
        N = configs.shape[0]
        shape = sampleShape if sampleShape is not None else self._shape
        out = torch.empty(N, dtype=torch.complex128, device=configs.device)
        d = self.desc(shape)
        theta = self.flat(params, precision)  # kept alive until the launch is enqueued
        _lib.call("vmc_cnn_logpsi", self._prec(precision), _lib.ctypes_ref(d), _lib.ptr(configs), N,
                  _lib.ptr(theta), _lib.ptr(out), _lib.stream())
        return out

    def gradients(self, params, configs, precision="fp64", layout=_lib.VMC_GRAD_REFERENCE, sampleShape=None):
        N = configs.shape[0]
        shape = sampleShape if sampleShape is not None else self._shape
        d = self.desc(shape)
        P = sum(p.numel() for p in params.values())
        if layout == _lib.VMC_GRAD_REFERENCE:
            out = torch.empty((N, P), dtype=torch.complex128, device=configs.device)
        else:
            out = torch.empty((N, P), dtype=torch.float64, device=configs.device)
        theta = self.flat(params, precision)
        _lib.call("vmc_cnn_gradients", self._prec(precision), _lib.ctypes_ref(d), _lib.ptr(configs), N,
                  _lib.ptr(theta), layout, _lib.ptr(out), _lib.stream())
        return out


import ctypes as _ct


class _CnnDesc(_ct.Structure):
    _fields_ = [("ndim", _ct.c_int32), ("dims", _ct.c_int32 * 2), ("filter", _ct.c_int32 * 2),
                ("num_layers", _ct.c_int32), ("channels", _ct.c_int32 * 4), ("activation", _ct.c_int32 * 4),
                ("has_bias", _ct.c_int32 * 4)]
