"""Real CNN ansatz (mirror of jVMC/nets/cnn.py:18-83)."""

import numpy as np
import torch

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
