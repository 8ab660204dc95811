"""Variational quantum state (mirror of jVMC/vqs.py:85-492).

Parameters live on the GPU as torch tensors in jVMC's leaf order; the flat
parameter vector has jVMC's layout ``[Re(leaf); Im(leaf)]`` per leaf for
complex nets (vqs.py:449-466) and is float64.  Network evaluation and
gradients run in the CUDA kernels of the network's ``nets`` module.
"""

import numpy as np
import torch

from . import _lib
from . import global_defs


def as_configs(s, device=None):
    """Configurations as a contiguous int32 CUDA tensor of shape (1, N, *sampleShape)."""
    if not isinstance(s, torch.Tensor):
        s = torch.as_tensor(np.asarray(s))
    device = global_defs.device() if device is None else device
    if s.device != device or s.dtype != torch.int32:
        s = s.to(device=device, dtype=torch.int32)
    return s.contiguous()


class NQS:
    """Wrapper class providing basic functionality of variational states.

    Initializer arguments (vqs.py:115-182):
        * ``net``: network (``nets.CpxRBM``, ``nets.CNN`` or
          ``nets.SymNet`` of a CpxRBM).
        * ``logarithmic``: the net returns log psi (only True is supported).
        * ``batchSize``: kept for interface compatibility; the CUDA kernels
          evaluate any number of configurations in one launch.
        * ``seed``: seed of the parameter initialisation.
        * ``orbit``: ``util.symmetries.LatticeSymmetry``; wraps ``net`` in a
          ``SymNet`` (vqs.py:167-168).
        * ``avgFun``: the SymNet's average (default
          ``avgFun_Coefficients_Exp``).
        * ``precision``: arithmetic of the network kernels, ``"fp64"``
          (default, the reference's FP64) or ``"fp32"``.
    """

    def __init__(self, net, logarithmic=True, batchSize=1000, seed=1234, orbit=None, avgFun=None,
                 precision="fp64"):
        if isinstance(net, (list, tuple)):
            raise NotImplementedError("two-network ansatz (TwoNets) has no CUDA path")
        if orbit is not None:
            from .nets.sym_wrapper import SymNet, avgFun_Coefficients_Exp
            net = SymNet(orbit=orbit, net=net, avgFun=avgFun_Coefficients_Exp if avgFun is None else avgFun)
        if not logarithmic:
            raise NotImplementedError("only logarithmic networks are supported")
        _lib.require_cuda()
        self.net = net
        self.logarithmic = True
        self.batchSize = batchSize
        self.seed = seed
        self.initialized = False
        self.parameters = None
        self.holomorphic = False
        self.realParams = getattr(net, "realParams", False)
        self.precision = precision
        self._version = 0
        self._cache = {}

    # -------------------------------------------------------------- setup
    def init_net(self, s):
        """Initialise parameters from an example input (vqs.py:187-218)."""
        if self.initialized:
            return
        sampleShape = tuple(s.shape[2:])
        self.sampleShape = sampleShape
        self.parameters = {"params": self.net.init(self.seed, sampleShape, global_defs.device())}
        self.holomorphic = bool(self.net.holomorphic)
        self.realParams = bool(self.net.realParams)
        leaves = self.parameters["params"]
        self.paramShapes = [(int(p.numel()), tuple(p.shape)) for p in leaves.values()]
        self.numParameters = int(sum(p.numel() for p in leaves.values()))
        self.initialized = True

    @property
    def params(self):
        if self.initialized:
            return self.parameters["params"]
        return None

    @params.setter
    def params(self, val):
        self.parameters["params"] = dict(val)
        self._touch()

    def _touch(self):
        self._version += 1
        self._cache.clear()

    def params_for(self, precision=None):
        """Parameters in the dtype of the requested kernel precision."""
        precision = self.precision if precision is None else precision
        if precision == "fp64":
            return self.params
        key = ("params", precision)
        if key not in self._cache:
            dt = torch.float32 if self.realParams else torch.complex64
            self._cache[key] = {k: v.to(dt).contiguous() for k, v in self.params.items()}
        return self._cache[key]

    def rbm_tables(self, precision=None):
        precision = self.precision if precision is None else precision
        key = ("tables", precision)
        if key not in self._cache:
            self._cache[key] = self.net.tables(self.params_for(precision), precision)
        return self._cache[key]

    # ---------------------------------------------------------- evaluation
    def __call__(self, s):
        """log psi(s) for configurations s of shape (1, N, *sampleShape)
        (vqs.py:223-251); returns (1, N) complex128 (float64 promoted to
        complex128 for real nets, as the reference's NQS output dtype)."""
        s = as_configs(s)
        self.init_net(s)
        flat = s.reshape(s.shape[0] * s.shape[1], -1)
        out = self.net.logpsi(self.params_for(), flat, self.precision)
        return out.reshape(s.shape[:2])

    def gradients(self, s):
        """d log psi / d theta per configuration (vqs.py:256-287): (1, N, 2P)
        ``[g, i g]`` per leaf for holomorphic nets, (1, N, P) for real
        parameters."""
        s = as_configs(s)
        self.init_net(s)
        flat = s.reshape(s.shape[0] * s.shape[1], -1)
        g = self.net.gradients(self.params_for(), flat, self.precision, _lib.VMC_GRAD_REFERENCE)
        return g.reshape(s.shape[:2] + (g.shape[-1],))

    def gradients_dict(self, s):
        """Gradients as a dict of leaves (vqs.py:292-314)."""
        g = self.gradients(s)
        out = {}
        start = 0
        for name, p in self.params.items():
            n = p.numel()
            w = 2 * n if self.holomorphic else n
            out[name] = g[..., start:start + w]
            start += w
        return out

    def get_sampler_net(self):
        """A function of (params, configs) returning Re log psi, and the
        current parameters (vqs.py:337-352)."""
        def evalReal(params, x):
            x = as_configs(x)
            flat = x.reshape(-1, int(np.prod(self.sampleShape)))
            return torch.real(self.net.logpsi(params, flat, "fp64")).reshape(x.shape[:-len(self.sampleShape)])
        return evalReal, self.params

    # ---------------------------------------------------------- parameters
    def get_parameters(self):
        """Flat float64 parameter vector (vqs.py:449-466)."""
        if not self.initialized:
            return None
        if self.realParams:
            return torch.cat([p.reshape(-1) for p in self.params.values()]).to(torch.float64)
        return torch.cat([torch.cat([p.reshape(-1).real, p.reshape(-1).imag]) for p in self.params.values()])

    def _param_unflatten(self, P):
        """vqs.py:430-444."""
        if not isinstance(P, torch.Tensor):
            P = torch.as_tensor(np.asarray(P))
        cplx = P.is_complex()
        P = P.to(device=global_defs.device(), dtype=torch.complex128 if cplx else torch.float64)
        out = {}
        start = 0
        for (name, p), (n, shape) in zip(self.params.items(), self.paramShapes):
            if not self.realParams:
                if cplx:  # P[a] + 1j * P[b] in complex arithmetic, as vqs.py:437
                    out[name] = (P[start:start + n] + 1.j * P[start + n:start + 2 * n]).reshape(shape)
                else:
                    out[name] = torch.complex(P[start:start + n], P[start + n:start + 2 * n]).reshape(shape)
                start += 2 * n
            else:
                out[name] = P[start:start + n].reshape(shape).clone()
                start += n
        return out

    def set_parameters(self, P):
        """vqs.py:409-425."""
        if not self.initialized:
            raise RuntimeError("Error in NQS.set_parameters(): Network not initialized. "
                               "Evaluate net on example input for initialization.")
        if isinstance(P, dict):
            self.params = {k: torch.as_tensor(v).to(global_defs.device()) for k, v in P.items()}
        else:
            self.params = self._param_unflatten(P)

    def update_parameters(self, deltaP):
        """vqs.py:384-404."""
        if not self.initialized:
            self.set_parameters(deltaP)
        d = self._param_unflatten(deltaP)
        self.params = {k: self.params[k] + d[k] for k in self.params}

    @property
    def is_generator(self):
        return False

    def sample(self, numSamples, key, parameters=None):
        return None
