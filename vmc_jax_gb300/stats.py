"""Sample statistics (mirror of jVMC/stats.py:136-336) on GPU arrays.

``SampledObs`` keeps jVMC's semantics for user code and the generic TDVP
path: ``mean = sum_n w_n O_n``, data ``sqrt(w_n)(O_n - mean)``, covariances
``sum_n conj(d1_n) d2_n``.  The per-step TDVP of a CpxRBM does not go
through this class: its statistics come from the fused FP64 kernels
(csrc/rbm.cu, csrc/stats.cu).
"""

import numpy as np
import torch

from . import global_defs


def _t(x):
    if isinstance(x, torch.Tensor):
        return x
    return torch.as_tensor(np.asarray(x), device=global_defs.device())


def _w(weights, nd):
    """weights (1, N) reshaped to broadcast against data (1, N, ...)."""
    return weights.reshape(weights.shape + (1,) * (nd - 2))


class SampledObs:
    """Statistics of Monte Carlo or exact samples.

    Initializer arguments:
        * ``observations``: (device, batch, ...) array of per-sample values.
        * ``weights``: (device, batch) weights w_n.
    """

    def __init__(self, observations=None, weights=None, estimator=None, params=None):
        if estimator is not None:
            raise NotImplementedError("estimator functions are JAX closures without a CUDA path")
        self._weights = None if weights is None else _t(weights).to(torch.float64)
        self._data = None
        self._mean = None
        if observations is not None and weights is not None:
            self._compute_data_and_mean(_t(observations))

    def _compute_data_and_mean(self, obs):
        """stats.py:197-205."""
        if obs.dim() == 2:
            obs = obs[..., None]
        w = self._weights.to(obs.device)
        wd = w.to(obs.dtype) if (obs.is_complex() or obs.is_floating_point()) else w
        if not (obs.is_complex() or obs.is_floating_point()):
            obs = obs.to(torch.float64)
            wd = w
        self._mean = torch.tensordot(wd[0], obs[0], dims=([0], [0]))
        self._data = torch.sqrt(_w(w, obs.dim())).to(obs.dtype) * (obs - self._mean[None, None])

    def mean(self):
        return self._mean

    def covar(self, other=None):
        """sum_n conj(d1_n)^T d2_n (stats.py:235-245)."""
        if other is None:
            other = self
        a, b = self._data[0], other._data[0]
        dt = torch.promote_types(a.dtype, b.dtype)
        return torch.tensordot(torch.conj(a.to(dt)), b.to(dt), dims=([0], [0]))

    def var(self):
        """sum_n |d_n|^2 (stats.py:248-252)."""
        return (torch.abs(self._data) ** 2).sum(dim=(0, 1))

    def covar_data(self, other=None):
        """Per-sample conj(d1_n) (x) d2_n / w_n as a new SampledObs (stats.py:255-265)."""
        if other is None:
            other = self
        a, b = torch.conj(self._data[0]), other._data[0]
        dt = torch.promote_types(a.dtype, b.dtype)
        d = a.to(dt)[:, :, None] * b.to(dt)[:, None, :] / self._weights[0][:, None, None].to(dt)
        return SampledObs(d[None], self._weights)

    def covar_var(self, other=None):
        """stats.py:268-279."""
        if other is None:
            other = self
        a, b = torch.conj(self._data[0]), other._data[0]
        dt = torch.promote_types(a.dtype, b.dtype)
        v = (torch.abs(a.to(dt)[:, :, None] * b.to(dt)[:, None, :]) ** 2
             / self._weights[0][:, None, None]).sum(0)
        return v - torch.abs(self.covar(other)) ** 2

    def transform(self, nonLinearFun=lambda x: x, linearFun=None):
        """SampledObs of f(O_n), optionally followed by v @ f(O_n) (stats.py:282-292)."""
        d = self._data[0]
        x = d / torch.sqrt(_w(self._weights, d.dim() + 1)[0]).to(d.dtype) + self._mean[None]
        x = nonLinearFun(x)
        if linearFun is not None:
            v = _t(linearFun).to(x.device)
            dt = torch.promote_types(v.dtype, x.dtype)
            x = torch.matmul(v.to(dt), x.to(dt))
        return SampledObs(x[None], self._weights)

    def select(self, ixs):
        """stats.py:295-307."""
        new = SampledObs()
        new._data = self._data[:, :, ixs]
        new._mean = self._mean[ixs]
        new._weights = self._weights
        return new

    def subset(self, start=None, end=None, step=None):
        """stats.py:310-329."""
        new = SampledObs()
        w = self._weights[:, start:end:step]
        nrm = w.sum()
        d = self._data[:, start:end:step] / torch.sqrt(nrm)
        w = w / nrm
        new._weights = w
        new._mean = torch.tensordot(torch.sqrt(w[0]).to(d.dtype), d[0], dims=([0], [0])) + self._mean
        new._data = d + torch.sqrt(_w(w, d.dim())).to(d.dtype) * (self._mean - new._mean)[None, None]
        return new

    def tangent_kernel(self):
        """stats.py:332-336."""
        d = self._data.reshape((-1,) + tuple(self._data.shape[2:]))
        return torch.matmul(d, torch.conj(d.T))
