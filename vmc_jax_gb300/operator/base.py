"""Operator interface (mirror of jVMC/operator/base.py:20-317)."""

import abc

import torch

from .. import _lib
from ..vqs import as_configs


class Operator(metaclass=abc.ABCMeta):
    """Interface to compute operator matrix elements and local estimators.

    Sub-classes implement ``compile()``.  The CUDA path supports
    ``BranchFreeOperator``; other operators raise ``NotImplementedError``
    (there is no CPU fallback).
    """

    def __init__(self, ElocBatchSize=-1):
        self.compiled = False
        self.compiled_argnum = -1
        self.ElocBatchSize = ElocBatchSize

    def get_s_primes(self, s, *args):
        raise NotImplementedError("get_s_primes has a CUDA path for BranchFreeOperator only")

    def fused_capable(self, psi):
        return False

    def get_O_loc(self, samples, psi, logPsiS=None, *args):
        """O_loc(s) = sum_s' O_{s,s'} psi(s')/psi(s) (base.py:166-192)."""
        if self.fused_capable(psi):
            if self.ElocBatchSize > 0:
                return self.get_O_loc_batched(samples, psi, logPsiS, self.ElocBatchSize, *args)
            return self.get_O_loc_fused(samples, psi, logPsiS, *args)
        if logPsiS is None:
            logPsiS = psi(samples)
        if self.ElocBatchSize > 0:
            return self.get_O_loc_batched(samples, psi, logPsiS, self.ElocBatchSize, *args)
        sampleOffdConfigs, _ = self.get_s_primes(samples, *args)
        logPsiSP = psi(sampleOffdConfigs)
        return self.get_O_loc_unbatched(logPsiS, logPsiSP)

    def get_O_loc_unbatched(self, logPsiS, logPsiSP):
        """sum_k matEl_k exp(logPsiSP_k - logPsiS) with the matrix elements of
        the last ``get_s_primes`` call (base.py:162-164, 194-212)."""
        m = self.matEl
        dev = m.device
        lps = torch.as_tensor(logPsiS).to(device=dev, dtype=torch.complex128).reshape(-1).contiguous()
        lpsp = torch.as_tensor(logPsiSP).to(device=dev, dtype=torch.complex128).reshape(-1).contiguous()
        N = m.shape[0] * m.shape[1]
        K = m.shape[2]
        out = torch.empty(N, dtype=torch.complex128, device=dev)
        mc = m.reshape(N, K).contiguous()
        _lib.call("vmc_oloc_from_sprimes", _lib.ptr(mc), _lib.ptr(lps), _lib.ptr(lpsp), N, K, _lib.ptr(out),
                  _lib.stream())
        return out.reshape(m.shape[:2])

    def get_O_loc_batched(self, samples, psi, logPsiS, batchSize, *args):
        """O_loc in batches of configurations (base.py:214-278); results do
        not depend on the batch size."""
        s = as_configs(samples)
        numSamples = s.shape[1]
        if logPsiS is None and not self.fused_capable(psi):
            logPsiS = psi(s)
        out = []
        for b0 in range(0, numSamples, batchSize):
            sb = s[:, b0:b0 + batchSize]
            lb = None if logPsiS is None else torch.as_tensor(logPsiS)[:, b0:b0 + batchSize]
            if self.fused_capable(psi):
                out.append(self.get_O_loc_fused(sb, psi, lb, *args))
            else:
                sp, _ = self.get_s_primes(sb, *args)
                out.append(self.get_O_loc_unbatched(lb, psi(sp)))
        return torch.cat(out, dim=1)

    @abc.abstractmethod
    def compile(self):
        """Return the operator's matrix-element function (base.py:280-285)."""

    def get_estimator_function(self, psi, *args):
        raise NotImplementedError("estimator functions of (theta, s) are JAX closures; the CUDA path "
                                  "evaluates O_loc with get_O_loc")
