"""MinSR solver (mirror of jVMC/util/minsr.py:16-165).

update = -O^dagger (O O^dagger)^+ E_loc with the N_s x N_s tangent kernel
(stats.py:332-336) instead of the P x P matrix S: the cheaper solve when
N_s < P.  For a CpxRBM the centred, weighted log-derivatives come from the
CUDA producer (compact P layout), the kernel O O^dagger is one GEMM and the
pseudo-inverse an FP64 eigendecomposition on the GPU; the holomorphic update
is returned in the reference's complex 2P form [-w, i w] per leaf
(w = g^dagger T^+ e), which the integrators add to the real parameter vector
exactly as jVMC does.
"""

import numpy as np
import torch

from .. import _lib
from ..nets.rbm import CpxRBM
from ..stats import SampledObs


def pinv_hermitian(T, rtol):
    """jnp.linalg.pinv(T, rtol, hermitian=True) (minsr.py:63,74) by eigh:
    eigenvalues with |l| <= rtol max|l| are dropped."""
    ev, V = torch.linalg.eigh(T)
    cut = rtol * torch.max(torch.abs(ev))
    inv = torch.where(torch.abs(ev) > cut, 1.0 / ev, torch.zeros_like(ev))
    return (V * inv.to(V.dtype)) @ V.mH


class MinSR:
    """Energy minimisation via MinSR (arXiv:2302.01941), minsr.py:16-165.

    Initializer arguments: ``sampler``, ``pinvTol``, ``diagonalShift``,
    ``diagonalizeOnDevice`` (must be True), ``precision`` ("fp64" or "fp32":
    arithmetic of the tangent-kernel GEMM; the pseudo-inverse is FP64)."""

    def __init__(self, sampler, pinvTol=1e-14, diagonalShift=0., diagonalizeOnDevice=True, precision="fp64"):
        if not diagonalizeOnDevice:
            raise NotImplementedError("diagonalisation runs on the GPU; there is no host path")
        self.sampler = sampler
        self.pinvTol = pinvTol
        self.diagonalShift = diagonalShift
        self.diagonalizeOnDevice = True
        self.precision = precision
        self.metaData = None

    def set_pinv_tol(self, tol):
        self.pinvTol = tol

    def get_metadata(self):
        return self.metaData

    def get_energy_variance(self):
        return self.ElocVar0

    def get_energy_mean(self):
        return torch.real(torch.as_tensor(self.ElocMean0))

    def solve(self, eloc, gradients, holomorphic):
        """minsr.py:53-80 on SampledObs inputs."""
        G = gradients._data.reshape((-1,) + tuple(gradients._data.shape[2:]))
        e = eloc._data.reshape(-1)
        if holomorphic:
            T = gradients.tangent_kernel()
            T_inv = pinv_hermitian(T, self.pinvTol)
            return -(G.conj().T @ (T_inv @ e.to(T_inv.dtype)))
        G = torch.cat([G.real, G.imag], dim=0).to(torch.float64)
        T = G @ G.T + self.diagonalShift * torch.eye(G.shape[0], dtype=G.dtype, device=G.device)
        T_inv = pinv_hermitian(T, self.pinvTol)
        ee = torch.cat([e.real, e.imag]).to(torch.float64)
        return -(G.T @ (T_inv @ ee))

    def _rbm_update(self, psi, configs, Eloc, p):
        """The holomorphic MinSR update for a CpxRBM from the CUDA kernels."""
        dev = configs.device
        st = _lib.stream()
        flat = configs.reshape(configs.shape[0] * configs.shape[1], -1)
        N, L = flat.shape
        w = p.reshape(-1).to(torch.float64).contiguous()
        E = Eloc.reshape(-1).to(torch.complex128).contiguous()
        kp = "fp64" if self.precision == "fp64" else "fp32"
        params = psi.params_for(kp)
        prec = CpxRBM._prec(kp)
        M = int(params["kernel"].shape[1])
        P = L * M + (M if "bias" in params else 0)
        Wk, bk = _lib.ptr(params["kernel"]), _lib.ptr(params.get("bias"))
        emean = torch.empty(1, dtype=torch.complex128, device=dev)
        evar = torch.empty(1, dtype=torch.float64, device=dev)
        ws = _lib.Workspace.get(_lib.query("vmc_reduce_workspace_bytes", 2))
        _lib.call("vmc_weighted_mean_var", _lib.ptr(E), _lib.ptr(w), N, _lib.ptr(emean), _lib.ptr(evar),
                  _lib.ptr(ws), ws.numel(), st)
        okMean = torch.empty(P, dtype=torch.complex128, device=dev)
        cov = torch.empty(P, dtype=torch.complex128, device=dev)
        ws = _lib.Workspace.get(_lib.query("vmc_rbm_grad_stats_workspace_bytes", N, L, M))
        _lib.call("vmc_rbm_grad_stats", prec, _lib.ptr(flat), N, L, M, Wk, bk, _lib.ptr(w), _lib.ptr(E),
                  _lib.ptr(emean), _lib.ptr(okMean), _lib.ptr(cov), _lib.ptr(ws), ws.numel(), st)
        fmt, dt = (0, torch.complex128) if self.precision == "fp64" else (1, torch.complex64)
        X = torch.empty((N, P), dtype=dt, device=dev)
        _lib.call("vmc_rbm_centered_gradients", prec, _lib.ptr(flat), N, L, M, Wk, bk, _lib.ptr(w),
                  _lib.ptr(okMean), fmt, _lib.ptr(X), None, P, st)
        # reference 2P data [g, i g] per leaf: its tangent kernel is 2 g g^dagger
        T = (2.0 * (X @ X.mH)).to(torch.complex128)
        T_inv = pinv_hermitian(T, self.pinvTol)
        e = torch.sqrt(w).to(torch.complex128) * (E - emean[0])
        v = T_inv @ e
        wv = X.to(torch.complex128).mH @ v     # g^dagger T^+ e  (P)
        parts, start = [], 0
        for name, prm in psi.params.items():
            n = prm.numel()
            parts += [-wv[start:start + n], 1.j * wv[start:start + n]]
            start += n
        self.ElocMean, self.ElocVar = emean[0], evar[0]
        return torch.cat(parts)

    def __call__(self, netParameters, t, *, psi, hamiltonian, **rhsArgs):
        """theta_dot from MinSR (minsr.py:82-165)."""
        tmp = psi.get_parameters()
        psi.set_parameters(netParameters)
        configs, logPsi, p = self.sampler.sample(numSamples=rhsArgs.get("numSamples", None))
        if isinstance(psi.net, CpxRBM) and hasattr(hamiltonian, "fused_capable") and hamiltonian.fused_capable(psi):
            Eloc = hamiltonian.get_O_loc_fused(configs, psi, None, t)
            update = self._rbm_update(psi, configs, Eloc, p)
            mean, var = self.ElocMean, self.ElocVar
        else:
            Eloc = SampledObs(hamiltonian.get_O_loc(configs, psi, logPsi, t), p)
            grads = SampledObs(psi.gradients(configs), p)
            update = self.solve(Eloc, grads, holomorphic=psi.holomorphic)
            mean, var = Eloc.mean()[0], Eloc.var()[0]
        psi.set_parameters(tmp)
        if rhsArgs.get("intStep", None) == 0:
            self.ElocMean0 = mean
            self.ElocVar0 = var
            self.metaData = {}
        return update
