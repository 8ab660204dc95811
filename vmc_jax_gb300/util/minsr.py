"""MinSR solver (mirror of jVMC/util/minsr.py:16-165).

update = -O^dagger (O O^dagger)^+ E_loc with the N_s x N_s tangent kernel
(stats.py:332-336) instead of the P x P matrix S: the cheaper solve when
N_s < P.  For a CpxRBM the centred, weighted log-derivatives come from the
CUDA producer (compact P layout); the kernel O O^dagger is the tcgen05
BF16x3 Gram kernel on the real representation of the samples (precision
"mixed") or one cuBLAS GEMM (FP64 / FP32); the pseudo-inverse is an FP64
eigendecomposition on the GPU applied as V (inv * (V^dagger e)) (two
matrix-vector products, no N_s^3 product).  The holomorphic update is
returned in the reference's complex 2P form [-w, i w] per leaf
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
    eigenvalues with |l| <= rtol max|l| are dropped.  Returned factored as
    (V, inv): T^+ = V diag(inv) V^dagger."""
    from .gram import eigh_fp64
    ev, V = eigh_fp64(T)
    cut = rtol * torch.max(torch.abs(ev))
    inv = torch.where(torch.abs(ev) > cut, 1.0 / ev, torch.zeros_like(ev))
    return V, inv


def pinv_apply(factors, x):
    """T^+ x = V (inv * (V^dagger x)) from the factors of pinv_hermitian."""
    V, inv = factors
    x = x.to(V.dtype)
    return V @ (inv.to(V.dtype) * (V.mH @ x))


def tangent_kernel_fp64(X):
    """X X^dagger (N x N) of complex128 samples X (N x P, row-major): the
    FP64-accurate Hermitian tensor-core product (vmc_zgemm_ozaki) for
    N >= 1024 and P within its reduction limit, cuBLAS ZGEMM below."""
    from . import gram as _gram
    N, P = X.shape
    if N < _gram.OZAKI_MIN_DIM or P > _gram.OZAKI_MAX_K:
        return X @ X.mH
    # row-major X is M = X^T column-major (ld P); M^H M = conj(X X^dagger),
    # whose column-major storage read row-major is X X^dagger
    return _gram.fp64_product("C", X, P, "N", X, P, N, N, P, hermitian=True)


def tangent_kernel_mixed(X):
    """X X^dagger (N x N complex128) of complex samples X (N x P) on the
    tcgen05 Gram kernel: rows [Re X; Im X] as BF16 hi/lo planes, FP32
    accumulation, assembled in FP64 (the Gram assembly forms sum conj(x_a) x_b
    over the rows x_a of X, the conjugate of X X^dagger, conjugated back)."""
    from .gram import _round_up
    N, P = X.shape
    dev = X.device
    ld = _round_up(P, 64)
    R = 2 * N
    hi = torch.zeros((R, ld), dtype=torch.bfloat16, device=dev)
    lo = torch.zeros((R, ld), dtype=torch.bfloat16, device=dev)
    for half, part in ((0, X.real), (1, X.imag)):
        x = part.to(torch.float32)
        h = x.to(torch.bfloat16)
        hi[half * N:(half + 1) * N, :P] = h
        lo[half * N:(half + 1) * N, :P] = (x - h.to(torch.float32)).to(torch.bfloat16)
    ldg = _round_up(R, 16)
    G = torch.empty((R, ldg), dtype=torch.float32, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    st = _lib.stream()
    _lib.call("vmc_gram_bf16x3", _lib.ptr(hi), _lib.ptr(lo), R, P, ld, _lib.ptr(G), ldg, 3, _lib.ptr(status), st)
    del hi, lo
    A = torch.empty((N, N), dtype=torch.complex128, device=dev)
    _lib.call("vmc_gram_to_hermitian", _lib.VMC_F32, _lib.ptr(G), ldg, N, 0.0, _lib.ptr(A), st)
    if int(status.item()):
        raise _lib.VmcError("MinSR: the tangent-kernel Gram kernel gave up waiting (code %d)" % int(status.item()))
    return torch.conj_physical(A)


class MinSR:
    """Energy minimisation via MinSR (arXiv:2302.01941), minsr.py:16-165.

    Initializer arguments: ``sampler``, ``pinvTol``, ``diagonalShift``,
    ``diagonalizeOnDevice`` (must be True), ``precision`` ("fp64", "fp32" or
    "mixed": arithmetic of the log-derivative kernels and of the
    tangent-kernel product -- cuBLAS FP64 / FP32, or the BF16x3 tcgen05 Gram
    kernel; the pseudo-inverse is FP64 in every case)."""

    def __init__(self, sampler, pinvTol=1e-14, diagonalShift=0., diagonalizeOnDevice=True, precision="fp64"):
        if precision not in ("fp64", "fp32", "mixed"):
            raise ValueError("precision must be 'fp64', 'fp32' or 'mixed'")
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
            v = pinv_apply(pinv_hermitian(T, self.pinvTol), e)
            return -(G.conj().T @ v.to(G.dtype))
        G = torch.cat([G.real, G.imag], dim=0).to(torch.float64)
        T = G @ G.T + self.diagonalShift * torch.eye(G.shape[0], dtype=G.dtype, device=G.device)
        ee = torch.cat([e.real, e.imag]).to(torch.float64)
        return -(G.T @ pinv_apply(pinv_hermitian(T, self.pinvTol), ee))

    def _rbm_update(self, psi, configs, Eloc, p):
        """The holomorphic MinSR update for a CpxRBM from the CUDA kernels."""
        dev = configs.device
        st = _lib.stream()
        flat = configs.reshape(configs.shape[0] * configs.shape[1], -1)
        N, L = flat.shape
        w = p.reshape(-1).to(torch.float64).contiguous()
        E = Eloc.reshape(-1).to(torch.complex128).contiguous()
        kp = "fp64" if self.precision == "fp64" else "fp32"  # "mixed": FP32 kernels
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
        if self.precision == "mixed":
            T = 2.0 * tangent_kernel_mixed(X)
        else:
            T = 2.0 * (tangent_kernel_fp64(X) if self.precision == "fp64" else (X @ X.mH).to(torch.complex128))
        e = torch.sqrt(w).to(torch.complex128) * (E - emean[0])
        v = pinv_apply(pinv_hermitian(T, self.pinvTol), e)
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
