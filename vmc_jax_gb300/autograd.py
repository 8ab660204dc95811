"""Differentiable log psi: the hand-written O_k backward kernels behind a
``torch.autograd.Function``.

``log_psi(psi, theta, configs)`` returns (N, 2) float64 = [Re log psi, Im
log psi] as a function of jVMC's flat real parameter vector theta
(vqs.py:449-466 layout).  Its backward is the vector-Jacobian product:

* CpxRBM: one kernel (``vmc_rbm_vjp``) forms v_k = sum_n conj(g_n) O_nk
  without materialising O (tanh(theta) recomputed from the configurations),
  and d theta = [Re v; -Im v] per leaf, since d log psi / d Re theta_k = O_k
  and d log psi / d Im theta_k = i O_k for a holomorphic net.
* SymNet(CpxRBM): O (holomorphic, weighted over the orbit) in chunks of
  at most ``chunk_bytes``, v = conj(g) O, d theta as for the CpxRBM.
* CNN (real parameters): the backward kernel recomputes every activation of
  each configuration in shared memory; O is formed in chunks of at most
  ``chunk_bytes`` so that N_s x N_p never has to fit in HBM at once.
"""

import torch

from . import _lib
from .nets.cnn import CNN
from .nets.rbm import CpxRBM
from .nets.sym_wrapper import SymNet


def _flat_configs(psi, configs):
    from .vqs import as_configs
    s = as_configs(configs)
    return s.reshape(s.shape[0] * s.shape[1], -1)


class _LogPsi(torch.autograd.Function):

    @staticmethod
    def forward(ctx, theta, configs, psi, chunk_bytes):
        saved = psi.get_parameters()
        psi.set_parameters(theta.detach())
        flat = _flat_configs(psi, configs)
        lp = psi.net.logpsi(psi.params_for(), flat, psi.precision)
        params = {k: v.clone() for k, v in psi.params_for().items()}
        psi.set_parameters(saved)
        ctx.psi, ctx.flat, ctx.params, ctx.chunk_bytes = psi, flat, params, chunk_bytes
        return torch.stack([lp.real, lp.imag], dim=1)

    @staticmethod
    def backward(ctx, grad_out):
        psi, flat, params = ctx.psi, ctx.flat, ctx.params
        g = torch.complex(grad_out[:, 0].contiguous().to(torch.float64),
                          grad_out[:, 1].contiguous().to(torch.float64)).contiguous()
        N, L = flat.shape
        if isinstance(psi.net, CpxRBM):
            M = int(params["kernel"].shape[1])
            P = L * M + (M if "bias" in params else 0)
            v = torch.empty(P, dtype=torch.complex128, device=flat.device)
            ws = _lib.Workspace.get(_lib.query("vmc_rbm_vjp_workspace_bytes", N, L, M))
            _lib.call("vmc_rbm_vjp", psi.net._prec(psi.precision), _lib.ptr(flat), N, L, M,
                      _lib.ptr(params["kernel"]), _lib.ptr(params.get("bias")), _lib.ptr(g), _lib.ptr(v),
                      _lib.ptr(ws), ws.numel(), _lib.stream())
            parts, start = [], 0
            for name, p in params.items():
                n = p.numel()
                parts += [v[start:start + n].real, -v[start:start + n].imag]
                start += n
            return torch.cat(parts), None, None, None
        if isinstance(psi.net, SymNet):
            P = sum(p.numel() for p in params.values())
            rows = max(1, int(ctx.chunk_bytes // (16 * P)))
            v = torch.zeros(P, dtype=torch.complex128, device=flat.device)
            for n0 in range(0, N, rows):
                O = psi.net.gradients(params, flat[n0:n0 + rows].contiguous(), psi.precision,
                                      _lib.VMC_GRAD_COMPACT)
                v += torch.conj(g[n0:n0 + rows]) @ O
            parts, start = [], 0
            for name, p in params.items():
                n = p.numel()
                parts += [v[start:start + n].real, -v[start:start + n].imag]
                start += n
            return torch.cat(parts), None, None, None
        if isinstance(psi.net, CNN):
            P = sum(p.numel() for p in params.values())
            rows = max(1, int(ctx.chunk_bytes // (8 * P)))
            out = torch.zeros(P, dtype=torch.float64, device=flat.device)
            for n0 in range(0, N, rows):
                O = psi.net.gradients(params, flat[n0:n0 + rows].contiguous(), psi.precision,
                                      _lib.VMC_GRAD_COMPACT)
                out += g[n0:n0 + rows].real @ O
            return out, None, None, None
        raise NotImplementedError(type(psi.net).__name__)


def log_psi(psi, theta, configs, chunk_bytes=1 << 30):
    """Differentiable [Re log psi, Im log psi] (N, 2) of ``psi`` at flat
    parameters ``theta`` (requires_grad) for ``configs`` (1, N, ...)."""
    return _LogPsi.apply(theta, configs, psi, chunk_bytes)
