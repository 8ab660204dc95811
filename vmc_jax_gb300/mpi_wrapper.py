"""Reductions over samples (mirror of jVMC/mpi_wrapper.py for one process).

jVMC sums over its (device, batch) dimensions and then over MPI processes
with ``Allreduce``.  Here a job is one process on one GPU: the sums stay on
the device (FP64) and no host round trip or collective is made.  The
sample-count bookkeeping (``distribute_sampling``, ``globNumSamples``) is
kept because the TDVP signal-to-noise ratio uses it.
"""

import time

import numpy as np
import torch

from . import _lib

rank = 0
commSize = 1

globNumSamples = 0
myNumSamples = 0
communicationTime = 0.


def distribute_sampling(numSamples, localDevices=None, numChainsPerDevice=1):
    """Samples per chain and the number of samples actually drawn, for one
    process (the contract of mpi_wrapper.py:53-95 at commSize 1).

    Without a chain count every requested sample is drawn: (numSamples,
    numSamples).  With C = localDevices * numChainsPerDevice chains each
    chain draws ceil(numSamples / C) samples, so C * ceil(numSamples / C)
    samples are drawn in total.  That total is stored in ``globNumSamples``,
    which the TDVP signal-to-noise ratio uses."""
    global globNumSamples
    if localDevices is None:
        globNumSamples = int(numSamples)
        return int(numSamples), globNumSamples
    chains = int(localDevices) * int(numChainsPerDevice)
    perChain = -(-int(numSamples) // chains)
    globNumSamples = perChain * chains
    return perChain, globNumSamples


def first_sample_id():
    """Index of this process's first sample in the global sample order
    (mpi_wrapper.py:98-111); a single process starts at 0."""
    return 0


def _as_tensor(data):
    if isinstance(data, torch.Tensor):
        return data
    return torch.as_tensor(np.asarray(data))


def global_sum(data):
    """Sum over the device and batch dimensions (mpi_wrapper.py:114-147);
    result has shape ``data.shape[2:]``."""
    d = _as_tensor(data)
    return d.sum(dim=(0, 1))


def global_mean(data, p):
    """sum_j p_j X_j over the sample dimension (mpi_wrapper.py:150-174)."""
    d = _as_tensor(data)
    p = _as_tensor(p).to(d.device)
    if d.is_cuda and d.dim() == 3 and d.shape[2] == 1:
        mean, _ = _mean_var_kernel(d[0, :, 0], p[0])
        return mean.reshape(1).to(d.dtype if d.is_complex() else mean.dtype)
    w = p[0].to(torch.float64)
    return torch.tensordot(w.to(d.dtype) if d.is_complex() else w, d[0], dims=([0], [0]))


def global_variance(data, p):
    """sum_j p_j |X_j - <X>|^2 (mpi_wrapper.py:177-217)."""
    d = _as_tensor(data)
    p = _as_tensor(p).to(d.device)
    if d.is_cuda and d.dim() == 3 and d.shape[2] == 1:
        _, var = _mean_var_kernel(d[0, :, 0], p[0])
        return var.reshape(1)
    mean = global_mean(d, p)
    x = d[0] - mean[None]
    return torch.einsum("ij,ij,i->j", torch.conj(x), x, p[0].to(x.dtype)) if x.is_complex() else \
        torch.einsum("ij,ij,i->j", x, x, p[0].to(x.dtype))


def _mean_var_kernel(x, w):
    """FP64 weighted mean and variance of one per-sample scalar on the GPU."""
    x = x.to(torch.complex128).contiguous()
    w = w.to(torch.float64).contiguous()
    mean = torch.empty(1, dtype=torch.complex128, device=x.device)
    var = torch.empty(1, dtype=torch.float64, device=x.device)
    nb = _lib.query("vmc_reduce_workspace_bytes", 2)
    ws = _lib.Workspace.get(nb, x.device)
    _lib.call("vmc_weighted_mean_var", _lib.ptr(x), _lib.ptr(w), x.numel(), _lib.ptr(mean), _lib.ptr(var),
              _lib.ptr(ws), ws.numel(), _lib.stream())
    return mean, var


def gather(data):
    """All samples of all processes, flattened (mpi_wrapper.py:278-292)."""
    d = _as_tensor(data)
    return d.reshape((-1,) + tuple(d.shape[2:]))


def bcast_unknown_size(data, root=0):
    """mpi_wrapper.py:246-275 (a single process keeps its data)."""
    if np.asarray(data).dtype != np.float64:
        raise TypeError("Datatype has to be float64.")
    return np.array(data)


def get_communication_time():
    global communicationTime
    t = communicationTime
    communicationTime = 0.
    return t
