"""Samplers (mirror of jVMC/sampler.py).

``MCSampler`` runs the Metropolis chains of a CpxRBM in one CUDA kernel
(one warp per chain, incremental hidden-unit fields, Philox4x32-10 random
numbers; one block per chain for a symmetrised RBM; for a CNN, one warp per
chain that recomputes only the activations a flip can change, from the
stored activations of every layer) and keeps the chains on the GPU between
calls.  ``ExactSampler``
enumerates the basis and forms the Born weights on the GPU.
"""

import math

import numpy as np
import torch

from . import _lib
from . import global_defs
from . import mpi_wrapper as mpi
from .vqs import as_configs


def propose_spin_flip(key, s, info):
    """Flip one randomly chosen site (sampler.py:15-19).

    The CUDA sampler recognises this proposer and runs it inside the
    Metropolis kernel; called directly (host side) ``key`` is a
    ``numpy.random.Generator``."""
    s = np.array(s, copy=True)
    idx = int(key.integers(0, s.size))
    flat = s.reshape(-1)
    flat[idx] = (flat[idx] + 1) % 2
    return s


def _seed_from_key(key):
    if isinstance(key, (int, np.integer)):
        return int(key) & 0xFFFFFFFFFFFFFFFF
    a = np.asarray(key).astype(np.uint64).reshape(-1)
    v = 0
    for x in a:
        v = ((v << 32) ^ int(x)) & 0xFFFFFFFFFFFFFFFF
    return v


class MCSampler:
    """Metropolis sampler of p_mu(s) = |psi(s)|^mu / sum |psi|^mu
    (sampler.py:67-382).

    Initializer arguments as in the reference: ``net`` (an NQS),
    ``sampleShape``, ``key`` (an int seed or an array of uint32 words),
    ``updateProposer`` (``propose_spin_flip``), ``numChains``,
    ``updateProposerArg``, ``numSamples``, ``thermalizationSweeps``,
    ``sweepSteps``, ``initState``, ``mu``, ``logProbFactor``.
    """

    def __init__(self, net, sampleShape, key, updateProposer=None, numChains=1, updateProposerArg=None,
                 numSamples=100, thermalizationSweeps=10, sweepSteps=10, initState=None, mu=2, logProbFactor=0.5):
        from .nets.rbm import CpxRBM
        if updateProposer is None:
            raise RuntimeError("Instantiation of MCSampler: `updateProposer` is `None` and cannot be used for "
                               "MCMC sampling.")
        if updateProposer is not propose_spin_flip:
            raise NotImplementedError("the CUDA Metropolis kernel implements propose_spin_flip")
        if mu < 0 or mu > 2:
            raise ValueError("mu must be in the range [0, 2]")
        if isinstance(sampleShape, int):
            sampleShape = (sampleShape,)
        self.sampleShape = tuple(sampleShape)
        self.net = net
        self.L = int(np.prod(self.sampleShape))
        if initState is None:
            initState = np.zeros(self.sampleShape, dtype=np.int32)
        init = torch.as_tensor(np.asarray(initState), dtype=torch.int32, device=global_defs.device())
        self.states = init.reshape(1, 1, -1).repeat(1, numChains, 1).contiguous()
        # make sure that net is initialised (sampler.py:124)
        self.net(self.states.reshape((1, numChains) + self.sampleShape))
        from .nets.cnn import CNN
        from .nets.sym_wrapper import SymNet
        if not isinstance(self.net.net, (CpxRBM, CNN, SymNet)):
            raise NotImplementedError("MCSampler has CUDA kernels for CpxRBM, SymNet(CpxRBM) and CNN states")
        self.logProbFactor = logProbFactor
        self.mu = mu
        self.updateProposer = updateProposer
        self.updateProposerArg = updateProposerArg
        self.seed = _seed_from_key(key)
        self.thermalizationSweeps = thermalizationSweeps
        self.sweepSteps = sweepSteps
        self.numSamples = numSamples
        self.numChains = numChains
        self.callIndex = 0
        self.counters = torch.zeros(2, dtype=torch.int64, device=global_defs.device())
        self.globNumSamples = 0

    def set_number_of_samples(self, N):
        self.numSamples = N

    def set_random_key(self, key):
        self.seed = _seed_from_key(key)
        self.callIndex = 0

    def get_last_number_of_samples(self):
        return self.globNumSamples

    def sample(self, parameters=None, numSamples=None, multipleOf=1):
        """Configurations, log psi and weights of the samples
        (sampler.py:195-235)."""
        if numSamples is None:
            numSamples = self.numSamples
        psi = self.net
        tmp = None
        if parameters is not None:
            tmp = psi.params
            psi.set_parameters(parameters)
        perChain, self.globNumSamples = mpi.distribute_sampling(
            numSamples, localDevices=1, numChainsPerDevice=int(np.lcm(self.numChains, multipleOf)))
        configs = self._run_chains(psi, perChain)
        logPsi = psi(configs)
        if tmp is not None:
            psi.params = tmp
        n = configs.shape[1]
        p = torch.empty(n, dtype=torch.float64, device=configs.device)
        nb = _lib.query("vmc_reduce_workspace_bytes", 1)
        ws = _lib.Workspace.get(nb)
        lp = logPsi.reshape(-1).contiguous()
        _lib.call("vmc_mc_probabilities", _lib.ptr(lp), n, float(1.0 / self.logProbFactor - self.mu), _lib.ptr(p),
                  _lib.ptr(ws), ws.numel(), _lib.stream())
        return configs, logPsi, p.reshape(1, n)

    def _run_chains(self, psi, perChain):
        from .nets.cnn import CNN
        params = psi.params_for()
        prec = psi.net._prec(psi.precision)
        C = self.numChains
        if isinstance(psi.net, CNN):
            out = torch.empty((perChain * C, self.L), dtype=torch.int32, device=self.states.device)
            self.counters.zero_()
            d = psi.net.desc(self.sampleShape)
            theta = psi.net.flat(params, psi.precision)  # kept alive until the launch is enqueued
            _lib.call("vmc_cnn_metropolis", prec, _lib.ctypes_ref(d), _lib.ptr(self.states), C,
                      _lib.ptr(theta), float(self.mu), self.seed,
                      self.callIndex & 0xFFFFFFFF, int(self.thermalizationSweeps * self.sweepSteps),
                      int(self.sweepSteps), int(perChain), _lib.ptr(out), _lib.ptr(self.counters), _lib.stream())
            self.callIndex += 1
            return out.reshape((1, perChain * C) + self.sampleShape)
        from .nets.sym_wrapper import SymNet
        L, M = psi.net.dims(params)
        out = torch.empty((perChain * C, L), dtype=torch.int32, device=self.states.device)
        self.counters.zero_()
        if isinstance(psi.net, SymNet):
            _lib.call("vmc_sym_rbm_metropolis", prec, _lib.ptr(self.states), C, L, M, _lib.ptr(params["kernel"]),
                      _lib.ptr(params.get("bias")), _lib.ptr(psi.rbm_tables()),
                      _lib.ctypes_ref(psi.net.desc(self.states.device)), float(self.mu), self.seed,
                      self.callIndex & 0xFFFFFFFF, int(self.thermalizationSweeps * self.sweepSteps),
                      int(self.sweepSteps), int(perChain), _lib.ptr(out), _lib.ptr(self.counters), _lib.stream())
            self.callIndex += 1
            return out.reshape((1, perChain * C) + self.sampleShape)
        _lib.call("vmc_rbm_metropolis", prec, _lib.ptr(self.states), C, L, M, _lib.ptr(params["kernel"]),
                  _lib.ptr(params.get("bias")), _lib.ptr(psi.rbm_tables()), float(self.mu), self.seed,
                  self.callIndex & 0xFFFFFFFF, int(self.thermalizationSweeps * self.sweepSteps),
                  int(self.sweepSteps), int(perChain), _lib.ptr(out), _lib.ptr(self.counters), _lib.stream())
        self.callIndex += 1
        return out.reshape((1, perChain * C) + self.sampleShape)

    @property
    def numProposed(self):
        return self.counters[0:1]

    @property
    def numAccepted(self):
        return self.counters[1:2]

    def acceptance_ratio(self):
        """Accepted / proposed in the last call (sampler.py:369-380)."""
        c = self.counters.cpu()
        if c[0] > 0:
            return torch.tensor([float(c[1]) / float(c[0])])
        return torch.tensor([0.])


class ExactSampler:
    """Full enumeration of the basis (sampler.py:385-534).

    Initialization arguments: ``net``, ``sampleShape``, ``lDim``,
    ``logProbFactor``."""

    def __init__(self, net, sampleShape, lDim=2, logProbFactor=0.5):
        if isinstance(sampleShape, int):
            sampleShape = (sampleShape,)
        self.psi = net
        self.sampleShape = tuple(sampleShape)
        self.N = int(np.prod(self.sampleShape))
        self.lDim = lDim
        self.logProbFactor = logProbFactor
        self.get_basis()
        self.psi(self.basis)
        self.lastNorm = torch.zeros(1, dtype=torch.float64, device=global_defs.device())

    def get_basis(self):
        """sampler.py:421-440."""
        myNumStates, _ = mpi.distribute_sampling(self.lDim ** self.N)
        first = mpi.first_sample_id()
        self.numStatesPerDevice = [myNumStates]
        basis = torch.empty((myNumStates, self.N), dtype=torch.int32, device=global_defs.device())
        _lib.call("vmc_exact_basis", _lib.ptr(basis), first, myNumStates, self.N, self.lDim, _lib.stream())
        self.basis = basis.reshape((1, myNumStates) + self.sampleShape)

    def sample(self, parameters=None, numSamples=None, multipleOf=None):
        """All basis configurations, log psi and normalised |psi|^(1/logProbFactor)
        (sampler.py:492-526); lastNorm is updated on the device."""
        if parameters is not None:
            tmp = self.psi.get_parameters()
            self.psi.set_parameters(parameters)
        logPsi = self.psi(self.basis)
        if parameters is not None:
            self.psi.set_parameters(tmp)
        n = logPsi.shape[1]
        p = torch.empty(n, dtype=torch.float64, device=logPsi.device)
        nb = _lib.query("vmc_reduce_workspace_bytes", 1)
        ws = _lib.Workspace.get(nb)
        lp = logPsi.reshape(-1).contiguous()
        _lib.call("vmc_exact_probabilities", _lib.ptr(lp), n, int(self.numStatesPerDevice[0]), _lib.ptr(self.lastNorm),
                  float(self.logProbFactor), _lib.ptr(p), None, _lib.ptr(ws), ws.numel(), _lib.stream())
        return self.basis, logPsi, p.reshape(1, n)

    def set_number_of_samples(self, N):
        pass

    def get_last_number_of_samples(self):
        return math.inf
