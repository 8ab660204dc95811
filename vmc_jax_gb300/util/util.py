"""Drivers (mirror of jVMC/util/util.py:91-212)."""

import collections
import time

import numpy as np
import torch

from .. import mpi_wrapper as mpi
from . import stepper as jVMCstepper


def get_iterable(x):
    if isinstance(x, collections.abc.Iterable):
        return x
    return (x,)


def measure(observables, psi, sampler, numSamples=None):
    """Means, variances and MC errors of operators (util.py:91-157)."""
    sampleConfigs, sampleLogPsi, p = sampler.sample(numSamples=numSamples)
    result = {}
    for name, ops in observables.items():
        tmpMeans, tmpVariances, tmpErrors = [], [], []
        for op in get_iterable(ops):
            args = ()
            if isinstance(op, collections.abc.Iterable):
                args = tuple(op[1:])
                op = op[0]
            Oloc = op.get_O_loc(sampleConfigs, psi, sampleLogPsi, *args)
            tmpMeans.append(mpi.global_mean(Oloc[..., None], p)[0])
            tmpVariances.append(mpi.global_variance(Oloc[..., None], p)[0])
            tmpErrors.append(torch.sqrt(torch.as_tensor(tmpVariances[-1]))
                             / np.sqrt(sampler.get_last_number_of_samples()))
        result[name] = {"mean": torch.real(torch.stack([torch.as_tensor(m) for m in tmpMeans])),
                        "variance": torch.real(torch.stack([torch.as_tensor(v) for v in tmpVariances])),
                        "MC_error": torch.real(torch.stack([torch.as_tensor(e) for e in tmpErrors]))}
    return result


def ground_state_search(psi, ham, tdvpEquation, sampler, numSteps=200, varianceTol=1e-10, stepSize=1e-2,
                        observables=None, outp=None):
    """Imaginary-time / SR ground-state search with Euler steps (util.py:160-212)."""
    delta = tdvpEquation.diagonalShift if "diagonalShift" in dir(tdvpEquation) else 0.
    stepper = jVMCstepper.Euler(timeStep=stepSize)
    n = 0
    varE = 1.0
    while n < numSteps and varE > varianceTol:
        tic = time.perf_counter()
        dp, _ = stepper.step(0, tdvpEquation, psi.get_parameters(), hamiltonian=ham, psi=psi, numSamples=None,
                             outp=outp)
        psi.set_parameters(dp)
        n += 1
        varE = float(tdvpEquation.get_energy_variance())
        if "set_diagonal_shift" in dir(tdvpEquation):
            delta = 0.95 * delta
            tdvpEquation.set_diagonal_shift(delta)
        if outp is not None:
            outp.print(" STEP %d" % n)
            outp.print("   Energy mean: %f" % float(tdvpEquation.get_energy_mean()))
            outp.print("   Energy variance: %f" % varE)
            outp.print("   == Time for step: %fs" % (time.perf_counter() - tic))
    return n
