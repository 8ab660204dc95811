"""Host drivers over the TDVP path: measurement of operators and the
ground-state search (the functions of jVMC/util/util.py:91-212).  They only
call the sampler, the operators and the stepper of this package."""

import collections.abc
import time

import torch

from .. import mpi_wrapper as mpi
from . import stepper as jVMCstepper


def _operator_calls(spec):
    """(operator, extra arguments) for one entry of an observables dict.  An
    entry is an operator, an ``(operator, *args)`` tuple, or a list of
    those."""
    items = spec if isinstance(spec, collections.abc.Iterable) else (spec,)
    for item in items:
        if isinstance(item, collections.abc.Iterable):
            head, *rest = item
            yield head, tuple(rest)
        else:
            yield item, ()


def measure(observables, psi, sampler, numSamples=None):
    """Mean, variance and Monte Carlo error of each observable on one fresh
    sample (the result layout of util.py:91-157): ``{name: {"mean",
    "variance", "MC_error"}}``, one entry per operator of the name, real
    parts.  Means and variances are the FP64 weighted sums of the sample
    weights ``p``; the error is sqrt(variance / number of samples)."""
    configs, logPsi, p = sampler.sample(numSamples=numSamples)
    count = float(sampler.get_last_number_of_samples())
    result = {}
    for name, spec in observables.items():
        rows = []
        for op, args in _operator_calls(spec):
            oloc = op.get_O_loc(configs, psi, logPsi, *args)
            mean = torch.as_tensor(mpi.global_mean(oloc[..., None], p)[0])
            var = torch.real(torch.as_tensor(mpi.global_variance(oloc[..., None], p)[0]))
            rows.append(torch.stack([torch.real(mean).to(torch.float64), var.to(torch.float64),
                                     torch.sqrt(var.to(torch.float64) / count)]))
        table = torch.stack(rows)
        result[name] = {"mean": table[:, 0], "variance": table[:, 1], "MC_error": table[:, 2]}
    return result


def ground_state_search(psi, ham, tdvpEquation, sampler, numSteps=200, varianceTol=1e-10, stepSize=1e-2,
                        observables=None, outp=None):
    """Stochastic-reconfiguration descent (util.py:160-212): Euler steps of
    ``stepSize`` on ``tdvpEquation`` until the energy variance of a step is
    at most ``varianceTol`` or ``numSteps`` steps were made; returns the
    number of steps.  A solver with a diagonal shift has it scaled by 0.95
    after every step.  With ``outp`` given, each step is reported through
    ``outp.print``, and with ``observables`` also given they are measured
    before the first and after every step (``outp.write_observables``)."""
    euler = jVMCstepper.Euler(timeStep=stepSize)
    shift = getattr(tdvpEquation, "diagonalShift", 0.)
    decaying = hasattr(tdvpEquation, "set_diagonal_shift")
    record = outp is not None and observables is not None and hasattr(outp, "write_observables")
    if record:
        outp.write_observables(0, **measure(observables, psi, sampler))
    for step in range(1, numSteps + 1):
        started = time.perf_counter()
        theta, _ = euler.step(0, tdvpEquation, psi.get_parameters(), hamiltonian=ham, psi=psi, numSamples=None,
                              outp=outp)
        psi.set_parameters(theta)
        variance = float(tdvpEquation.get_energy_variance())
        if record:
            outp.write_observables(step, **measure(observables, psi, sampler))
        if decaying:
            shift *= 0.95
            tdvpEquation.set_diagonal_shift(shift)
        if outp is not None:
            outp.print("step %4d  E = %.12g  var(E) = %.6g  (%.3f s)"
                       % (step, float(tdvpEquation.get_energy_mean()), variance, time.perf_counter() - started))
        if variance <= varianceTol:
            return step
    return numSteps
