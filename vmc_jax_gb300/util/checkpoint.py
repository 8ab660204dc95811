"""Checkpoint and resume of a run's device state: the role of
OutputManager.write_network_checkpoint / get_network_checkpoint
(output_manager.py:118-174), which append the flat parameter vector to an
HDF5 file, here as one torch file (h5py is not available) that also holds
what the reference does not keep: the Metropolis chains, their random-stream
position and the adaptive integrator's step, so that a resumed run draws the
same samples as an uninterrupted one."""

import torch

from .. import global_defs

FORMAT = "vmc_jax_gb300.checkpoint/1"


def save_checkpoint(path, psi, sampler=None, stepper=None, t=None):
    """Write the parameters of ``psi`` and, when given, the sampler's chain
    state and the integrator's time step; ``t`` is stored as is."""
    state = {"format": FORMAT, "params": psi.get_parameters().detach().cpu(), "t": t}
    if sampler is not None:
        s = {}
        if hasattr(sampler, "states"):
            s["states"] = sampler.states.detach().cpu()
            s["callIndex"] = int(sampler.callIndex)
            s["seed"] = int(sampler.seed)
        if hasattr(sampler, "lastNorm"):
            s["lastNorm"] = sampler.lastNorm.detach().cpu()
        state["sampler"] = s
    if stepper is not None:
        state["stepper"] = {"dt": float(stepper.dt)}
    torch.save(state, path)


def load_checkpoint(path, psi, sampler=None, stepper=None):
    """Restore what :func:`save_checkpoint` wrote into existing objects of the
    same shapes; returns the stored ``t``."""
    state = torch.load(path, map_location="cpu")
    if state.get("format") != FORMAT:
        raise ValueError("%s is not a checkpoint of this library" % (path,))
    psi.set_parameters(state["params"].to(global_defs.device()))
    if sampler is not None and "sampler" in state:
        s = state["sampler"]
        if "states" in s:
            if tuple(s["states"].shape) != tuple(sampler.states.shape):
                raise ValueError("checkpoint chains %s do not match the sampler's %s"
                                 % (tuple(s["states"].shape), tuple(sampler.states.shape)))
            sampler.states.copy_(s["states"].to(sampler.states.device))
            sampler.callIndex = s["callIndex"]
            sampler.seed = s["seed"]
        if "lastNorm" in s:
            sampler.lastNorm.copy_(s["lastNorm"].to(sampler.lastNorm.device))
    if stepper is not None and "stepper" in state:
        stepper.dt = state["stepper"]["dt"]
    return state.get("t")
