"""Solvers, integrators and drivers (mirror of jVMC.util)."""

from .tdvp import TDVP, realFun, imagFun
from .minsr import MinSR
from . import stepper
from . import symmetries
from .checkpoint import save_checkpoint, load_checkpoint
from .util import measure, ground_state_search

__all__ = ["TDVP", "MinSR", "realFun", "imagFun", "stepper", "symmetries", "save_checkpoint", "load_checkpoint", "measure", "ground_state_search"]
