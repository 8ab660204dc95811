"""Solvers, integrators and drivers (mirror of jVMC.util)."""

from .tdvp import TDVP, realFun, imagFun
from .minsr import MinSR
from . import stepper
from . import symmetries
from .util import measure, ground_state_search

__all__ = ["TDVP", "MinSR", "realFun", "imagFun", "stepper", "symmetries", "measure", "ground_state_search"]
