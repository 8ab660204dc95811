"""Network ansätze with CUDA kernels (mirror of jVMC.nets)."""

from .rbm import CpxRBM
from .cnn import CNN
from .sym_wrapper import SymNet
from . import activation_functions
from . import sym_wrapper

__all__ = ["CpxRBM", "CNN", "SymNet", "activation_functions", "sym_wrapper"]
