"""Network ansätze with CUDA kernels (mirror of jVMC.nets)."""

from .rbm import CpxRBM
from .cnn import CNN
from . import activation_functions

__all__ = ["CpxRBM", "CNN", "activation_functions"]
