"""GB300-native (sm_103a) per-step VMC hot path of jVMC.

The package mirrors jVMC's public modules for the hot path --
``vqs.NQS``, ``sampler.MCSampler`` / ``ExactSampler``, ``operator``
(branch-free operators), ``stats.SampledObs``, ``util.TDVP`` and the
integrators -- and runs their work in the CUDA kernels of
``libvmc_gb300.so`` (C ABI: include/vmc_gb300.h).  Arrays are torch CUDA
tensors with jVMC's leading device dimension of 1.
"""

from . import _lib
from . import global_defs
from . import mpi_wrapper
from . import nets
from . import vqs
from . import sampler
from . import operator
from . import stats
from . import util
from .version import __version__

__all__ = ["global_defs", "mpi_wrapper", "nets", "vqs", "sampler", "operator", "stats", "util", "__version__"]
