"""Device and dtype definitions (mirror of jVMC/global_defs.py).

jVMC maps its data-parallel work over every local device with ``jax.pmap``
and carries a leading device dimension on every array.  This package runs
one process on one GPU, so that dimension is always 1 and
``set_pmap_devices`` accepts exactly one device.
"""

import numpy as np
import torch

# Complex floating point (global_defs.py:4)
tCpx = np.complex128
# Real floating point (global_defs.py:6)
tReal = np.float64

torch_cpx = torch.complex128
torch_real = torch.float64

myPmapDevices = [0]
myDeviceCount = 1


def device():
    """The CUDA device all arrays live on."""
    return torch.device("cuda", myPmapDevices[0])


def device_count():
    return 1


def devices():
    return list(myPmapDevices)


def set_pmap_devices(devices):
    """Select the device (global_defs.py:38-46); only one device per process."""
    if isinstance(devices, (list, tuple)):
        if len(devices) != 1:
            raise NotImplementedError("one device per process: data parallelism over several GPUs "
                                      "runs one process per GPU")
        devices = devices[0]
    if isinstance(devices, torch.device):
        devices = devices.index or 0
    global myPmapDevices
    myPmapDevices = [int(devices)]
