"""Activation functions of the CNN path (mirror of
jVMC/nets/activation_functions.py).  The CUDA CNN kernels implement the
polynomial activations listed in ``KERNEL_CODES``; each name below is also a
callable on torch/numpy values for host-side use."""


def square(x):
    return x ** 2


def poly6(x):
    """activation_functions.py:10-12."""
    x = x ** 2
    return ((0.022222222 * x - 0.083333333) * x + 0.5) * x


def poly5(x):
    """activation_functions.py:15-17."""
    xsq = x ** 2
    return ((0.133333333 * xsq - 0.333333333) * xsq + 1.) * x


def poly4(x):
    """x^2/2 - x^4/12, the two leading Taylor terms of log(cosh(x))."""
    x2 = x * x
    return 0.5 * x2 - x2 * x2 / 12.0


activationFunctions = {"square": square, "poly5": poly5, "poly6": poly6, "poly4": poly4}

# activation id understood by the CUDA CNN kernels
KERNEL_CODES = {poly4: 0, poly6: 1, square: 2, poly5: 3}


def kernel_code(f):
    if isinstance(f, str):
        f = activationFunctions[f]
    if f not in KERNEL_CODES:
        raise NotImplementedError("activation %r has no CUDA kernel; supported: %s"
                                  % (getattr(f, "__name__", f), sorted(n for n in activationFunctions)))
    return KERNEL_CODES[f]
