"""ctypes binding of ``libvmc_gb300.so`` (the C ABI in include/vmc_gb300.h).

The argument types of every entry point are read from the header itself, so
the Python side and the C side cannot drift apart.  Device buffers are torch
CUDA tensors; only their raw pointers cross the boundary.

There is no fallback: if the library is missing and cannot be built, or no
CUDA device is present, every call raises.
"""

import ctypes
import os
import re
import threading

import torch

from . import build_ext

HEADER = os.path.join(build_ext.ROOT, "include", "vmc_gb300.h")

VMC_F64 = 0
VMC_F32 = 1
VMC_GRAD_REFERENCE = 0
VMC_GRAD_COMPACT = 1


class VmcError(RuntimeError):
    """A non-zero status returned by the CUDA library."""


class BfOperator(ctypes.Structure):
    """Mirror of ``vmc_bf_operator`` (device pointers to the compiled tables)."""
    _fields_ = [
        ("num_ops", ctypes.c_int32),
        ("max_len", ctypes.c_int32),
        ("local_dim", ctypes.c_int32),
        ("num_diag", ctypes.c_int32),
        ("idx", ctypes.c_void_p),
        ("map", ctypes.c_void_p),
        ("mat_els", ctypes.c_void_p),
        ("fermi", ctypes.c_void_p),
        ("prefactor", ctypes.c_void_p),
        ("diag", ctypes.c_void_p),
    ]


_CTYPES = {
    "int32_t": ctypes.c_int32, "int64_t": ctypes.c_int64, "uint32_t": ctypes.c_uint32,
    "uint64_t": ctypes.c_uint64, "size_t": ctypes.c_size_t, "double": ctypes.c_double,
    "float": ctypes.c_float, "int": ctypes.c_int, "vmc_stream_t": ctypes.c_void_p,
}


def _ctype(decl):
    decl = decl.strip()
    base = decl.replace("const", "").strip()
    if base.endswith("*"):
        inner = base.rstrip("*").strip()
        if inner == "vmc_bf_operator":
            return ctypes.POINTER(BfOperator)
        if inner in ("vmc_cnn_desc", "vmc_sym_desc"):
            return ctypes.c_void_p
        if inner == "char":
            return ctypes.c_char_p
        return ctypes.c_void_p
    if base == "void":
        return None
    return _CTYPES[base]


def parse_header(path=HEADER):
    """Return {name: (restype, [argtypes])} for every function in the header."""
    with open(path) as f:
        src = f.read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"//[^\n]*", "", src)
    protos = {}
    for m in re.finditer(r"\b(int|size_t|const char\*|void)\s+(vmc_\w+)\s*\(([^)]*)\)\s*;", src):
        ret, name, args = m.group(1), m.group(2), m.group(3)
        argtypes = []
        a = args.strip()
        if a and a != "void":
            for part in a.split(","):
                part = part.strip()
                # strip the parameter name
                pm = re.match(r"(.*?[\s\*])(\w+)$", part)
                typ = pm.group(1).strip() if pm else part
                argtypes.append(_ctype(typ))
        restype = {"int": ctypes.c_int, "size_t": ctypes.c_size_t, "const char*": ctypes.c_char_p,
                   "void": None}[ret]
        protos[name] = (restype, argtypes)
    return protos


_lock = threading.Lock()
_lib = None


def load(build_if_missing=True):
    """Load (building first if needed) the shared library and bind every
    function declared in the header."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(build_ext.LIB) or not build_ext.up_to_date():
            if not build_if_missing:
                raise VmcError("libvmc_gb300.so is not built (run python -m vmc_jax_gb300.build_ext)")
            build_ext.build()
        lib = ctypes.CDLL(build_ext.LIB)
        for name, (res, args) in parse_header().items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


# kernels launched by one successful call of each entry point
KERNELS_PER_CALL = {
    "vmc_exact_basis": 1, "vmc_exact_probabilities": 2, "vmc_mc_probabilities": 2, "vmc_rbm_prepare": 2,
    "vmc_rbm_logpsi": 1, "vmc_rbm_gradients": 1, "vmc_rbm_metropolis": 1, "vmc_bf_matrix_elements": 1,
    "vmc_bf_gather": 1, "vmc_oloc_from_sprimes": 1, "vmc_rbm_oloc_fused": 1, "vmc_weighted_mean_var": 3,
    "vmc_rbm_grad_stats": 3, "vmc_rbm_centered_gradients": 1, "vmc_rbm_snr_data": 1, "vmc_gram_to_hermitian": 1,
    "vmc_zgemv": 2, "vmc_tdvp_snr": 1, "vmc_tdvp_regularize": 3, "vmc_gram_bf16x3": 1,
    "vmc_gemm_bf16x3_colsq": 2, "vmc_eigvec_bf16x2": 1, "vmc_cnn_logpsi": 1, "vmc_cnn_gradients": 1,
    "vmc_cnn_metropolis": 1, "vmc_rbm_vjp": 4, "vmc_rbm_grad_stats_noalloc": 3,
    "vmc_rbm_metropolis_devcall": 2, "vmc_sym_rbm_logpsi": 1, "vmc_sym_rbm_gradients": 1,
    "vmc_sym_rbm_oloc_fused": 1, "vmc_sym_rbm_metropolis": 1, "vmc_dense_grad_stats": 2,
    "vmc_dense_centered_gradients": 1, "vmc_dense_snr_data": 1, "vmc_cnn_oloc_fused": 1,
}
launch_count = 0


def _slice_launches(K):
    """Kernels of one Ozaki operand slicing: row exponents, slices, and the
    padding columns when 2K is not a multiple of 64."""
    return 2 + (1 if (2 * K) % 64 else 0)


def _refine_launches(args):
    """Kernels of one vmc_eigh_refine_top call (n, A, lda, k, steps, ...)."""
    n, k, q = int(args[0]), int(args[3]), int(args[4])
    b = n - k
    c = _slice_launches(n)                                  # A
    c += q * (_slice_launches(n) + 3)                       # power steps: slice, product, assembly, scaling
    c += 3 * (_slice_launches(n) + 2)                       # Y, G, H
    c += 2 * _slice_launches(k) + 2                         # X C
    if b > 0:
        chunks = (b + 4095) // 4096
        c += _slice_launches(n) + _slice_launches(k)        # V_top^H and V_top
        c += chunks * (_slice_launches(n) + _slice_launches(k) + 4) + 1
    return c


KERNELS_PER_CALL.update({
    "vmc_zgemm_ozaki": lambda a: _slice_launches(int(a[4])) * 2 + 2,
    "vmc_eigh_fp32": 2, "vmc_eigh_fp64": 0, "vmc_eigh_refine_top": _refine_launches,
    "vmc_tc_wait_check": 1,
})


def call(name, *args):
    """Call a status-returning entry point; raise VmcError on failure."""
    global launch_count
    lib = load()
    rc = getattr(lib, name)(*args)
    n = KERNELS_PER_CALL.get(name, 1)
    if callable(n):
        n = n(args)
    if name == "vmc_zgemv" and args and args[0]:
        n = 1  # the adjoint product is one kernel, the plain one two
    launch_count += n
    if rc != 0:
        msg = lib.vmc_last_error_string().decode(errors="replace")
        raise VmcError(f"{name} failed with status {rc}: {msg}")
    return rc


def query(name, *args):
    """Call a value-returning entry point (sizes, version)."""
    return getattr(load(), name)(*args)


def ctypes_ref(struct):
    """Address of a ctypes structure for a ``const T*`` argument."""
    return ctypes.addressof(struct)


def ptr(t):
    """Raw device pointer of a CUDA tensor (None -> NULL)."""
    if t is None:
        return None
    if not t.is_cuda:
        raise VmcError("expected a CUDA tensor, got a tensor on %s" % t.device)
    if t.is_complex() and t.is_conj():
        raise VmcError("a tensor with a lazy conjugate bit holds the unconjugated values: call resolve_conj() first")
    return t.data_ptr()


def stream():
    return torch.cuda.current_stream().cuda_stream


def require_cuda():
    if not torch.cuda.is_available():
        raise VmcError("vmc_jax_gb300 runs on a CUDA device; none is available")


class Workspace:
    """Grow-only per-device scratch buffer handed to entry points that need
    workspace (the library itself never allocates)."""

    _bufs = {}

    @classmethod
    def get(cls, nbytes, device=None):
        """Scratch of at least nbytes for the calling thread on ``device``
        (one buffer per host thread, so concurrent solvers never share)."""
        device = torch.device("cuda", torch.cuda.current_device()) if device is None else device
        key = (device.index, threading.get_ident())
        buf = cls._bufs.get(key)
        if buf is None or buf.numel() < nbytes:
            cls._bufs.pop(key, None)
            buf = None
            buf = torch.empty(max(int(nbytes), 1 << 20), dtype=torch.uint8, device=device)
            cls._bufs[key] = buf
        return buf

    @classmethod
    def release(cls):
        """Drop the calling thread's buffers (on every device).  A host thread
        that ends calls this, or its scratch would stay allocated: buffers are
        kept per thread so that concurrent solvers never share one."""
        tid = threading.get_ident()
        for key in [k for k in cls._bufs if k[1] == tid]:
            cls._bufs.pop(key, None)
