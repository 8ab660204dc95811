"""Branch-free operators (mirror of jVMC/operator/branch_free.py).

Operator strings are built with the same algebra as the reference
(``LocalOp``, ``OpStr``, ``scal_opstr``); ``BranchFreeOperator.compile``
produces the same tables (strings stored right-to-left, padded with Id(0)),
uploads them to the GPU, and the CUDA kernels of csrc/branch_free.cu and
csrc/rbm.cu expand them.
"""

import numpy as np
import torch

from .. import _lib
from .. import global_defs
from ..vqs import as_configs
from .base import Operator

opDtype = global_defs.tCpx


class LocalOp(dict):
    """Operator acting on one local Hilbert space (branch_free.py:279-308):
    keys ``idx``, ``map``, ``matEls``, ``diag`` and optionally ``fermionic``.
    A product with anything else gives an ``OpStr``."""

    def __init__(self, **kwargs):
        super().__init__(**kwargs)

    def __mul__(self, other):
        return OpStr(self) * other

    def __rmul__(self, other):
        return other * OpStr(self)


def Id(idx=0, lDim=2):
    """Identity (branch_free.py:17-33)."""
    return LocalOp(idx=idx, map=np.array(list(range(lDim)), dtype=np.int32),
                   matEls=np.array([1.] * lDim, dtype=opDtype), diag=True)


def Sx(idx):
    """Pauli sigma^x (branch_free.py:36-51)."""
    return LocalOp(idx=idx, map=np.array([1, 0], dtype=np.int32), matEls=np.array([1.0, 1.0], dtype=opDtype),
                   diag=False)


def Sy(idx):
    """Pauli sigma^y (branch_free.py:54-69)."""
    return LocalOp(idx=idx, map=np.array([1, 0], dtype=np.int32), matEls=np.array([1.j, -1.j], dtype=opDtype),
                   diag=False)


def Sz(idx):
    """Pauli sigma^z (branch_free.py:72-87)."""
    return LocalOp(idx=idx, map=np.array([0, 1], dtype=np.int32), matEls=np.array([-1.0, 1.0], dtype=opDtype),
                   diag=True)


def Sp(idx):
    """S^+ ladder operator (branch_free.py:90-105)."""
    return LocalOp(idx=idx, map=np.array([1, 0], dtype=np.int32), matEls=np.array([1.0, 0.0], dtype=opDtype),
                   diag=False)


def Sm(idx):
    """S^- ladder operator (branch_free.py:108-123)."""
    return LocalOp(idx=idx, map=np.array([0, 0], dtype=np.int32), matEls=np.array([0.0, 1.0], dtype=opDtype),
                   diag=False)


def number(idx):
    """Fermionic number operator c^dagger c (branch_free.py:128-146)."""
    return LocalOp(idx=idx, map=np.array([0, 1], dtype=np.int32), matEls=np.array([0., 1.], dtype=opDtype),
                   diag=True, fermionic=False)


def creation(idx):
    """Fermionic creation operator (branch_free.py:150-168)."""
    return LocalOp(idx=idx, map=np.array([1, 0], dtype=np.int32), matEls=np.array([1., 0.], dtype=opDtype),
                   diag=False, fermionic=True)


def annihilation(idx):
    """Fermionic annihilation operator (branch_free.py:172-190)."""
    return LocalOp(idx=idx, map=np.array([1, 0], dtype=np.int32), matEls=np.array([0., 1.], dtype=opDtype),
                   diag=False, fermionic=True)


class Coefficient:
    """Prefactor of an operator string: the product of its factors, each a
    number or a function of the operator's arguments (the time, for
    instance).  Calling it evaluates every factor with the arguments given
    and multiplies the values, left to right."""

    __slots__ = ("factors",)

    def __init__(self, factors):
        self.factors = tuple(factors)

    def __call__(self, *args, **kwargs):
        value = 1.0
        for f in self.factors:
            value = value * (f(*args) if callable(f) else f)
        return value

    def __repr__(self):
        return "Coefficient%r" % (self.factors,)


def _factors_and_ops(x):
    """Split an operand of the string algebra into (prefactor factors, local
    operators).  Local operators given as plain dicts become ``LocalOp``."""
    if isinstance(x, LocalOp):
        return [], [x]
    if isinstance(x, dict):
        return [], [LocalOp(**x)]
    if isinstance(x, Coefficient):
        return list(x.factors), []
    if isinstance(x, tuple):
        factors, ops = [], []
        for item in x:
            f, o = _factors_and_ops(item)
            factors += f
            ops += o
        return factors, ops
    return [x], []  # a number or a function of the operator arguments


class OpStr(tuple):
    """Operator string (branch_free.py:203-255), stored as a tuple
    ``(Coefficient, op_1, ..., op_n)``, or ``(op_1, ..., op_n)`` when it
    has no prefactor.  Items may be given in any order; all numbers and
    functions among them are collected into the one leading ``Coefficient``.
    ``op_1 ... op_n`` act right to left, as in the reference.  A product
    of strings (or of a string and a local operator, number or function)
    multiplies the coefficients and concatenates the local operators in
    the order of the factors."""

    def __new__(cls, *items):
        factors, ops = _factors_and_ops(items)
        head = (Coefficient(factors),) if factors else ()
        return super().__new__(cls, head + tuple(ops))

    def __mul__(self, other):
        return OpStr(self, other)

    def __rmul__(self, other):
        return OpStr(other, self)


def scal_opstr(a, op):
    """The operator string ``op`` (an ``OpStr`` or a tuple of local
    operators) multiplied by ``a``, a number or a function of the operator
    arguments (branch_free.py:258-276)."""
    if not isinstance(op, tuple):
        raise RuntimeError("scal_opstr: the operator must be an OpStr or a tuple of local operators, not %s"
                           % type(op).__name__)
    return OpStr(a, op)


class BranchFreeOperator(Operator):
    """Operator given as a sum of operator strings (branch_free.py:311-487).

    Initializer arguments:
        * ``lDim``: Dimension of local Hilbert space.
        * ``ElocBatchSize``: batch size of ``get_O_loc`` (results do not depend on it).
    """

    def __init__(self, lDim=2, **kwargs):
        self.ops = []
        self.lDim = lDim
        super().__init__(**kwargs)

    def add(self, opDescr):
        """Add an operator string (branch_free.py:330-342)."""
        if not isinstance(opDescr, tuple):
            opDescr = (opDescr,)
        self.ops.append(opDescr)
        self.compiled = False

    def __iadd__(self, opDescr):
        self.add(opDescr)
        return self

    def compile(self):
        """Tables of the operator strings (branch_free.py:348-441): idx, map,
        matEls and fermion flags of shape (numOps, maxOpStrLength[, lDim]),
        every string right-to-left and padded with Id(0); the diagonal
        strings; the prefactor functions.  The tables are uploaded to the GPU."""
        self.maxOpStrLength = 0
        for op in self.ops:
            tmpLen = len(op)
            if callable(op[0]):
                tmpLen -= 1
            self.maxOpStrLength = max(self.maxOpStrLength, tmpLen)
        IdOp = Id(lDim=self.lDim)
        idx, mp, me, fe, diag, pref = [], [], [], [], [], []
        for o, op in enumerate(self.ops):
            k0 = 0
            if callable(op[0]):
                pref.append((o, op[0]))
                k0 = 1
            isDiagonal = True
            ri, rm, rme, rf = [], [], [], []
            for k in range(self.maxOpStrLength):
                kRev = len(op) - k - 1
                if kRev >= k0:
                    lo = op[kRev]
                    if not lo["diag"]:
                        isDiagonal = False
                    ri.append(lo["idx"])
                    rm.append(np.asarray(lo["map"]))
                    rme.append(np.asarray(lo["matEls"]))
                    rf.append(1 if lo.get("fermionic", False) else 0)
                else:
                    ri.append(IdOp["idx"])
                    rm.append(IdOp["map"])
                    rme.append(IdOp["matEls"])
                    rf.append(0)
            if isDiagonal:
                diag.append(o)
            idx.append(ri)
            mp.append(rm)
            me.append(rme)
            fe.append(rf)
        self.idxC = np.array(idx, dtype=np.int32)
        self.mapC = np.array(mp, dtype=np.int32)
        self.matElsC = np.array(me, dtype=opDtype)
        self.fermionicC = np.array(fe, dtype=np.int32)
        self.diag = np.array(diag, dtype=np.int32)
        self.prefactor = pref
        if self.maxOpStrLength > _MAX_LEN:
            raise NotImplementedError("operator strings longer than %d" % _MAX_LEN)
        dev = global_defs.device()
        self._dev = {
            "idx": torch.as_tensor(self.idxC, device=dev),
            "map": torch.as_tensor(self.mapC, device=dev),
            "mat_els": torch.as_tensor(self.matElsC, device=dev),
            "fermi": torch.as_tensor(self.fermionicC, device=dev),
            "diag": torch.as_tensor(self.diag if len(self.diag) else np.zeros(1, np.int32), device=dev),
        }
        self._pref_cache = None
        self.compiled = True
        return self.arg_fun

    def arg_fun(self, *args):
        """Values of the prefactors for the operator arguments
        (branch_free.py:416-438)."""
        res = np.ones(self.idxC.shape[0], dtype=opDtype)
        for i, f in self.prefactor:
            res[i] = f(*args)
        return res

    def _device_operator(self, *args):
        if not self.compiled:
            self.compile()
        pref = self.arg_fun(*args)
        if self._pref_cache is None or not np.array_equal(self._pref_cache[0], pref):
            self._pref_cache = (pref, torch.as_tensor(pref, device=global_defs.device()))
        d = self._dev
        st = _lib.BfOperator(
            num_ops=int(self.idxC.shape[0]), max_len=int(self.idxC.shape[1]), local_dim=int(self.lDim),
            num_diag=int(len(self.diag)), idx=_lib.ptr(d["idx"]), map=_lib.ptr(d["map"]),
            mat_els=_lib.ptr(d["mat_els"]), fermi=_lib.ptr(d["fermi"]), prefactor=_lib.ptr(self._pref_cache[1]),
            diag=_lib.ptr(d["diag"]))
        return st

    # --------------------------------------------------- reference layout
    def get_s_primes(self, s, *args):
        """Connected configurations s' and matrix elements (base.py:116-160)
        in the reference layout: s' (1, N*K, *sampleShape) int32 and matrix
        elements (1, N, K) complex128, K = max number of nonzeros."""
        s = as_configs(s)
        op = self._device_operator(*args)
        sampleShape = tuple(s.shape[2:])
        flat = s.reshape(-1, int(np.prod(sampleShape)))
        N, L = flat.shape
        K0 = op.num_ops
        dev = flat.device
        mfull = torch.empty((N, K0), dtype=torch.complex128, device=dev)
        nzi = torch.empty((N, K0), dtype=torch.int32, device=dev)
        cnt = torch.empty(N, dtype=torch.int32, device=dev)
        kmax = torch.empty(1, dtype=torch.int32, device=dev)
        _lib.call("vmc_bf_matrix_elements", _lib.ptr(flat), N, L, op, _lib.ptr(mfull), _lib.ptr(nzi), _lib.ptr(cnt),
                  _lib.ptr(kmax), _lib.stream())
        K = int(kmax.item())  # host sync, as jnp.max(numNonzero) in base.py:157
        sp = torch.empty((N * K, L), dtype=torch.int32, device=dev)
        mat = torch.empty((N, K), dtype=torch.complex128, device=dev)
        _lib.call("vmc_bf_gather", _lib.ptr(flat), N, L, op, _lib.ptr(mfull), _lib.ptr(nzi), _lib.ptr(cnt), K,
                  _lib.ptr(sp), _lib.ptr(mat), _lib.stream())
        self.numNonzero = cnt.reshape(s.shape[:2])
        self.matEl = mat.reshape(s.shape[:2] + (K,))
        self.sp = sp.reshape((s.shape[0], N * K // s.shape[0]) + sampleShape)
        return self.sp, self.matEl

    # ------------------------------------------------------- fused path
    def fused_capable(self, psi):
        from ..nets.cnn import CNN
        from ..nets.rbm import CpxRBM
        from ..nets.sym_wrapper import SymNet
        if isinstance(psi.net, SymNet):
            return psi.net.average == 0 and self.lDim == 2
        return isinstance(psi.net, (CpxRBM, CNN)) and self.lDim == 2

    def get_O_loc_fused(self, samples, psi, logPsiS=None, *args):
        """O_loc(s) of a CpxRBM, symmetrised CpxRBM or CNN state without
        materialising s': one kernel applies every string and forms
        psi(s')/psi(s) from tanh(theta) and the exp(+-2W) tables (csrc/rbm.cu,
        csrc/sym_rbm.cu) or from local updates of the CNN's activations
        (csrc/cnn.cu).  With ``logPsiS`` given the result is
        relative to it, as in base.py:162-164."""
        s = as_configs(samples)
        psi.init_net(s)
        op = self._device_operator(*args)
        flat = s.reshape(s.shape[0] * s.shape[1], -1)
        N, L = flat.shape
        params = psi.params_for()
        prec = psi.net._prec(psi.precision)
        lps = None
        if logPsiS is not None:
            lps = torch.as_tensor(logPsiS).to(device=flat.device, dtype=torch.complex128).reshape(-1).contiguous()
        out = torch.empty(N, dtype=torch.complex128, device=flat.device)
        from ..nets.cnn import CNN
        if isinstance(psi.net, CNN):
            d = psi.net.desc(tuple(s.shape[2:]))
            theta = psi.net.flat(params, psi.precision)  # kept alive until the launch is enqueued
            _lib.call("vmc_cnn_oloc_fused", prec, _lib.ctypes_ref(d), _lib.ptr(flat), N, _lib.ptr(theta), op,
                      _lib.ptr(lps), _lib.ptr(out), _lib.stream())
            return out.reshape(s.shape[:2])
        M = int(params["kernel"].shape[1])
        from ..nets.sym_wrapper import SymNet
        if isinstance(psi.net, SymNet):
            _lib.call("vmc_sym_rbm_oloc_fused", prec, _lib.ptr(flat), N, L, M, _lib.ptr(params["kernel"]),
                      _lib.ptr(params.get("bias")), _lib.ptr(psi.rbm_tables()),
                      _lib.ctypes_ref(psi.net.desc(flat.device)), op, _lib.ptr(lps), _lib.ptr(out), _lib.stream())
            return out.reshape(s.shape[:2])
        _lib.call("vmc_rbm_oloc_fused", prec, _lib.ptr(flat), N, L, M, _lib.ptr(params["kernel"]),
                  _lib.ptr(params.get("bias")), _lib.ptr(psi.rbm_tables()), op, _lib.ptr(lps), _lib.ptr(out),
                  _lib.stream())
        return out.reshape(s.shape[:2])


_MAX_LEN = 16
