"""TDVP solver (mirror of jVMC/util/tdvp.py:26-326).

For a CpxRBM (or symmetrised CpxRBM) state the right-hand side runs as one
GPU pipeline:

  sample -> fused O_loc -> FP64 mean/variance of E_loc -> FP64 means of O_k
  and force F -> centred data -> Gram contraction S (FP64 / FP32 / mixed
  BF16x3 on tcgen05) -> eigendecomposition -> SNR contraction ->
  cutoff loop on the device -> update.

The centred data come from the configurations (CpxRBM: O is never stored)
or from the materialised O of the network's gradient kernel (SymNet); see
util/sr_data.py.

The holomorphic ansatz makes the reference's 2P real representation of S
(tdvp.py:144: makeReal of the 2P x 2P covariance) the real representation
of the complex P x P matrix A = <O^dagger O>_c; its spectrum is that of A
with every eigenvalue paired ({l, l} for makeReal='real', {l, -l} for
'imag'), and the update solves A z = -x covar(O, E) with the same
regulariser, returned as [Re z; Im z] per leaf.  The eigendecomposition is
therefore done on the P x P complex matrix: cuSOLVER FP64, or, in the mixed
form with Monte Carlo samples, FP32 cuSOLVER followed by FP64-accurate
Rayleigh-Ritz refinement of the eigenpairs that carry the solve
(csrc/eigh.cu).

SNR: for makeReal='imag' the SNR of a pair is unique and identical to the
reference's; for makeReal='real' the reference's eigenvectors within a
degenerate pair are an arbitrary LAPACK basis and so is the split of the
SNR between them; here both members get the rotation-invariant pair value
N|u^H f|^2 / sum_n w_n |u^H (h_n - f)|^2.
"""

import warnings

import numpy as np
import torch

from .. import _lib
from .. import global_defs
from .. import mpi_wrapper as mpi
from ..sampler import ExactSampler
from ..stats import SampledObs
from .timing import TIMER


def _gram_mod():
    from . import gram
    return gram


def realFun(x):
    """tdvp.py:14-15."""
    return torch.real(x) if isinstance(x, torch.Tensor) else np.real(x)


def imagFun(x):
    """tdvp.py:18-19."""
    return 0.5 * (x - (torch.conj(x) if isinstance(x, torch.Tensor) else np.conj(x)))


def transform_helper(x, rhsPrefactor, makeReal):
    """tdvp.py:22-23."""
    return makeReal((-rhsPrefactor) * x)


# Share of the update the eigenpairs left at FP32 accuracy may carry.  The
# mixed form's update already moves by ~1e-7 relative with the arbitrary
# phases of the eigenvectors (its per-eigenvector SNR contraction runs in
# BF16x3, whose rounding depends on them) and differs from the FP64 form by
# ~4e-4 through the BF16x3 S; a bulk share below 1e-6 stays under both.
REFINE_EXCLUDED_NORM = 1e-6
REFINE_MAX_FRACTION = 0.5      # refine at most this fraction of the spectrum
REFINE_MAX_RHO = 0.25          # largest |lambda_excluded / lambda_carrying| accepted
REFINE_TARGET = 1e-15          # FP32 start error along the rest left after the power steps
# The FP32 mixing (~u32 lambda_max / (lambda_j - lambda_i), ~6e-8 for the
# pairs far apart) of a larger refined eigenvector j into the column of a
# smaller one i grows by lambda_j / lambda_i per power step (the steps scale
# each column by its own 1 / lambda); over the q steps by at most
# (lambda_max / lambda_b)^q.  Below 1e10 the mixing stays below ~1e3, the
# Rayleigh-Ritz Gram matrix X^H X keeps a condition number below ~1e6 and
# the refined pairs lose at most ~6 of their ~15 digits; far above it the
# columns become numerically dependent (zhegvd fails, and the step falls
# back to the FP64 eigensolver).
REFINE_MAX_GROWTH = 1e10


def solve_weights(ev, vtf, snr, pinvCutoff, snrTol, snrMargin=1.0):
    """Upper bound of every eigenpair's share |pinv_k (U^H f)_k| of the
    update (tdvp.py:195-211): the regulariser at the smallest cutoff the
    loop can reach, the SNR scaled by snrMargin."""
    lmax = np.max(np.abs(ev))
    r = np.abs(ev) / lmax if lmax > 0 else np.zeros_like(ev)
    with np.errstate(divide="ignore", over="ignore", invalid="ignore"):
        regc = np.where(r > 0, 1.0 / (1.0 + (pinvCutoff / r) ** 6), 0.0)
        regs = 1.0 / (1.0 + (snrTol / (snrMargin * np.maximum(snr, 1e-300))) ** 6)
        inv = np.where(r > 1e-14, 1.0 / np.maximum(np.abs(ev), 1e-300), 0.0)
    return inv * regc * regs * np.abs(vtf)


def refine_plan(ev, vtf, snr, pinvCutoff, snrTol):
    """Number k of top eigenpairs to refine to FP64 accuracy and the power
    steps q, from the FP32 eigendecomposition (ev ascending); None when the
    FP64 eigensolver of the whole matrix is to be used.

    Only the spectrum is used: FP32 eigenvalues below the FP32 noise floor
    (the size of the most negative one of this positive semi-definite S,
    at least 64 u32 lambda_max) are not resolved, and the FP32 bulk vectors
    carry a ~1e-6 share of the top block that inflates their projections of
    F and their SNR (which enters to the 6th power), so their weights say
    nothing about the bulk.  The split b is the largest relative gap
    |lambda_b / lambda_(b-1)| with lambda_b at least 10x the noise floor and
    at most REFINE_MAX_FRACTION of the spectrum above it; whether the
    eigenpairs below it may keep FP32 accuracy is decided after the
    refinement, from their share of the update (bulk_weight).  Per power step
    the FP32 error of the refined vectors along the rest (~1e-7 lambda_max /
    gap) shrinks by rho = lambda_(b-1) / lambda_b; q steps take it to
    REFINE_TARGET, and a plan whose steps would grow the mixing inside the
    refined block by more than REFINE_MAX_GROWTH is refused.  vtf and snr
    are not used and kept for the interface."""
    n = ev.shape[0]
    a = np.abs(ev)
    lmax = a.max()
    if lmax == 0.0 or n < 2:
        return None
    noise = max(-float(ev.min()), 0.0) + 64 * 6e-8 * lmax
    lo = max(1, int(np.ceil((1.0 - REFINE_MAX_FRACTION) * n)))
    cand = np.arange(lo, n)
    cand = cand[a[cand] >= 10.0 * noise]
    if cand.size == 0:
        return None
    with np.errstate(divide="ignore", invalid="ignore"):
        ratio = a[cand] / np.maximum(a[cand - 1], noise)
    b = int(cand[int(np.argmax(ratio))])
    k = n - b
    rho = max(a[b - 1], noise) / a[b]
    if not rho < REFINE_MAX_RHO:
        return None
    gap = max(a[b] - a[b - 1], 1e-300)
    eps0 = min(1.0, 1e-7 * lmax / gap)
    # down to REFINE_TARGET: below the 2^-48 (3.6e-15) of the operand
    # scales to which the Ozaki products themselves are accurate
    q = int(min(max(np.ceil(np.log(REFINE_TARGET / eps0) / np.log(rho)), 1), 16))
    if q * np.log(lmax / a[b]) > np.log(REFINE_MAX_GROWTH):
        return None
    return k, q


def bulk_weight(ev, vtf, snr, k, pinvCutoff, snrTol):
    """Share of the update carried by the n - k eigenpairs left at FP32
    accuracy, from the values after the refinement (the bulk vectors are then
    orthogonal to the refined block, so their projections are free of its
    share); the solve falls back to the FP64 eigensolver above
    REFINE_EXCLUDED_NORM."""
    c = solve_weights(ev, vtf, snr, pinvCutoff, snrTol)
    tot = np.sqrt(np.sum(c * c))
    return float(np.sqrt(np.sum(c[:len(c) - k] ** 2)) / tot) if tot > 0 else 0.0


class TDVP:
    """Solver of the TDVP equation  q[S] theta_dot = -q[x F]  by regularised
    pseudo-inverse (tdvp.py:26-94).

    Initializer arguments as in the reference: ``sampler``, ``snrTol``,
    ``pinvTol``, ``pinvCutoff``, ``makeReal``, ``rhsPrefactor``,
    ``diagonalShift``, ``crossValidation``, ``diagonalizeOnDevice`` (must be
    True: there is no host path).  Additional:

        * ``precision``: arithmetic of the sampling, E_loc and S/F stages:
          ``"fp64"`` (the reference's), ``"fp32"`` (plain FP32 GPU form:
          FP32 kernels, FP32 complex GEMMs) or ``"mixed"`` (FP32 kernels,
          S and the SNR contraction in BF16 with hi/lo split correction and
          FP32 accumulation on tcgen05).  Means, variances and the solve are
          FP64 in every mode; the eigendecomposition is cuSOLVER's FP64 one,
          except in the mixed form with Monte Carlo samples, where the
          eigenpairs that carry the SNR-regularised solve are made
          FP64-accurate on the tensor cores from an FP32 eigendecomposition
          (util/tdvp.py refine_plan; the rest keep FP32 eigenvalues).
    """

    def __init__(self, sampler, snrTol=2, pinvTol=1e-14, pinvCutoff=1e-8, makeReal='imag', rhsPrefactor=1.j,
                 diagonalShift=0., crossValidation=False, diagonalizeOnDevice=True, precision="fp64"):
        if not diagonalizeOnDevice:
            raise NotImplementedError("diagonalisation runs on the GPU; there is no host path")
        if precision not in ("fp64", "fp32", "mixed"):
            raise ValueError("precision must be 'fp64', 'fp32' or 'mixed'")
        self.sampler = sampler
        self.snrTol = snrTol
        self.pinvTol = pinvTol
        self.pinvCutoff = pinvCutoff
        self.diagonalShift = diagonalShift
        self.rhsPrefactor = rhsPrefactor
        self.crossValidation = crossValidation
        self.diagonalizeOnDevice = True
        self.precision = precision
        self.metaData = None
        self.makeRealName = makeReal
        self.makeReal = imagFun if makeReal == 'imag' else realFun
        self.timings = {}
        # BF16 products of the mixed S build and SNR contraction: 3 (hi/lo
        # split correction) or 1 (plain BF16; accuracy studies)
        self.splitProducts = 3

    def set_diagonal_shift(self, delta):
        self.diagonalShift = delta

    def set_cross_validation(self, crossValidation=True):
        self.crossValidation = crossValidation

    def get_residuals(self):
        return self.metaData["tdvp_error"], self.metaData["tdvp_residual"]

    def get_snr(self):
        return self.metaData["SNR"]

    def get_spectrum(self):
        return self.metaData["spectrum"]

    def get_metadata(self):
        return self.metaData

    def get_energy_variance(self):
        return self.ElocVar0

    def get_energy_mean(self):
        return torch.real(self.ElocMean0) if isinstance(self.ElocMean0, torch.Tensor) else np.real(self.ElocMean0)

    def get_S(self):
        return self.S

    # ========================================== complex (holomorphic) path
    def _complex_capable(self, psi):
        """CpxRBM and SymNet(CpxRBM) states take the complex P x P pipeline;
        a real-parameter CNN takes it with makeReal='real' (S and F real)."""
        from ..nets.cnn import CNN
        from ..nets.rbm import CpxRBM
        from ..nets.sym_wrapper import SymNet
        if isinstance(psi.net, CNN):
            return self.makeRealName == 'real'
        return isinstance(psi.net, (CpxRBM, SymNet))

    def _rbm_capable(self, psi, hamiltonian):
        return self._complex_capable(psi)

    def _kernel_precision(self):
        return "fp64" if self.precision == "fp64" else "fp32"

    def _rbm_rhs(self, psi, configs, Eloc, p, weights=None):
        return self._complex_rhs(psi, configs, Eloc, p, weights)

    def _complex_rhs(self, psi, configs, Eloc, p, weights=None):
        """Everything after E_loc for a holomorphic state; returns the 2P
        update, the residual and the cutoff (device scalars)."""
        from .sr_data import producer
        dev = configs.device
        st = _lib.stream()
        status = self._status_word(dev)
        flat = configs.reshape(configs.shape[0] * configs.shape[1], -1)
        w = (p if weights is None else weights).reshape(-1).to(torch.float64).contiguous()
        E = Eloc.reshape(-1).to(torch.complex128).contiguous()
        TIMER.mark("statistics")
        data = producer(psi, flat, self._kernel_precision())
        N, P = data.N, data.P

        # E_loc statistics (stats.py:197-205, 248-252)
        emean = torch.empty(1, dtype=torch.complex128, device=dev)
        evar = torch.empty(1, dtype=torch.float64, device=dev)
        ws = _lib.Workspace.get(_lib.query("vmc_reduce_workspace_bytes", 2))
        _lib.call("vmc_weighted_mean_var", _lib.ptr(E), _lib.ptr(w), N, _lib.ptr(emean), _lib.ptr(evar),
                  _lib.ptr(ws), ws.numel(), st)
        # mean of O_k and covar(O, E) (stats.py:50-58 via tdvp.py:139)
        okMean = torch.empty(P, dtype=torch.complex128, device=dev)
        covOE = torch.empty(P, dtype=torch.complex128, device=dev)
        data.stats(w, E, emean, okMean, covOE)
        x = complex(self.rhsPrefactor)
        f = (-x) * covOE                       # complex form of F0 (tdvp.py:139)
        realParams = bool(getattr(data, "real", False))
        if realParams:                         # makeReal = Re (tdvp.py:140)
            f = torch.complex(f.real, torch.zeros_like(f.real))

        # S = <O^dagger O>_c  (tdvp.py:142)
        shift = float(self.diagonalShift) if (self.diagonalShift > 1e-10 and self.makeRealName != 'imag') else 0.0
        TIMER.mark("s_build")
        A = self._gram(data, w, okMean, shift, status)

        # eigendecomposition (tdvp.py:153-171) and SNR (tdvp.py:173-181)
        TIMER.mark("eigh")
        self.refineInfo = None
        useSnr = not isinstance(self.sampler, ExactSampler)
        if self._two_stage(realParams, useSnr, P):
            # the C ABI reads matrices column-major: the row-major storage of
            # conj(A) is A column-major (A Hermitian)
            Acm = torch.conj_physical(A)
            ev, U = self._eigh_fp32(Acm)
            plan = refine_plan(ev.cpu().numpy(), None, None, self.pinvCutoff, self.snrTol)
            weight, fallback = None, None if plan is not None else "no refinement plan"
            if plan is not None:
                TIMER.mark("eigh_refine")
                if not self._eigh_refine(Acm, ev, U, plan[0], plan[1], status):
                    plan, fallback = None, "Rayleigh-Ritz failed"
            if plan is not None:
                vtf = self._project(U, f)
                TIMER.mark("snr")
                snr = self._snr(data, w, okMean, E, emean, f, U, vtf, status)
                weight = bulk_weight(ev.cpu().numpy(), vtf.cpu().numpy(), snr.cpu().numpy(), plan[0],
                                     self.pinvCutoff, self.snrTol)
                if weight > REFINE_EXCLUDED_NORM:
                    plan, fallback = None, "bulk share"
            del Acm
            if plan is None:
                TIMER.mark("eigh")
                ev, U = _gram_mod().eigh_fp64(A)
                if U.stride(0) != 1:
                    U = U.mT.contiguous().mT
                vtf = self._project(U, f)
                TIMER.mark("snr")
                snr = self._snr(data, w, okMean, E, emean, f, U, vtf, status)
            self.refineInfo = {"refined": None if plan is None else plan[0],
                               "power_steps": None if plan is None else plan[1], "n": P,
                               "fp32_bulk_weight": weight, "fallback": fallback}
        else:
            if realParams:  # S real symmetric: the real eigensolver, vectors as complex
                ev, U = _gram_mod().eigh_fp64(A.real.contiguous())
                U = U.to(torch.complex128)
            else:
                ev, U = _gram_mod().eigh_fp64(A)
            if U.stride(0) != 1:
                U = U.mT.contiguous().mT
            vtf = self._project(U, f)
            TIMER.mark("snr")
            snr = self._snr(data, w, okMean, E, emean, f, U, vtf, status)

        # regularised pseudo-inverse (tdvp.py:183-213)
        TIMER.mark("solve")
        pinv = torch.empty(P, dtype=torch.float64, device=dev)
        res = torch.empty(3, dtype=torch.float64, device=dev)
        ws = _lib.Workspace.get(_lib.query("vmc_tdvp_regularize_workspace_bytes", P, float(self.pinvCutoff)))
        _lib.call("vmc_tdvp_regularize", _lib.ptr(ev), _lib.ptr(vtf), _lib.ptr(snr) if useSnr else None, P,
                  float(self.pinvCutoff), float(self.pinvTol), float(self.snrTol), _lib.ptr(pinv), _lib.ptr(res),
                  _lib.ptr(ws), ws.numel(), st)
        coef = (pinv.to(torch.complex128) * vtf).contiguous()
        z = torch.empty(P, dtype=torch.complex128, device=dev)
        ws = _lib.Workspace.get(_lib.query("vmc_zgemv_workspace_bytes", P))
        _lib.call("vmc_zgemv", 0, _lib.ptr(U), U.stride(1), P, _lib.ptr(coef), _lib.ptr(z), _lib.ptr(ws), ws.numel(),
                  st)

        self._check_status(status)

        # bookkeeping in the reference's 2P layout
        self._A, self._shift, self._z, self._covOE = A, shift, z, covOE
        self._leafSizes = [int(q.numel()) for q in psi.params.values()]
        self._complexLast = True
        self._realParams = realParams
        self.ev_c, self.V, self.VtF, self.snr_c = ev, U, vtf, snr
        self.ElocMean = emean[0]
        self.ElocVar = evar[0]
        if realParams:
            return z.real.contiguous(), res[0], res[1]
        return self._realrep(psi, z), res[0], res[1]

    # ------------------------------------------- eigendecomposition stages
    TWO_STAGE_MIN_P = 2048

    def _two_stage(self, realParams, useSnr, P):
        """The mixed form with Monte Carlo samples solves through the two-stage
        eigensolver (FP32 eigendecomposition, then the eigenpairs that carry
        the SNR-regularised solve refined to FP64 accuracy on the tensor
        cores); every other case through the FP64 cuSOLVER eigensolver."""
        return self.precision == "mixed" and useSnr and not realParams and P >= self.TWO_STAGE_MIN_P

    def _project(self, U, f):
        """U^H f (FP64, fixed-order reduction)."""
        P = U.shape[0]
        vtf = torch.empty(P, dtype=torch.complex128, device=U.device)
        ws = _lib.Workspace.get(_lib.query("vmc_zgemv_workspace_bytes", P))
        _lib.call("vmc_zgemv", 1, _lib.ptr(U), U.stride(1), P, _lib.ptr(f), _lib.ptr(vtf), _lib.ptr(ws), ws.numel(),
                  _lib.stream())
        return vtf

    def _eigh_fp32(self, A):
        """Stage 1: complex64 eigendecomposition of A (given column-major),
        widened (vmc_eigh_fp32)."""
        P = A.shape[0]
        dev = A.device
        ev = torch.empty(P, dtype=torch.float64, device=dev)
        U = torch.empty((P, P), dtype=torch.complex128, device=dev).mT  # column-major
        info = torch.zeros(1, dtype=torch.int32, device=dev)
        ws = _lib.Workspace.get(_lib.query("vmc_eigh_fp32_workspace_bytes", P))
        _lib.call("vmc_eigh_fp32", P, _lib.ptr(A), A.stride(0), _lib.ptr(ev), _lib.ptr(U), U.stride(1),
                  _lib.ptr(ws), ws.numel(), _lib.ptr(info), _lib.stream())
        if int(info.item()) != 0:
            raise _lib.VmcError("TDVP: the FP32 eigensolver did not converge (info %d)" % int(info.item()))
        return ev, U

    def _eigh_refine(self, A, ev, U, k, steps, status):
        """Stage 2: the top k eigenpairs FP64-accurate (vmc_eigh_refine_top);
        A given column-major.  False when the Rayleigh-Ritz step failed."""
        P = A.shape[0]
        info = torch.zeros(1, dtype=torch.int32, device=A.device)
        ws = _lib.Workspace.get(_lib.query("vmc_eigh_refine_workspace_bytes", P, k))
        _lib.call("vmc_eigh_refine_top", P, _lib.ptr(A), A.stride(0), k, steps, _lib.ptr(ev), _lib.ptr(U),
                  U.stride(1), _lib.ptr(ws), ws.numel(), _lib.ptr(status), _lib.ptr(info), _lib.stream())
        # info != 0: the k x k generalized eigensolver found X^H X not
        # positive definite or did not converge; the caller then falls back
        # to the FP64 eigensolver of the whole matrix
        return int(info.item()) == 0

    def _status_word(self, dev):
        """Device int32 that a tensor-core kernel of this solver sets when one
        of its bounded waits runs out; zeroed at the start of every RHS."""
        word = getattr(self, "_status", None)
        if word is None or word.device != dev:
            word = torch.zeros(1, dtype=torch.int32, device=dev)
            self._status = word
        else:
            word.zero_()
        return word

    def _check_status(self, word):
        code = int(word.item())
        if code:
            raise _lib.VmcError("TDVP: a tensor-core kernel gave up waiting (code %d); its output is incomplete"
                                % code)

    def S_dot(self, v):
        """S0 v (tdvp.py:215-216) for a flat real vector v in the
        get_parameters layout, S0 = covar(O) of the reference's 2P layout.
        After the complex path, S0 = [[A, iA], [-iA, A]] per leaf with
        A = <O^dagger O>_c, so S0 [a; b] = [A z; -i A z] with z = a + i b
        (A taken without the diagonal shift, as S0 is)."""
        if not getattr(self, "_complexLast", False):
            return torch.matmul(self.S0, torch.as_tensor(v, device=self.S0.device).to(self.S0.dtype))
        v = torch.as_tensor(v, device=self._A.device).to(torch.float64)
        if self._realParams:
            z = v.to(torch.complex128)
            y = torch.mv(self._A, z)
            if self._shift:
                y = y - (self._shift / (1.0 + self._shift)) * self._A.diagonal() * z
            return y
        zs, start = [], 0
        for n in self._leafSizes:
            zs.append(torch.complex(v[start:start + n], v[start + n:start + 2 * n]))
            start += 2 * n
        z = torch.cat(zs)
        y = torch.mv(self._A, z)
        if self._shift:
            y = y - (self._shift / (1.0 + self._shift)) * self._A.diagonal() * z
        out, start = [], 0
        for n in self._leafSizes:
            yy = y[start:start + n]
            out += [yy, -1j * yy]
            start += n
        return torch.cat(out)

    def get_sr_equation(self, Eloc, gradients):
        """The TDVP equation with rhsPrefactor 1 (tdvp.py:150-151)."""
        saved = self.rhsPrefactor
        self.rhsPrefactor = 1.
        try:
            return self.get_tdvp_equation(Eloc, gradients)
        finally:
            self.rhsPrefactor = saved

    def _realrep(self, psi, z):
        """[Re z_leaf; Im z_leaf] per leaf (get_parameters layout, vqs.py:461-462)."""
        parts = []
        start = 0
        for name, p in psi.params.items():
            n = p.numel()
            zz = z[start:start + n]
            parts += [zz.real, zz.imag]
            start += n
        return torch.cat(parts)

    def _gram(self, data, w, okMean, shift, status=None):
        if self.precision == "mixed":
            from . import gram as _gram
            return _gram.mixed_hermitian(data, w, okMean, shift, status, self.splitProducts)
        from . import gram as _gram
        fmt, dt = (0, torch.complex128) if self.precision == "fp64" else (1, torch.complex64)
        X = torch.empty((data.N, data.P), dtype=dt, device=data.device)
        data.centered(w, okMean, fmt, X, None, data.P)
        N, P = data.N, data.P
        if self.precision == "fp64" and P >= _gram.OZAKI_MIN_DIM and N <= _gram.OZAKI_MAX_K:
            # X row-major (N x P) is M = X^T column-major; M M^H = conj(A),
            # whose column-major storage read row-major is A
            A = _gram.fp64_product("N", X, P, "C", X, P, P, P, N, hermitian=True, status=status)
        else:
            A = torch.matmul(X.mH, X).to(torch.complex128)
        del X
        if shift:
            A.diagonal().mul_(1.0 + shift)
        return A

    def _snr(self, data, w, okMean, E, emean, f, U, vtf, status=None):
        dev = data.device
        st = _lib.stream()
        x = complex(self.rhsPrefactor)
        P = data.P
        snr = torch.empty(P, dtype=torch.float64, device=dev)
        if self.precision == "mixed":
            from . import gram as _gram
            colsq = _gram.mixed_snr_colsq(data, w, okMean, E, emean, f, U, x, status, self.splitProducts)
            realRep, cprec = 1, _lib.VMC_F32
        else:
            from . import gram as _gram
            fmt, dt = (0, torch.complex128) if self.precision == "fp64" else (1, torch.complex64)
            H = torch.empty((data.N, P), dtype=dt, device=dev)
            data.snr_data(w, okMean, E, emean, -x, f, fmt, H, None, P)
            if self.precision == "fp64" and P >= _gram.OZAKI_MIN_DIM and P <= _gram.OZAKI_MAX_K and U.stride(0) == 1:
                # Y^T = U^H H^T (P x N column-major) is Y (N x P) row-major
                Y = _gram.fp64_product("C", U, U.stride(1), "N", H, P, P, data.N, P, status=status)
            else:
                Y = torch.matmul(H, torch.conj(U).to(dt))
            del H
            colsq = (Y.real ** 2 + Y.imag ** 2).sum(0).to(torch.float64).contiguous()
            del Y
            realRep, cprec = 0, _lib.VMC_F64
        self.rhoVar_c = torch.empty(P, dtype=torch.float64, device=dev)
        _lib.call("vmc_tdvp_snr", _lib.ptr(vtf), cprec, _lib.ptr(colsq), P, realRep, float(self._num_samples()),
                  _lib.ptr(snr), _lib.ptr(self.rhoVar_c), st)
        return snr

    def _num_samples(self):
        """The global sample count of the last sampling call (mpi.globNumSamples,
        tdvp.py:179), taken from this solver's sampler so that solvers of
        different jobs can run concurrently."""
        n = getattr(self.sampler, "globNumSamples", None)
        if isinstance(self.sampler, ExactSampler) or not n:
            return mpi.globNumSamples
        return n

    def _rbm_metadata(self, psi, update, residual, cutoff):
        """tdvp_error (tdvp.py:102-104) and the 2P spectrum / SNR."""
        z, A, shift = self._z, self._A, self._shift
        Az = torch.mv(A, z)
        if shift:
            Az = Az - (shift / (1.0 + shift)) * A.diagonal() * z
        zAz = torch.real(torch.vdot(z, Az))
        x = complex(self.rhsPrefactor)
        zF = torch.vdot(z, (-x) * self._covOE)
        err = torch.abs(1. + (zAz - 2. * torch.real(zF)) / self.ElocVar0)
        if self._realParams:
            spectrum, snr = self.ev_c, self.snr_c
        elif self.makeRealName == 'imag':
            spectrum = torch.cat([-torch.flip(self.ev_c, [0]), self.ev_c])
            snr = torch.cat([torch.flip(self.snr_c, [0]), self.snr_c])
        else:
            spectrum = torch.repeat_interleave(self.ev_c, 2)
            snr = torch.repeat_interleave(self.snr_c, 2)
        self.ev = spectrum
        self.snr = snr
        return {"tdvp_error": err, "tdvp_residual": residual, "pinv_cutoff": cutoff, "SNR": snr,
                "spectrum": spectrum}

    # ===================================================== generic path
    def get_tdvp_equation(self, Eloc, gradients):
        """tdvp.py:134-148 on SampledObs inputs."""
        self._complexLast = False
        self.ElocMean = Eloc.mean()[0]
        self.ElocVar = Eloc.var()[0]
        self.F0 = (-self.rhsPrefactor) * gradients.covar(Eloc).reshape(-1)
        F = self.makeReal(self.F0)
        self.S0 = gradients.covar()
        S = self.makeReal(self.S0)
        if self.diagonalShift > 1e-10:
            S = S + torch.diag(self.diagonalShift * torch.diag(S))
        return S, F

    def _transform_to_eigenbasis(self, S, F):
        self.ev, self.V = _gram_mod().eigh_fp64(S.contiguous())
        self.VtF = torch.matmul(torch.conj(self.V).T, F.to(self.V.dtype))

    def _get_snr(self, Eloc, gradients):
        EO = gradients.covar_data(Eloc).transform(linearFun=torch.conj(self.V).T,
                                                  nonLinearFun=lambda v: transform_helper(v, self.rhsPrefactor,
                                                                                          self.makeReal))
        self.rhoVar = EO.var().reshape(-1)
        self.snr = torch.sqrt(torch.abs(mpi.globNumSamples * (torch.conj(self.VtF) * self.VtF) / self.rhoVar)).reshape(-1)

    def solve(self, Eloc, gradients):
        """TDVP.solve (tdvp.py:183-213) for SampledObs inputs, in the 2P
        representation (FP64, GPU)."""
        self.S, F = self.get_tdvp_equation(Eloc, gradients)
        self._transform_to_eigenbasis(self.S, F)
        self._get_snr(Eloc, gradients)
        ev = torch.real(self.ev) if self.ev.is_complex() else self.ev
        self.invEv = torch.where(torch.abs(ev / ev[-1]) > 1e-14, 1. / ev, torch.zeros_like(ev))
        residual = 1.0
        cutoff = 1e-2
        F_norm = torch.linalg.norm(F)
        while residual > self.pinvTol and cutoff > self.pinvCutoff:
            cutoff *= 0.8
            regularizer = 1. / (1. + (max(cutoff, self.pinvCutoff) / torch.abs(ev / ev[-1])) ** 6)
            if not isinstance(self.sampler, ExactSampler):
                regularizer = regularizer * (1. / (1. + (self.snrTol / torch.real(self.snr)) ** 6))
            pinvEv = self.invEv * regularizer
            residual = float(torch.linalg.norm((pinvEv * ev - torch.ones_like(pinvEv)) * self.VtF) / F_norm)
        update = torch.real(torch.matmul(self.V, (pinvEv.to(self.VtF.dtype) * self.VtF)))
        return update, residual, max(cutoff, self.pinvCutoff)

    def _get_tdvp_error(self, update):
        """tdvp.py:102-104."""
        u = update.to(self.S0.dtype)
        return torch.abs(1. + torch.real(u.dot(self.S0.matmul(u)) - 2. * torch.real(u.dot(self.F0.to(u.dtype))))
                         / self.ElocVar0)

    # ========================================================== RHS
    def __call__(self, netParameters, t, *, psi, hamiltonian, **rhsArgs):
        """theta_dot = S^-1 F for the given parameters (tdvp.py:219-326)."""
        tmpParameters = psi.get_parameters()
        psi.set_parameters(netParameters)
        numSamples = rhsArgs.get("numSamples", None)
        outp = rhsArgs.get("outp", None)
        TIMER.mark("sampling")
        configs, sampleLogPsi, p = self.sampler.sample(numSamples=numSamples)
        fused = self._complex_capable(psi)
        if fused:
            TIMER.mark("eloc")
            if hasattr(hamiltonian, "fused_capable") and hamiltonian.fused_capable(psi):
                Eloc = hamiltonian.get_O_loc_fused(configs, psi, None, t)
            else:
                Eloc = hamiltonian.get_O_loc(configs, psi, sampleLogPsi, t)
            update, residual, cutoff = self._complex_rhs(psi, configs, Eloc, p)
            TIMER.mark("rhs_end")
        else:
            TIMER.mark("eloc")
            Eloc = hamiltonian.get_O_loc(configs, psi, sampleLogPsi, t)
            EObs = SampledObs(Eloc, p)
            TIMER.mark("gradients")
            gObs = SampledObs(psi.gradients(configs), p)
            TIMER.mark("solve")
            update, residual, cutoff = self.solve(EObs, gObs)
            TIMER.mark("rhs_end")
        psi.set_parameters(tmpParameters)
        if rhsArgs.get("intStep", None) == 0:
            self.ElocMean0 = self.ElocMean
            self.ElocVar0 = self.ElocVar
            if fused:
                self.metaData = self._rbm_metadata(psi, update, residual, cutoff)
                if self.crossValidation:
                    self._cross_validate_rbm(psi, configs, Eloc, p, update, residual)
            else:
                self.metaData = {"tdvp_error": self._get_tdvp_error(update), "tdvp_residual": residual,
                                 "pinv_cutoff": cutoff, "SNR": self.snr, "spectrum": self.ev}
                if self.crossValidation:
                    raise NotImplementedError("cross-validation is implemented for the fused CpxRBM path")
        return update

    def _cross_validate_rbm(self, psi, configs, Eloc, p, update, residual):
        """Cross-validation of tdvp.py:230-248: solve on the even samples,
        check on the odd ones.  A subset is the same sample with the other
        half's weights set to 0 and the rest renormalised (stats.py:310-329)."""
        w = p.reshape(-1)
        idx = torch.arange(w.numel(), device=w.device)
        w1 = torch.where(idx % 2 == 0, w, torch.zeros_like(w))
        w2 = torch.where(idx % 2 == 1, w, torch.zeros_like(w))
        w1 = w1 / w1.sum()
        w2 = w2 / w2.sum()
        saved = (self._A, self._shift, self._z, self._covOE, self.ev_c, self.V, self.VtF, self.snr_c,
                 self.ElocMean, self.ElocVar)
        update1, _, _ = self._complex_rhs(psi, configs, Eloc, p, weights=w1)
        z1 = self._z
        # tdvp error of update_1 against the full-sample S0, F0 and ElocVar0
        (self._A, self._shift, self._z, self._covOE) = saved[:4]
        Az1 = torch.mv(self._A, z1)
        if self._shift:
            Az1 = Az1 - (self._shift / (1.0 + self._shift)) * self._A.diagonal() * z1
        x = complex(self.rhsPrefactor)
        err1 = torch.abs(1. + (torch.real(torch.vdot(z1, Az1)) - 2. * torch.real(torch.vdot(z1, (-x) * self._covOE)))
                         / self.ElocVar0)
        # residual of update_1 on the odd half: ||S2 u1 - F2|| / ||F2||
        self._complex_rhs(psi, configs, Eloc, p, weights=w2)
        A2, z2shift, cov2 = self._A, self._shift, self._covOE
        r = torch.mv(A2, z1) - (-x) * cov2
        valRes = (torch.linalg.norm(r) / torch.linalg.norm((-x) * cov2)) / residual
        (self._A, self._shift, self._z, self._covOE, self.ev_c, self.V, self.VtF, self.snr_c,
         self.ElocMean, self.ElocVar) = saved
        self.crossValidationFactor_residual = valRes
        self.crossValidationFactor_tdvpErr = err1 / self.metaData["tdvp_error"]
        self.metaData["tdvp_residual_cross_validation_ratio"] = self.crossValidationFactor_residual
        self.metaData["tdvp_error_cross_validation_ratio"] = self.crossValidationFactor_tdvpErr
