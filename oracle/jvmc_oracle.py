"""CPU FP64 restatement of jVMC 1.5.8's per-step VMC hot path.

TEST INFRASTRUCTURE ONLY.  This module is the oracle that the CUDA path is
checked against.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU
baseline legs of ``bench.py`` may import it; the product package
``vmc_jax_gb300`` never does.

jVMC itself (JAX/Flax) cannot be imported in this environment, so every
function below restates the reference algorithm in numpy (float64 /
complex128) and cites the reference file:line it follows (paths relative to
the jVMC project root).  The restatement is pinned against the numeric
fixtures of the reference's own test-suite (``tests/golden``).

Not restated: JAX's PRNG (threefry) stream and Flax's default initialisers.
The Metropolis restatement instead consumes the counter-based Philox4x32-10
stream defined in :func:`philox4x32` so that the CUDA sampler can be checked
bit-exactly for the same random numbers; the reference's own random stream
is unpinned.
"""

import functools
import math

import numpy as np

tCpx = np.complex128
tReal = np.float64


# ---------------------------------------------------------------------------
# Activation functions  (jVMC/nets/activation_functions.py)
# ---------------------------------------------------------------------------

def log_cosh(x):
    """Stable complex log(cosh(x)); activation_functions.py:19-22."""
    x = np.asarray(x)
    sgn = -2 * np.signbit(x.real) + 1
    x = x * sgn
    return x + np.log1p(np.exp(-2.0 * x)) - np.log(2.0)


def poly6(x):
    """activation_functions.py:10-12."""
    x = x ** 2
    return ((0.022222222 * x - 0.083333333) * x + 0.5) * x


def poly5(x):
    """activation_functions.py:15-17."""
    xsq = x ** 2
    return ((0.133333333 * xsq - 0.333333333) * xsq + 1.) * x


def poly4(x):
    """x^2/2 - x^4/12: the two leading Taylor terms of log(cosh(x)).

    This is the CNN activation of the 10x10 transverse-field Ising workload;
    it is passed to jVMC's CNN as a user ``actFun`` (cnn.py:35,57-59)."""
    x2 = x * x
    return 0.5 * x2 - x2 * x2 / 12.0


def poly4_deriv(x):
    return x - x * x * x / 3.0


def poly6_deriv(x):
    x2 = x * x
    return ((6 * 0.022222222 * x2 - 4 * 0.083333333) * x2 + 2 * 0.5) * x


def square(x):
    return x ** 2


ACTIVATIONS = {"poly4": (poly4, poly4_deriv), "poly6": (poly6, poly6_deriv),
               "square": (square, lambda x: 2 * x)}


# ---------------------------------------------------------------------------
# Networks
# ---------------------------------------------------------------------------

class CpxRBM:
    """Complex RBM  log psi(s) = sum_j logcosh(sum_i W_ij (2 s_i - 1) + b_j).

    rbm.py:17-38.  Parameters are held as a dict in Flax leaf order
    (``bias`` before ``kernel``; kernel shape (L, M), Dense computes x @ W + b).
    """

    holomorphic = True
    realParams = False

    def __init__(self, numHidden=2, bias=False):
        self.numHidden = numHidden
        self.bias = bias

    def leaf_shapes(self, L):
        shapes = []
        if self.bias:
            shapes.append(("bias", (self.numHidden,)))
        shapes.append(("kernel", (L, self.numHidden)))
        return shapes

    def theta(self, params, s):
        s = np.asarray(s).reshape(s.shape[0], -1)
        x = (2 * s - 1).astype(np.float64)
        th = x @ params["kernel"]
        if self.bias:
            th = th + params["bias"]
        return th

    def apply(self, params, s):
        return log_cosh(self.theta(params, s)).sum(-1)

    def grad(self, params, s):
        """Per-sample d log psi / d theta for each leaf (holomorphic)."""
        s = np.asarray(s).reshape(s.shape[0], -1)
        t = np.tanh(self.theta(params, s))
        x = (2 * s - 1).astype(np.float64)
        out = {}
        if self.bias:
            out["bias"] = t
        out["kernel"] = (x[:, :, None] * t[:, None, :]).reshape(s.shape[0], -1)
        return out


class CNN:
    """Real CNN with periodic padding; cnn.py:18-83.

    ``x -> 2x-1``; per layer: wrap-pad (0, F-1) on every spatial axis,
    VALID cross-correlation with HWIO kernel, optional bias (never on the
    first layer unless ``firstLayerBias``), activation.  Output is
    ``sum(x) / sqrt(prod(x.shape))`` over (1, *spatial, C).
    """

    holomorphic = False
    realParams = True

    def __init__(self, F=(8,), channels=(10,), strides=(1,), actFun=("poly4",),
                 bias=True, firstLayerBias=False, periodicBoundary=True):
        self.F = tuple(F)
        self.channels = tuple(channels)
        self.strides = tuple(strides)
        if any(s != 1 for s in self.strides):
            raise NotImplementedError("only unit strides are restated")
        if not periodicBoundary:
            raise NotImplementedError("only periodic boundaries are restated")
        acts = list(actFun)
        while len(acts) < len(self.channels):
            acts.append(acts[-1])
        self.actFun = acts
        self.bias = bias
        self.firstLayerBias = firstLayerBias

    def layer_bias(self, l):
        return self.firstLayerBias if l == 0 else self.bias

    def leaf_shapes(self, sampleShape):
        shapes = []
        cin = 1
        for l, c in enumerate(self.channels):
            if self.layer_bias(l):
                shapes.append((f"Conv_{l}/bias", (c,)))
            shapes.append((f"Conv_{l}/kernel", self.F + (cin, c)))
            cin = c
        return shapes

    def _conv(self, x, K, b):
        # x: (N, *sp, Cin) ; K: (*F, Cin, Cout) ; periodic cross-correlation
        nd = len(self.F)
        out = 0.0
        for off in np.ndindex(*self.F):
            xs = x
            for ax, o in enumerate(off):
                xs = np.roll(xs, -o, axis=1 + ax)
            out = out + xs @ K[off]
        if b is not None:
            out = out + b
        return out

    def forward(self, params, s, keep=False):
        s = np.asarray(s)
        x = (2 * s - 1).astype(np.float64)[..., None]
        pre = []
        ins = []
        for l, c in enumerate(self.channels):
            K = params[f"Conv_{l}/kernel"]
            b = params.get(f"Conv_{l}/bias") if self.layer_bias(l) else None
            ins.append(x)
            z = self._conv(x, K, b)
            pre.append(z)
            x = ACTIVATIONS[self.actFun[l]][0](z)
        nrm = math.sqrt(float(np.prod(x.shape[1:])))
        out = x.reshape(x.shape[0], -1).sum(-1) / nrm
        if keep:
            return out, pre, ins, nrm
        return out

    def apply(self, params, s):
        return self.forward(params, s).astype(np.float64)

    def grad(self, params, s):
        out, pre, ins, nrm = self.forward(params, s, keep=True)
        N = out.shape[0]
        nd = len(self.F)
        g = {}
        dx = np.full(pre[-1].shape, 1.0 / nrm)
        for l in reversed(range(len(self.channels))):
            dz = dx * ACTIVATIONS[self.actFun[l]][1](pre[l])
            if self.layer_bias(l):
                g[f"Conv_{l}/bias"] = dz.reshape(N, -1, dz.shape[-1]).sum(1)
            K = params[f"Conv_{l}/kernel"]
            gK = np.zeros((N,) + K.shape)
            dxin = np.zeros(ins[l].shape)
            for off in np.ndindex(*self.F):
                xs = ins[l]
                for ax, o in enumerate(off):
                    xs = np.roll(xs, -o, axis=1 + ax)
                # out[p, co] += xs[p, ci] K[off, ci, co]
                gK[(slice(None),) + off] = np.einsum(
                    "npi,npo->nio", xs.reshape(N, -1, xs.shape[-1]), dz.reshape(N, -1, dz.shape[-1]))
                contrib = dz @ K[off].T
                for ax, o in enumerate(off):
                    contrib = np.roll(contrib, o, axis=1 + ax)
                dxin += contrib
            g[f"Conv_{l}/kernel"] = gK.reshape(N, -1)
            dx = dxin
        return g


class LookupNet:
    """Table wave function used by the reference's fermion test
    (operator_test.py Target, lines 17-38): log|k[idx]| + i angle(k[idx]),
    idx = sum_l d^l s[L-1-l]."""

    holomorphic = False
    realParams = False

    def __init__(self, L, d=2, delta=1e-15):
        self.L, self.d, self.delta = L, d, delta

    def apply(self, params, s):
        s = np.asarray(s).reshape(s.shape[0], -1)
        idx = (s[:, ::-1] * (self.d ** np.arange(self.L))).sum(-1).astype(int)
        k = params["kernel"][idx]
        return np.log(np.abs(k + self.delta)) + 1.j * np.angle(k)


# ---------------------------------------------------------------------------
# Variational state (jVMC/vqs.py)
# ---------------------------------------------------------------------------

# ---------------------------------------------------------------------------
# Lattice symmetries and the symmetrised network
# (jVMC/util/symmetries.py, jVMC/nets/sym_wrapper.py)
# ---------------------------------------------------------------------------

def _perm_matrix(maps_row, idx):
    o = np.zeros((idx.size, idx.size), dtype=np.int32)
    o[idx.ravel(), maps_row.ravel()] = 1
    return o


def _unique_orbit(orbits, factors, n):
    """np.unique over the flattened matrices (rows sorted lexicographically)
    with the factor of each first occurrence (symmetries.py:142-144, 207-209)."""
    uo, ind = np.unique(orbits.reshape((-1, n * n)), return_index=True, axis=0)
    return uo.reshape(-1, n, n), np.asarray(factors)[ind]


def get_orbit_1D(L, *args, translation_factor=1., reflection_factor=1., spinflip_factor=1.):
    """symmetries.py:146-212: orbit matrices (|S|, L, L) and factors."""
    idx = np.arange(L)
    refl = {"maps": [idx], "factor": [1.]}
    trans = {"maps": [idx], "factor": [1.]}
    if "reflection" in args:
        refl["maps"].append(idx[::-1])
        refl["factor"].append(reflection_factor)
    if "translation" in args:
        for x in range(1, L):
            trans["maps"].append(np.roll(idx, x, axis=(0,)))
            trans["factor"].append(translation_factor ** x)
    orbits, factors = [], []
    for mt, ft in zip(trans["maps"], trans["factor"]):
        for mr, fr in zip(refl["maps"], refl["factor"]):
            orbits.append(_perm_matrix(mt, idx) @ _perm_matrix(mr, idx))
            factors.append(ft * fr)
    orbits = np.array(orbits)
    factors = np.array(factors)
    if "spinflip" in args:
        orbits = np.concatenate([orbits, -orbits], axis=0)
        factors = np.concatenate([factors, spinflip_factor * factors])
    return _unique_orbit(orbits, factors, L)


def get_orbit_2D_square(L, *args, translation_factor=1., reflection_factor=1., rotation_factor=1.,
                        spinflip_factor=1.):
    """symmetries.py:51-148: orbit matrices (|S|, L^2, L^2) and factors."""
    idx = np.arange(L ** 2).reshape((L, L))
    rot = {"maps": [idx], "factor": [1.]}
    refl = {"maps": [idx], "factor": [1.]}
    trans = {"maps": [idx], "factor": [1.]}
    if "rotation" in args:
        rot["maps"] += [idx[::-1, :].T, idx[::-1, ::-1], idx[:, ::-1].T]
        rot["factor"] += [rotation_factor, rotation_factor ** 2, rotation_factor ** 3]
    if "reflection" in args:
        refl["maps"] += [idx[::-1, :], idx[:, ::-1], idx[::-1, ::-1]]
        refl["factor"] += [reflection_factor, reflection_factor, reflection_factor ** 2]
    if "translation" in args:
        for x in range(L):
            for y in range(L):
                if x == 0 and y == 0:
                    continue
                trans["maps"].append(np.roll(idx, (y, x), axis=(0, 1)))
                trans["factor"].append(translation_factor ** (x + y))
    # symmetries.py:134 passes (translation, reflection, rotation) into the
    # parameters (translation, rotation, reflection) of
    # get_orbits_from_maps_2D (51-75), whose loops then run over translation,
    # rotation, reflection and form T @ Rot @ Refl
    orbits, factors = [], []
    for mt, ft in zip(trans["maps"], trans["factor"]):
        for mo, fo in zip(rot["maps"], rot["factor"]):
            for mr, fr in zip(refl["maps"], refl["factor"]):
                orbits.append(_perm_matrix(mt, idx) @ _perm_matrix(mo, idx) @ _perm_matrix(mr, idx))
                factors.append(ft * fo * fr)
    orbits = np.array(orbits)
    factors = np.array(factors)
    if "spinflip" in args:
        orbits = np.concatenate([orbits, -orbits], axis=0)
        factors = np.concatenate([factors, spinflip_factor * factors])
    return _unique_orbit(orbits, factors, L ** 2)


def avgFun_Coefficients_Exp(coeffs, factor):
    """sym_wrapper.py:7-9: logsumexp(coeffs, b=factor) along axis 0 in the
    form of jax.scipy.special.logsumexp for complex input: terms with
    factor 0 are dropped, the maximum real part is taken out, and the result
    is the principal complex log of the scaled sum plus that maximum."""
    b = np.asarray(factor).reshape((-1,) + (1,) * (coeffs.ndim - 1))
    a = np.where(b != 0, coeffs, -np.inf)
    amax = np.max(np.real(a), axis=0)
    amax = np.where(np.isfinite(amax), amax, 0.0)
    s = np.sum(np.exp(a - amax) * b, axis=0)
    return np.log(s.astype(tCpx)) + amax


def avgFun_Coefficients_Log(coeffs, factor):
    """sym_wrapper.py:12-13: mean of the log-coefficients (factor unused)."""
    return np.mean(coeffs, axis=0)


class SymNet:
    """sym_wrapper.py:22-64: log psi_sym(s) = avgFun_tau(log psi(tau(s)), factor)
    with tau(s) = (o_tau (2s - 1) + 1) // 2.  The gradient of the holomorphic
    average is the weighted mean of the per-element gradients, with weights
    factor_tau exp(log psi(tau s) - log psi_sym(s)) (Exp) or 1/|S| (Log)."""

    def __init__(self, net, orbit, factor, avgFun=avgFun_Coefficients_Exp):
        self.net = net
        self.orbit = np.asarray(orbit)
        self.factor = np.asarray(factor)
        self.avgFun = avgFun
        self.holomorphic = net.holomorphic
        self.realParams = net.realParams

    def leaf_shapes(self, L):
        return self.net.leaf_shapes(L)

    def transformed(self, s):
        """(|S|, N, L) configurations tau(s) (sym_wrapper.py:51-54)."""
        s = np.asarray(s).reshape(np.asarray(s).shape[0], -1)
        x = 2 * s - 1
        y = np.einsum("tij,nj->tni", self.orbit, x)
        return (y + 1) // 2

    def _per_element(self, params, s):
        ts = self.transformed(s)
        S, N, L = ts.shape
        return ts, self.net.apply(params, ts.reshape(S * N, L)).reshape(S, N).astype(tCpx)

    def apply(self, params, s):
        _, lp = self._per_element(params, s)
        return self.avgFun(lp, self.factor)

    def grad(self, params, s):
        ts, lp = self._per_element(params, s)
        S, N, L = ts.shape
        if self.avgFun is avgFun_Coefficients_Log:
            w = np.full((S, N), 1.0 / S, dtype=tCpx)
        else:
            lsym = self.apply(params, s)
            w = self.factor.reshape(S, 1) * np.exp(lp - lsym[None, :])
        g = self.net.grad(params, ts.reshape(S * N, L))
        return {k: np.einsum("tn,tnk->nk", w, v.reshape(S, N, -1)) for k, v in g.items()}


class NQS:
    """Restatement of vqs.py:115-466 for the nets above.

    ``params`` is an ordered dict of leaves in Flax flatten order."""

    def __init__(self, net, params):
        self.net = net
        self.params = dict(params)
        self.holomorphic = net.holomorphic
        self.realParams = net.realParams

    def __call__(self, s):
        # vqs.py:223-251 (batching does not change values)
        s = np.asarray(s)
        return self.net.apply(self.params, s.reshape((-1,) + s.shape[2:])).reshape(s.shape[:2]).astype(tCpx)

    def gradients(self, s):
        """vqs.py:256-287 with flat_gradient_holo (66-69) for holomorphic
        nets and flat_gradient (46-51) for real-parameter nets."""
        s = np.asarray(s)
        flat = s.reshape((-1,) + s.shape[2:])
        g = self.net.grad(self.params, flat)
        parts = []
        for k in self.params:
            gk = g[k].reshape(flat.shape[0], -1)
            if self.holomorphic:
                parts += [gk, 1.j * gk]
            else:
                parts += [gk.astype(tCpx)]
        G = np.concatenate(parts, axis=1)
        return G.reshape(s.shape[:2] + (G.shape[-1],))

    def get_parameters(self):
        """vqs.py:449-466: [Re(leaf); Im(leaf)] per leaf (complex params)."""
        if self.realParams:
            return np.concatenate([p.ravel() for p in self.params.values()]).astype(tReal)
        return np.concatenate([np.concatenate([p.ravel().real, p.ravel().imag])
                               for p in self.params.values()])

    def set_parameters(self, P):
        """vqs.py:409-444 (_param_unflatten)."""
        P = np.asarray(P)
        start = 0
        for k, p in self.params.items():
            n = p.size
            if self.realParams:
                self.params[k] = P[start:start + n].reshape(p.shape).astype(tReal)
                start += n
            else:
                self.params[k] = (P[start:start + n] + 1.j * P[start + n:start + 2 * n]).reshape(p.shape)
                start += 2 * n

    @property
    def numParameters(self):
        return sum(p.size for p in self.params.values())


def init_cpx_rbm(L, M, bias, rng, scale=0.01, dist="normal"):
    """Seeded parameters for a CpxRBM in Flax leaf order."""
    params = {}
    if bias:
        if dist == "normal":
            params["bias"] = rng.normal(0, scale, M) + 1.j * rng.normal(0, scale, M)
        else:
            params["bias"] = np.zeros(M, dtype=tCpx)
    if dist == "normal":
        params["kernel"] = rng.normal(0, scale, (L, M)) + 1.j * rng.normal(0, scale, (L, M))
    else:  # initializers.py:17-20  U[0, scale) + i U[0, scale)
        params["kernel"] = rng.uniform(0, scale, (L, M)) + 1.j * rng.uniform(0, scale, (L, M))
    return params


# ---------------------------------------------------------------------------
# Operators (jVMC/operator/branch_free.py, base.py)
# ---------------------------------------------------------------------------

def LocalOp(idx, map, matEls, diag, fermionic=False):
    return {"idx": idx, "map": np.asarray(map, dtype=np.int32),
            "matEls": np.asarray(matEls, dtype=tCpx), "diag": diag, "fermionic": fermionic}


def Id(idx=0, lDim=2):  # branch_free.py:17-33
    return LocalOp(idx, list(range(lDim)), [1.] * lDim, True)


def Sx(idx):  # branch_free.py:36-51
    return LocalOp(idx, [1, 0], [1.0, 1.0], False)


def Sy(idx):  # branch_free.py:54-69
    return LocalOp(idx, [1, 0], [1.j, -1.j], False)


def Sz(idx):  # branch_free.py:72-87
    return LocalOp(idx, [0, 1], [-1.0, 1.0], True)


def Sp(idx):  # branch_free.py:90-105
    return LocalOp(idx, [1, 0], [1.0, 0.0], False)


def Sm(idx):  # branch_free.py:108-123
    return LocalOp(idx, [0, 0], [0.0, 1.0], False)


def number(idx):  # branch_free.py:128-146
    return LocalOp(idx, [0, 1], [0., 1.], True, False)


def creation(idx):  # branch_free.py:150-168
    return LocalOp(idx, [1, 0], [1., 0.], False, True)


def annihilation(idx):  # branch_free.py:172-190
    return LocalOp(idx, [1, 0], [0., 1.], False, True)


def scal_opstr(a, ops):
    """An operator string (prefactor, op_0, ..., op_{n-1}); prefactor may be
    a number or a callable of the operator arguments (branch_free.py:258-276)."""
    return (a,) + tuple(ops)


class BranchFreeOperator:
    """Restatement of branch_free.py:311-487 and base.py:91-212."""

    def __init__(self, lDim=2):
        self.ops = []
        self.lDim = lDim

    def add(self, opDescr):
        if not isinstance(opDescr, tuple):
            opDescr = (opDescr,)
        self.ops.append(opDescr)

    def compile(self):
        """Tables idx/map/matEls/fermi (numOps, maxOpStrLength[, lDim]),
        operators stored right-to-left and padded with Id(0);
        branch_free.py:348-414."""
        def has_pref(op):
            return not isinstance(op[0], dict)
        maxLen = 0
        for op in self.ops:
            maxLen = max(maxLen, len(op) - (1 if has_pref(op) else 0))
        IdOp = Id(lDim=self.lDim)
        idx, mp, me, fe, diag, pref = [], [], [], [], [], []
        for o, op in enumerate(self.ops):
            k0 = 1 if has_pref(op) else 0
            pref.append(op[0] if k0 else None)
            isDiag = True
            ri, rm, rme, rf = [], [], [], []
            for k in range(maxLen):
                kRev = len(op) - k - 1
                if kRev >= k0:
                    lo = op[kRev]
                    if not lo["diag"]:
                        isDiag = False
                    ri.append(lo["idx"]); rm.append(lo["map"]); rme.append(lo["matEls"])
                    rf.append(1 if lo.get("fermionic", False) else 0)
                else:
                    ri.append(IdOp["idx"]); rm.append(IdOp["map"]); rme.append(IdOp["matEls"]); rf.append(0)
            if isDiag:
                diag.append(o)
            idx.append(ri); mp.append(rm); me.append(rme); fe.append(rf)
        self.idxC = np.array(idx, dtype=np.int32)
        self.mapC = np.array(mp, dtype=np.int32)
        self.matElsC = np.array(me, dtype=tCpx)
        self.fermiC = np.array(fe, dtype=np.int32)
        self.diag = np.array(diag, dtype=np.int32)
        self.prefactor = pref

    def arg_fun(self, *args):
        """Prefactors of the strings (branch_free.py:416-438)."""
        res = np.ones(len(self.ops), dtype=tCpx)
        for i, f in enumerate(self.prefactor):
            if f is None:
                continue
            res[i] = f(*args) if callable(f) else f
        return res

    def _s_primes_one(self, s, matEl0):
        """branch_free.py:443-487 for one configuration."""
        shape = s.shape
        cfg0 = s.ravel().astype(np.int64)
        dim = cfg0.size
        numOps = self.idxC.shape[0]
        sp = np.empty((numOps, dim), dtype=np.int32)
        m = np.array(matEl0, dtype=tCpx)
        for o in range(numOps):
            c = cfg0.copy()
            me = m[o]
            for k in range(self.idxC.shape[1]):
                i = self.idxC[o, k]
                f = self.fermiC[o, k]
                sign = 1.0
                if f:
                    # (-1)^(number of occupied sites j > i); branch_free.py:463-466
                    sign = -1.0 if (c[i + 1:].sum() % 2) else 1.0
                me = me * self.matElsC[o, k, c[i]] * sign
                c[i] = self.mapC[o, k, c[i]]
            m[o] = me
            sp[o] = c
        if len(self.diag) > 1:
            m[self.diag[0]] = m[self.diag].sum()
            m[self.diag[1:]] = 0
        return sp.reshape((numOps,) + shape), m

    def get_s_primes(self, s, *args):
        """base.py:116-160: s' and matrix elements, compacted to the nonzeros
        (|m| > 1e-6, ascending op index), padded to the maximum count with the
        last op string's s' and matrix element 0."""
        self.compile()
        pref = self.arg_fun(*args)
        s = np.asarray(s)
        flat = s.reshape((-1,) + s.shape[2:])
        N = flat.shape[0]
        numOps = self.idxC.shape[0]
        sps, ms = [], []
        for n in range(N):
            sp, m = self._s_primes_one(flat[n], pref)
            sps.append(sp); ms.append(m)
        sps = np.array(sps); ms = np.array(ms)
        # _find_nonzero base.py:91-103
        nz = np.abs(ms) > 1e-6
        choice = np.where(nz, np.arange(numOps)[None, :], numOps - 1)
        idx = np.sort(choice, axis=1)
        cnt = nz.sum(1)
        K = int(cnt.max()) if N else 0
        idx = idx[:, :K]
        m = np.take_along_axis(ms, idx, axis=1)
        m = np.where(np.arange(K)[None, :] < cnt[:, None], m, 0)  # set_zero_to_zero 105-114
        sp = sps[np.arange(N)[:, None], idx]
        self.matEl = m.reshape(s.shape[:2] + (K,))
        self.numNonzero = cnt
        return sp.reshape((s.shape[0], N * K // s.shape[0]) + s.shape[2:]), self.matEl

    def get_O_loc_unbatched(self, logPsiS, logPsiSP):
        """base.py:162-164,194-212."""
        m = self.matEl
        return (m * np.exp(logPsiSP.reshape(m.shape) - logPsiS[..., None])).sum(-1)

    def get_O_loc(self, samples, psi, logPsiS=None, *args):
        """base.py:166-192."""
        if logPsiS is None:
            logPsiS = psi(samples)
        sp, _ = self.get_s_primes(samples, *args)
        logPsiSP = psi(sp)
        return self.get_O_loc_unbatched(logPsiS, logPsiSP)


def hamiltonian_matrix(op, L, *args):
    """Dense 2^L x 2^L matrix of a branch-free operator (bit i of the basis
    index = site i), built independently of the s' machinery from the tables.
    <s|H|s'> = m when s' = op-string applied to s (the reference convention:
    E_loc(s) = sum_s' <s|H|s'> psi(s')/psi(s))."""
    op.compile()
    pref = op.arg_fun(*args)
    D = 2 ** L
    H = np.zeros((D, D), dtype=tCpx)
    for a in range(D):
        s = np.array([(a >> i) & 1 for i in range(L)], dtype=np.int32)
        numOps = op.idxC.shape[0]
        for o in range(numOps):
            c = s.astype(np.int64).copy()
            me = pref[o]
            for k in range(op.idxC.shape[1]):
                i = op.idxC[o, k]
                sign = 1.0
                if op.fermiC[o, k]:
                    sign = -1.0 if (c[i + 1:].sum() % 2) else 1.0
                me = me * op.matElsC[o, k, c[i]] * sign
                c[i] = op.mapC[o, k, c[i]]
            b = int((c * (1 << np.arange(L))).sum())
            H[a, b] += me
    return H


def tfim(L, J=1.0, h=0.7, periodic=True, lattice=None):
    """H = -J sum Z_i Z_{i+1} - h sum X_i; per site ZZ then X (the add order
    used by the reference's tests and the workloads)."""
    H = BranchFreeOperator()
    if lattice is None:
        for l in range(L):
            if periodic or l + 1 < L:
                H.add(scal_opstr(-J, (Sz(l), Sz((l + 1) % L))))
            H.add(scal_opstr(-h, (Sx(l),)))
    else:
        Lx, Ly = lattice
        for y in range(Ly):
            for x in range(Lx):
                i = y * Lx + x
                H.add(scal_opstr(-J, (Sz(i), Sz(y * Lx + (x + 1) % Lx))))
                H.add(scal_opstr(-J, (Sz(i), Sz(((y + 1) % Ly) * Lx + x))))
                H.add(scal_opstr(-h, (Sx(i),)))
    return H


def xxz(L, delta=1.5, periodic=True):
    """H = sum (X X + Y Y + Delta Z Z) with Pauli matrices, add order XX, YY, ZZ."""
    H = BranchFreeOperator()
    for l in range(L):
        if periodic or l + 1 < L:
            r = (l + 1) % L
            H.add(scal_opstr(1.0, (Sx(l), Sx(r))))
            H.add(scal_opstr(1.0, (Sy(l), Sy(r))))
            H.add(scal_opstr(delta, (Sz(l), Sz(r))))
    return H


# ---------------------------------------------------------------------------
# MPI wrapper restated for one process / one device (jVMC/mpi_wrapper.py)
# ---------------------------------------------------------------------------

class Comm:
    globNumSamples = 0


def distribute_sampling(numSamples, localDevices=None, numChainsPerDevice=1):
    """mpi_wrapper.py:53-95 with commSize = 1."""
    if localDevices is None:
        Comm.globNumSamples = numSamples
        return numSamples, numSamples
    ncp = localDevices * numChainsPerDevice
    spc = int((numSamples + ncp - 1) // ncp)
    Comm.globNumSamples = spc * ncp
    return spc, Comm.globNumSamples


def global_sum(data):
    """mpi_wrapper.py:114-147: sum over (device, batch)."""
    return np.asarray(data).sum(axis=(0, 1))


def global_mean(data, p):
    """mpi_wrapper.py:150-174."""
    data = np.asarray(data)
    return np.tensordot(p[0], data[0], axes=(0, 0))


def global_variance(data, p):
    """mpi_wrapper.py:177-217."""
    data = np.asarray(data)
    mean = global_mean(data, p)
    d = data[0] - mean[None]
    return np.einsum("ij,ij,i->j", np.conj(d), d, p[0])


# ---------------------------------------------------------------------------
# Sample statistics (jVMC/stats.py)
# ---------------------------------------------------------------------------

class SampledObs:
    """stats.py:136-336 for one device."""

    def __init__(self, observations=None, weights=None):
        self._weights = None if weights is None else np.asarray(weights)
        self._data = None
        self._mean = None
        if observations is not None and weights is not None:
            obs = np.asarray(observations)
            if obs.ndim == 2:
                obs = obs[..., None]
            # _compute_data_and_mean stats.py:197-205
            self._mean = np.tensordot(self._weights[0], obs[0], axes=(0, 0))
            sw = np.sqrt(self._weights).reshape(self._weights.shape + (1,) * (obs.ndim - 2))
            self._data = sw * (obs - self._mean[None, None])

    def mean(self):
        return self._mean

    def _w(self, nd):
        return self._weights[0].reshape(self._weights.shape[1:] + (1,) * (nd - 1))

    def covar(self, other=None):
        if other is None:
            other = self
        return np.tensordot(np.conj(self._data[0]), other._data[0], axes=(0, 0))

    def var(self):
        return (np.abs(self._data) ** 2).sum(axis=(0, 1))

    def covar_data(self, other=None):
        if other is None:
            other = self
        d = np.conj(self._data[0])[:, :, None] * other._data[0][:, None, :] / self._weights[0][:, None, None]
        return SampledObs(d[None], self._weights)

    def covar_var(self, other=None):
        if other is None:
            other = self
        a = (np.abs(np.conj(self._data[0])[:, :, None] * other._data[0][:, None, :]) ** 2
             / self._weights[0][:, None, None]).sum(0)
        return a - np.abs(self.covar(other)) ** 2

    def transform(self, nonLinearFun=lambda x: x, linearFun=None):
        d = self._data[0]
        x = d / np.sqrt(self._w(d.ndim)) + self._mean[None]
        x = nonLinearFun(x)
        if linearFun is not None:
            x = np.matmul(np.asarray(linearFun), x)
        return SampledObs(x[None], self._weights)

    def subset(self, start=None, end=None, step=None):
        """stats.py:310-329."""
        new = SampledObs()
        w = self._weights[:, start:end:step]
        nrm = w.sum()
        d = self._data[:, start:end:step] / np.sqrt(nrm)
        w = w / nrm
        new._weights = w
        new._mean = np.tensordot(np.sqrt(w[0]), d[0], axes=(0, 0)) + self._mean
        new._data = d + np.sqrt(w)[..., None] * (self._mean - new._mean)[None, None]
        return new

    def tangent_kernel(self):
        d = self._data.reshape((-1,) + self._data.shape[2:])
        return d @ np.conj(d.T)


# ---------------------------------------------------------------------------
# Samplers (jVMC/sampler.py)
# ---------------------------------------------------------------------------

def exact_basis(L, lDim=2):
    """sampler.py:421-472: site i = bit i (lDim 2); for lDim > 2 the digits
    are written most-significant first."""
    n = lDim ** L
    ints = np.arange(n, dtype=np.int64)
    if lDim == 2:
        return ((ints[:, None] >> np.arange(L)[None, :]) & 1).astype(np.int32)
    digs = np.empty((n, L), dtype=np.int32)
    c = ints.copy()
    for k in range(L):
        digs[:, k] = c % lDim
        c //= lDim
    return digs[:, ::-1].copy()


class ExactSampler:
    """sampler.py:385-532 for one device."""

    def __init__(self, psi, sampleShape, lDim=2, logProbFactor=0.5):
        if isinstance(sampleShape, int):
            sampleShape = (sampleShape,)
        self.psi = psi
        self.sampleShape = tuple(sampleShape)
        self.N = int(np.prod(self.sampleShape))
        self.lDim = lDim
        self.logProbFactor = logProbFactor
        distribute_sampling(lDim ** self.N)
        self.basis = exact_basis(self.N, lDim).reshape((1, -1) + self.sampleShape)
        self.lastNorm = 0.

    def sample(self, parameters=None, numSamples=None, multipleOf=None):
        if parameters is not None:
            tmp = self.psi.get_parameters()
            self.psi.set_parameters(parameters)
        logPsi = self.psi(self.basis)
        if parameters is not None:
            self.psi.set_parameters(tmp)
        p = np.exp(np.real(logPsi - self.lastNorm) / self.logProbFactor)
        nrm = global_sum(p)
        p = p / nrm
        self.lastNorm += self.logProbFactor * np.log(nrm)
        return self.basis, logPsi, p

    def get_last_number_of_samples(self):
        return np.inf


PHILOX_M0 = np.uint64(0xD2511F53)
PHILOX_M1 = np.uint64(0xCD9E8D57)
PHILOX_W0 = np.uint32(0x9E3779B9)
PHILOX_W1 = np.uint32(0xBB67AE85)


def philox4x32(c0, c1, c2, c3, k0, k1, rounds=10):
    """Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw,
    "Parallel random numbers: as easy as 1, 2, 3", SC'11).  Vectorised over
    numpy uint32 arrays; returns four uint32 arrays."""
    M = np.uint64(0xFFFFFFFF)
    x0, x1, x2, x3 = (np.asarray(v, dtype=np.uint32) for v in (c0, c1, c2, c3))
    k0 = np.asarray(k0, dtype=np.uint32)
    k1 = np.asarray(k1, dtype=np.uint32)
    with np.errstate(over="ignore"):
        for r in range(rounds):
            p0 = PHILOX_M0 * x0.astype(np.uint64)
            p1 = PHILOX_M1 * x2.astype(np.uint64)
            hi0 = (p0 >> np.uint64(32)).astype(np.uint32)
            lo0 = (p0 & M).astype(np.uint32)
            hi1 = (p1 >> np.uint64(32)).astype(np.uint32)
            lo1 = (p1 & M).astype(np.uint32)
            x0, x1, x2, x3 = hi1 ^ x1 ^ k0, lo1, hi0 ^ x3 ^ k1, lo0
            k0 = (k0 + PHILOX_W0).astype(np.uint32)
            k1 = (k1 + PHILOX_W1).astype(np.uint32)
    return x0, x1, x2, x3


def metropolis_draws(seed, call, step, chains, L):
    """Random numbers of one Metropolis step for every chain.

    Counter = (step, chain, call, 0x5EED), key = (seed lo, seed hi).
    Flip site = (r0 * L) >> 32; acceptance uniform
    u = ((r1 >> 5) * 2^26 + (r2 >> 6)) / 2^53 in [0, 1)."""
    ch = np.arange(chains, dtype=np.uint32)
    st = np.full(chains, step & 0xFFFFFFFF, dtype=np.uint32)
    cl = np.full(chains, call & 0xFFFFFFFF, dtype=np.uint32)
    r0, r1, r2, r3 = philox4x32(st, ch, cl, np.full(chains, 0x5EED, np.uint32),
                                np.uint32(seed & 0xFFFFFFFF), np.uint32((seed >> 32) & 0xFFFFFFFF))
    site = ((r0.astype(np.uint64) * np.uint64(L)) >> np.uint64(32)).astype(np.int64)
    u = ((r1 >> np.uint32(5)).astype(np.float64) * 67108864.0 + (r2 >> np.uint32(6)).astype(np.float64)) / 9007199254740992.0
    return site, u


class MCSampler:
    """Metropolis sampler of sampler.py:67-382 (propose_spin_flip, 15-19)
    driven by the Philox stream of :func:`metropolis_draws`.

    Per step: every chain proposes one flip, computes
    P = exp(mu Re logpsi(s') - mu Re logpsi(s)) by full re-evaluation
    (sampler.py:335-336) and accepts iff u < P (bernoulli, 339-340)."""

    def __init__(self, psi, sampleShape, seed, numChains=1, numSamples=100,
                 thermalizationSweeps=10, sweepSteps=10, initState=None, mu=2, logProbFactor=0.5):
        self.psi = psi
        self.sampleShape = tuple(sampleShape)
        self.L = int(np.prod(self.sampleShape))
        self.seed = seed
        self.numChains = numChains
        self.numSamples = numSamples
        self.thermalizationSweeps = thermalizationSweeps
        self.sweepSteps = sweepSteps
        self.mu = mu
        self.logProbFactor = logProbFactor
        if initState is None:
            initState = np.zeros(self.sampleShape, dtype=np.int32)
        self.states = np.stack([np.asarray(initState, dtype=np.int32)] * numChains)
        self.calls = 0
        self.numProposed = 0
        self.numAccepted = 0

    def _logacc(self, states):
        return self.mu * np.real(self.psi(states[None]))[0]

    def _sweep(self, nsteps, step0):
        states = self.states
        C = self.numChains
        for t in range(nsteps):
            site, u = metropolis_draws(self.seed, self.calls, step0 + t, C, self.L)
            new = states.reshape(C, -1).copy()
            new[np.arange(C), site] = (new[np.arange(C), site] + 1) % 2
            new = new.reshape(states.shape)
            newLog = self._logacc(new)
            P = np.exp(newLog - self.logAcc)
            acc = u < P
            self.numProposed += C
            self.numAccepted += int(acc.sum())
            states = np.where(acc.reshape((C,) + (1,) * len(self.sampleShape)), new, states)
            self.logAcc = np.where(acc, newLog, self.logAcc)
        self.states = states
        return step0 + nsteps

    def sample(self, parameters=None, numSamples=None, multipleOf=1):
        if numSamples is None:
            numSamples = self.numSamples
        if parameters is not None:
            tmp = self.psi.get_parameters()
            self.psi.set_parameters(parameters)
        self.logAcc = self._logacc(self.states)
        self.numProposed = 0
        self.numAccepted = 0
        perChain, self.globNumSamples = distribute_sampling(
            numSamples, localDevices=1, numChainsPerDevice=int(np.lcm(self.numChains, multipleOf)))
        step = self._sweep(self.thermalizationSweeps * self.sweepSteps, 0)
        configs = []
        for k in range(perChain):
            step = self._sweep(self.sweepSteps, step)
            configs.append(self.states.copy())
        self.calls += 1
        configs = np.array(configs).reshape((1, perChain * self.numChains) + self.sampleShape)
        logPsi = self.psi(configs)
        if parameters is not None:
            self.psi.set_parameters(tmp)
        p = np.exp((1.0 / self.logProbFactor - self.mu) * np.real(logPsi))
        return configs, logPsi, p / global_sum(p)

    def acceptance_ratio(self):
        return self.numAccepted / self.numProposed if self.numProposed else 0.0

    def get_last_number_of_samples(self):
        return self.globNumSamples


# ---------------------------------------------------------------------------
# TDVP (jVMC/util/tdvp.py)
# ---------------------------------------------------------------------------

def realFun(x):  # tdvp.py:14-15
    return np.real(x)


def imagFun(x):  # tdvp.py:18-19
    return 0.5 * (x - np.conj(x))


class TDVP:
    """tdvp.py:64-326 restated for one device.  The eigendecomposition is
    numpy's LAPACK eigh of the full 2P representation, as in the reference."""

    def __init__(self, sampler, snrTol=2, pinvTol=1e-14, pinvCutoff=1e-8, makeReal='imag',
                 rhsPrefactor=1.j, diagonalShift=0., crossValidation=False, snrMode="reference",
                 perturbS=None):
        # perturbS = (relative size, seed): multiply every entry of S by
        # 1 + size * e with e a symmetric N(0, 1) matrix before the
        # eigendecomposition -- a planted roundoff-sized change that measures
        # how strongly the solve amplifies it (test instrumentation only).
        self.perturbS = perturbS
        self.sampler = sampler
        self.snrTol = snrTol
        self.pinvTol = pinvTol
        self.pinvCutoff = pinvCutoff
        self.diagonalShift = diagonalShift
        self.rhsPrefactor = rhsPrefactor
        self.crossValidation = crossValidation
        self.makeReal = imagFun if makeReal == 'imag' else realFun
        self.metaData = None
        self.snrMode = snrMode

    def set_diagonal_shift(self, delta):
        self.diagonalShift = delta

    def trafo_helper(self, x):  # tdvp.py:22-23
        return self.makeReal((-self.rhsPrefactor) * x)

    def _get_tdvp_error(self, update):  # tdvp.py:102-104
        return np.abs(1. + np.real(update.dot(self.S0.dot(update)) - 2. * np.real(update.dot(self.F0))) / self.ElocVar0)

    def get_tdvp_equation(self, Eloc, gradients):  # tdvp.py:134-148
        self.ElocMean = Eloc.mean()[0]
        self.ElocVar = Eloc.var()[0]
        self.F0 = (-self.rhsPrefactor) * gradients.covar(Eloc).ravel()
        F = self.makeReal(self.F0)
        self.S0 = gradients.covar()
        S = self.makeReal(self.S0)
        if self.diagonalShift > 1e-10:
            S = S + np.diag(self.diagonalShift * np.diag(S))
        return S, F

    def _transform_to_eigenbasis(self, S, F):  # tdvp.py:153-171
        if self.perturbS is not None:
            size, seed = self.perturbS
            e = np.random.default_rng(seed).normal(size=S.shape)
            S = S + S * (size * 0.5 * (e + e.T))
        self.ev, self.V = np.linalg.eigh(S)
        self.VtF = np.conj(self.V).T @ F

    def _get_snr(self, Eloc, gradients):  # tdvp.py:173-181
        EO = gradients.covar_data(Eloc).transform(linearFun=np.conj(self.V).T,
                                                  nonLinearFun=self.trafo_helper)
        self.rhoVar = EO.var().ravel()
        self.snr = np.sqrt(np.abs(Comm.globNumSamples * (np.conj(self.VtF) * self.VtF) / self.rhoVar)).ravel()
        if self.snrMode == "pair":
            # makeReal='real' with a holomorphic ansatz: eigenvalues come in
            # degenerate pairs (2k, 2k+1) whose basis LAPACK picks arbitrarily;
            # give both members the rotation-invariant pair SNR.
            v2 = np.abs(self.VtF) ** 2
            num = v2[0::2] + v2[1::2]
            den = self.rhoVar[0::2] + self.rhoVar[1::2]
            pair = np.sqrt(np.abs(Comm.globNumSamples * num / den))
            self.snr = np.repeat(pair, 2)

    def solve(self, Eloc, gradients):  # tdvp.py:183-213
        self.S, F = self.get_tdvp_equation(Eloc, gradients)
        self._transform_to_eigenbasis(self.S, F)
        self._get_snr(Eloc, gradients)
        self.invEv = np.where(np.abs(self.ev / self.ev[-1]) > 1e-14, 1. / self.ev, 0.)
        residual = 1.0
        cutoff = 1e-2
        F_norm = np.linalg.norm(F)
        while residual > self.pinvTol and cutoff > self.pinvCutoff:
            cutoff *= 0.8
            regularizer = 1. / (1. + (max(cutoff, self.pinvCutoff) / np.abs(self.ev / self.ev[-1])) ** 6)
            if not isinstance(self.sampler, ExactSampler):
                regularizer = regularizer * (1. / (1. + (self.snrTol / self.snr) ** 6))
            pinvEv = self.invEv * regularizer
            residual = np.linalg.norm((pinvEv * self.ev - np.ones_like(pinvEv)) * self.VtF) / F_norm
        update = np.real(self.V @ (pinvEv * self.VtF))
        return update, residual, max(cutoff, self.pinvCutoff)

    def __call__(self, netParameters, t, *, psi, hamiltonian, **rhsArgs):  # tdvp.py:219-326
        tmp = psi.get_parameters()
        psi.set_parameters(netParameters)
        numSamples = rhsArgs.get("numSamples", None)
        configs, logPsi, p = self.sampler.sample(numSamples=numSamples)
        Eloc = hamiltonian.get_O_loc(configs, psi, logPsi, t)
        Eloc = SampledObs(Eloc, p)
        grads = SampledObs(psi.gradients(configs), p)
        update, residual, cut = self.solve(Eloc, grads)
        psi.set_parameters(tmp)
        if rhsArgs.get("intStep", None) == 0:
            self.ElocMean0 = self.ElocMean
            self.ElocVar0 = self.ElocVar
            self.metaData = {"tdvp_error": self._get_tdvp_error(update), "tdvp_residual": residual,
                             "pinv_cutoff": cut, "SNR": self.snr, "spectrum": self.ev}
        return update

    def get_energy_variance(self):
        return self.ElocVar0

    def get_energy_mean(self):
        return np.real(self.ElocMean0)


# ---------------------------------------------------------------------------
# Integrators (jVMC/util/stepper.py)
# ---------------------------------------------------------------------------

class Euler:
    """stepper.py:6-42."""

    def __init__(self, timeStep=1e-3):
        self.dt = timeStep

    def step(self, t, f, yInitial, **rhsArgs):
        dy = f(yInitial, t, **rhsArgs, intStep=0)
        return yInitial + self.dt * dy, self.dt


class Heun:
    """stepper.py:45-95."""

    def __init__(self, timeStep=1e-3):
        self.dt = timeStep

    def step(self, t, f, yInitial, **rhsArgs):
        dt = rhsArgs.get("dt", self.dt)
        k0 = f(yInitial, t, **rhsArgs, intStep=0)
        y = yInitial + dt * k0
        k1 = f(y, t + dt, **rhsArgs, intStep=1)
        return yInitial + 0.5 * dt * (k0 + k1), dt


class AdaptiveHeun:
    """stepper.py:98-182."""

    def __init__(self, timeStep=1e-3, tol=1e-8, maxStep=1):
        self.dt = timeStep
        self.tolerance = tol
        self.maxStep = maxStep

    def step(self, t, f, y, normFunction=np.linalg.norm, **rhsArgs):
        fe = 0.5
        dt = self.dt
        yInitial = y.copy()
        while fe < 1.:
            y = yInitial.copy()
            k0 = f(y, t, **rhsArgs, intStep=0)
            y = y + dt * k0
            k1 = f(y, t + dt, **rhsArgs, intStep=1)
            dy0 = 0.5 * dt * (k0 + k1)
            y = y - 0.5 * dt * k0
            k10 = f(y, t + 0.5 * dt, **rhsArgs, intStep=2)
            dy1 = 0.25 * dt * (k0 + k10)
            y = yInitial + dy1
            k01 = f(y, t + 0.5 * dt, **rhsArgs, intStep=3)
            y = y + 0.5 * dt * k01
            k11 = f(y, t + dt, **rhsArgs, intStep=4)
            dy1 = dy1 + 0.25 * dt * (k01 + k11)
            updateDiff = normFunction(dy1 - dy0)
            fe = self.tolerance / updateDiff
            tmp = 0.2 if 0.2 > 0.9 * fe ** 0.33333 else 0.9 * fe ** 0.33333
            if tmp > 2.:
                tmp = 2.
            realDt = dt
            dt *= tmp
            if dt > self.maxStep:
                dt = self.maxStep
        self.dt = dt
        return yInitial + dy1, realDt


# ---------------------------------------------------------------------------
# Drivers (jVMC/util/util.py)
# ---------------------------------------------------------------------------

def measure(observables, psi, sampler, numSamples=None):
    """util.py:91-157."""
    configs, logPsi, p = sampler.sample(numSamples=numSamples)
    result = {}
    for name, ops in observables.items():
        if not isinstance(ops, (list, tuple)):
            ops = [ops]
        means, vars_, errs = [], [], []
        for op in ops:
            args = ()
            if isinstance(op, (list, tuple)):
                args = tuple(op[1:])
                op = op[0]
            Oloc = op.get_O_loc(configs, psi, logPsi, *args)
            means.append(global_mean(Oloc[..., None], p)[0])
            vars_.append(global_variance(Oloc[..., None], p)[0])
            errs.append(np.sqrt(vars_[-1]) / np.sqrt(sampler.get_last_number_of_samples()))
        result[name] = {"mean": np.real(np.array(means)), "variance": np.real(np.array(vars_)),
                        "MC_error": np.real(np.array(errs))}
    return result


def ground_state_search(psi, ham, tdvpEquation, sampler, numSteps=200, varianceTol=1e-10, stepSize=1e-2):
    """util.py:160-212 without output management."""
    delta = getattr(tdvpEquation, "diagonalShift", 0.)
    stepper = Euler(timeStep=stepSize)
    n = 0
    varE = 1.0
    while n < numSteps and varE > varianceTol:
        dp, _ = stepper.step(0, tdvpEquation, psi.get_parameters(), hamiltonian=ham, psi=psi, numSamples=None)
        psi.set_parameters(dp)
        n += 1
        varE = tdvpEquation.get_energy_variance()
        if hasattr(tdvpEquation, "set_diagonal_shift"):
            delta = 0.95 * delta
            tdvpEquation.set_diagonal_shift(delta)
    return n


# ---------------------------------------------------------------------------
# MinSR (jVMC/util/minsr.py)
# ---------------------------------------------------------------------------

def pinv_hermitian(T, rtol):
    """Pseudo-inverse of a Hermitian matrix through its eigendecomposition,
    dropping |eigenvalues| <= rtol * max |eigenvalue| (jnp.linalg.pinv with
    hermitian=True, as called at minsr.py:63,74)."""
    ev, V = np.linalg.eigh(T)
    cut = rtol * np.max(np.abs(ev))
    inv = np.where(np.abs(ev) > cut, 1.0 / ev, 0.0)
    return (V * inv) @ np.conj(V.T)


class MinSR:
    """minsr.py:16-165 for one device."""

    def __init__(self, sampler, pinvTol=1e-14, diagonalShift=0.):
        self.sampler = sampler
        self.pinvTol = pinvTol
        self.diagonalShift = diagonalShift

    def solve(self, eloc, gradients, holomorphic):  # minsr.py:53-80
        if holomorphic:
            T = gradients.tangent_kernel()
            T_inv = pinv_hermitian(T, self.pinvTol)
            e = eloc._data.reshape((-1,))
            G = gradients._data.reshape((-1,) + gradients._data.shape[2:])
            return -np.conj(G).T @ T_inv @ e
        G = gradients._data.reshape((-1,) + gradients._data.shape[2:])
        G = np.concatenate([np.real(G), np.imag(G)], axis=0)
        T = G @ G.T + self.diagonalShift * np.eye(G.shape[0])
        T_inv = pinv_hermitian(T, self.pinvTol)
        e = eloc._data.reshape((-1,))
        e = np.concatenate([np.real(e), np.imag(e)], axis=0)
        return -G.T @ T_inv @ e

    def __call__(self, netParameters, t, *, psi, hamiltonian, **rhsArgs):  # minsr.py:82-165
        tmp = psi.get_parameters()
        psi.set_parameters(netParameters)
        configs, logPsi, p = self.sampler.sample(numSamples=rhsArgs.get("numSamples", None))
        Eloc = SampledObs(hamiltonian.get_O_loc(configs, psi, logPsi, t), p)
        grads = SampledObs(psi.gradients(configs), p)
        update = self.solve(Eloc, grads, holomorphic=psi.holomorphic)
        psi.set_parameters(tmp)
        if rhsArgs.get("intStep", None) == 0:
            self.ElocMean0 = Eloc.mean()[0]
            self.ElocVar0 = Eloc.var()[0]
        return update

    def get_energy_variance(self):
        return self.ElocVar0

    def get_energy_mean(self):
        return np.real(self.ElocMean0)
