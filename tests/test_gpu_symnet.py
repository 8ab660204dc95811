"""Symmetrised CpxRBM (nets/sym_wrapper.py) against the oracle: log psi,
gradients, fused O_loc, Metropolis chains, and the reference's own SymNet
tests (symmetries_test.py:46-135 sector signs, sampler_test.py:32-82 MCMC
histogram with the fixed weights, vqs_test.py:104-125 finite differences).

Bars as in test_gpu_parity: FP64 within 1e-11 relative, FP32 within 5e-5,
Metropolis chains bit-exact for the same Philox stream (FP64)."""

import numpy as np
import pytest
import torch

from oracle import jvmc_oracle as O

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def _sym_pair(L, M, bias, orbit, avg="exp", seed=0, scale=0.3, precision="fp64"):
    import vmc_jax_gb300 as V
    from vmc_jax_gb300.nets import sym_wrapper as SW
    rng = np.random.default_rng(seed)
    prm = O.init_cpx_rbm(L, M, bias, rng, scale=scale / np.sqrt(L))
    oavg = O.avgFun_Coefficients_Exp if avg == "exp" else O.avgFun_Coefficients_Log
    opsi = O.NQS(O.SymNet(O.CpxRBM(M, bias), orbit.orbit, orbit.factor, oavg), prm)
    gavg = SW.avgFun_Coefficients_Exp if avg == "exp" else SW.avgFun_Coefficients_Log
    psi = V.vqs.NQS(V.nets.CpxRBM(numHidden=M, bias=bias), orbit=orbit, avgFun=gavg, precision=precision)
    psi(np.zeros((1, 1, L), np.int32))
    psi.set_parameters(opsi.get_parameters())
    return psi, opsi


def _configs(N, L, seed):
    return np.random.default_rng(seed).integers(0, 2, (1, N, L)).astype(np.int32)


def _orbit(L, *use, **kw):
    from vmc_jax_gb300.util import symmetries as S
    return S.get_orbit_1D(L, *use, **kw)


@pytest.mark.parametrize("avg", ["exp", "log"])
@pytest.mark.parametrize("use", [("translation",), ("translation", "reflection", "spinflip")])
def test_logpsi_and_gradients(cuda, avg, use):
    import vmc_jax_gb300 as V
    L, M = 8, 6
    # a phase on the translations that is not a lattice momentum keeps
    # psi away from exact zeros on symmetric configurations
    orbit = _orbit(L, *use, translation_factor=np.exp(0.4j))
    psi, opsi = _sym_pair(L, M, True, orbit, avg, seed=3)
    s = _configs(200, L, seed=4)
    assert _rel(psi(s).cpu().numpy(), opsi(s)) < 1e-12
    g = psi.gradients(s).cpu().numpy()
    assert _rel(g, opsi.gradients(s)) < 1e-11
    flat = torch.as_tensor(s[0], device=cuda)
    gc = psi.net.gradients(psi.params, flat, "fp64", V._lib.VMC_GRAD_COMPACT).cpu().numpy()
    P = gc.shape[1]
    assert _rel(gc, opsi.gradients(s)[0][:, np.r_[0:M, 2 * M:2 * M + L * M]]) < 1e-11 and P == M + L * M
    psi.precision = "fp32"
    psi._touch()
    assert _rel(psi(s).cpu().numpy(), opsi(s)) < 5e-5
    assert _rel(psi.gradients(s).cpu().numpy(), opsi.gradients(s)) < 5e-5


def test_gradients_orbit_chunks(cuda):
    """M = 1024 in FP64: the orbit is processed in several shared-memory
    chunks (5 elements each)."""
    L, M = 6, 1024
    orbit = _orbit(L, "translation", "reflection")
    psi, opsi = _sym_pair(L, M, True, orbit, "exp", seed=5, scale=0.05)
    s = _configs(40, L, seed=6)
    assert _rel(psi.gradients(s).cpu().numpy(), opsi.gradients(s)) < 1e-11


def test_gradients_finite_difference(cuda):
    """vqs_test.py:104-125: SymNet(CpxRBM(2, bias)) with the identity orbit."""
    L = 3
    orbit = _orbit(L)
    psi, _ = _sym_pair(L, 2, True, orbit, "exp", seed=7, scale=0.5)
    s = np.zeros((1, 4, L), np.int32)
    s[0, 1, 2] = 1
    s[0, 2, 2] = 1
    psi0 = psi(s).cpu().numpy()
    G = psi.gradients(s).cpu().numpy()
    delta = 1e-6
    for j in range(G.shape[-1]):
        u = np.zeros(G.shape[-1])
        u[j] = 1
        psi.update_parameters(delta * u)
        psi1 = psi(s).cpu().numpy()
        psi.update_parameters(-delta * u)
        assert np.max(np.abs((psi1 - psi0) / delta - G[..., j])) < 1e-5


@pytest.mark.parametrize("L,use", [(10, "reflection"), (10, "translation"), (10, "spinflip")])
def test_symmetry_sector_1d(cuda, L, use):
    """symmetries_test.py:46-85 with a biased CpxRBM (not spin-flip
    symmetric on its own): psi(g s) = -psi(s) in the odd sector."""
    import vmc_jax_gb300 as V
    orbit = _orbit(L, use, reflection_factor=-1., translation_factor=np.exp(1j * 2 * np.pi * L / 2 / L),
                   spinflip_factor=-1.)
    psi = V.vqs.NQS(V.nets.CpxRBM(numHidden=2, bias=True), orbit=orbit)
    psi(np.zeros((1, 1, L), np.int32))
    psi.set_parameters(np.random.default_rng(0).normal(0, 0.3, psi.numParameters * 2))
    c1 = np.random.default_rng(1).permutation(np.array([0, 1] * (L // 2)))
    c2 = {"reflection": c1[::-1], "translation": np.roll(c1, 1), "spinflip": 1 - c1}[use]
    a = psi(c1[None, None]).cpu().numpy()
    b = psi(c2[None, None].copy()).cpu().numpy()
    assert np.abs(1 + np.exp(a - b)) < 1e-10


@pytest.mark.parametrize("use", ["rotation", "reflection", "translation", "spinflip"])
def test_symmetry_sector_2d(cuda, use):
    """symmetries_test.py:87-131 (L = 4) with a biased CpxRBM."""
    import vmc_jax_gb300 as V
    from vmc_jax_gb300.util import symmetries as S
    L = 4
    orbit = S.get_orbit_2D_square(L, use, rotation_factor=-1., reflection_factor=-1.,
                                  translation_factor=np.exp(1j * 2 * np.pi * L / 2 / L), spinflip_factor=-1.)
    psi = V.vqs.NQS(V.nets.CpxRBM(numHidden=2, bias=True), orbit=orbit)
    psi(np.zeros((1, 1, L, L), np.int32))
    psi.set_parameters(np.random.default_rng(2).normal(0, 0.3, psi.numParameters * 2))
    c1 = np.random.default_rng(3).permutation(np.array([0, 1] * (L * L // 2))).reshape(L, L)
    c2 = {"rotation": c1[:, ::-1].T, "reflection": c1[::-1, :], "translation": np.roll(c1, 1, axis=0),
          "spinflip": 1 - c1}[use]
    a = psi(c1[None, None]).cpu().numpy()
    b = psi(np.ascontiguousarray(c2)[None, None]).cpu().numpy()
    assert np.abs(1 + np.exp(a - b)) < 1e-10


def _tfim(L, h):
    import vmc_jax_gb300.operator as op
    H = op.BranchFreeOperator()
    for l in range(L):
        H.add(op.scal_opstr(-1.0, (op.Sz(l), op.Sz((l + 1) % L))))
        H.add(op.scal_opstr(-h, (op.Sx(l),)))
    return H, O.tfim(L, 1.0, h)


def _xxz(L, delta):
    import vmc_jax_gb300.operator as op
    H = op.BranchFreeOperator()
    for l in range(L):
        r = (l + 1) % L
        H.add(op.scal_opstr(1.0, (op.Sx(l), op.Sx(r))))
        H.add(op.scal_opstr(1.0, (op.Sy(l), op.Sy(r))))
        H.add(op.scal_opstr(delta, (op.Sz(l), op.Sz(r))))
    return H, O.xxz(L, delta)


@pytest.mark.parametrize("model", ["tfim", "xxz"])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_fused_oloc(cuda, model, precision):
    L, M = 8, 5
    orbit = _orbit(L, "translation", "reflection", "spinflip", translation_factor=np.exp(0.4j))
    psi, opsi = _sym_pair(L, M, True, orbit, "exp", seed=8, precision=precision)
    H, Ho = _tfim(L, 0.7) if model == "tfim" else _xxz(L, 1.5)
    s = _configs(300, L, seed=9)
    ref = Ho.get_O_loc(s, opsi)
    tol = 1e-11 if precision == "fp64" else 5e-5
    assert _rel(H.get_O_loc(s, psi).cpu().numpy(), ref) < tol
    lp = opsi(s) + 0.25 - 0.1j
    got = H.get_O_loc(s, psi, torch.as_tensor(lp, device=cuda)).cpu().numpy()
    assert _rel(got, Ho.get_O_loc(s, opsi, lp)) < tol


def test_oloc_log_average_unfused(cuda):
    """avgFun_Coefficients_Log has no fused estimator: s' are formed and the
    symmetrised net evaluated on them."""
    L, M = 8, 4
    orbit = _orbit(L, "translation")
    psi, opsi = _sym_pair(L, M, True, orbit, "log", seed=10)
    H, Ho = _xxz(L, 1.5)
    s = _configs(100, L, seed=11)
    assert not H.fused_capable(psi)
    assert _rel(H.get_O_loc(s, psi).cpu().numpy(), Ho.get_O_loc(s, opsi)) < 1e-11


@pytest.mark.parametrize("avg,mu", [("exp", 2), ("log", 2), ("exp", 1)])
def test_metropolis_bit_exact(cuda, avg, mu):
    """Same Philox stream: the block-per-chain kernel with incremental tanh
    updates makes the same decisions as the oracle's full re-evaluation."""
    import vmc_jax_gb300 as V
    L, M = 8, 4
    orbit = _orbit(L, "translation", "reflection")
    psi, opsi = _sym_pair(L, M, True, orbit, avg, seed=12, scale=0.8)
    mc = V.sampler.MCSampler(psi, (L,), 4321, updateProposer=V.sampler.propose_spin_flip, numChains=12,
                             numSamples=48, thermalizationSweeps=3, sweepSteps=L, mu=mu)
    mco = O.MCSampler(opsi, (L,), 4321, numChains=12, numSamples=48, thermalizationSweeps=3, sweepSteps=L, mu=mu)
    for _ in range(2):
        s, lp, p = mc.sample()
        so, lpo, po = mco.sample()
        assert np.array_equal(s.cpu().numpy(), so)
        assert _rel(lp.cpu().numpy(), lpo) < 1e-12
        assert _rel(p.cpu().numpy(), po) < 1e-12
        c = mc.counters.cpu().numpy()
        assert c[0] == mco.numProposed and c[1] == mco.numAccepted


def test_metropolis_histogram_vs_exact(cuda, fixtures):
    """sampler_test.py:32-82: SymNet(CpxRBM(2)) over translation, reflection
    and spin flip with the fixed weights; MCMC histogram vs ExactSampler
    (< 2e-3), FP32 chains; log psi of the samples vs re-evaluation."""
    import vmc_jax_gb300 as V
    L = 4
    orbit = _orbit(L, "translation", "reflection", "spinflip")
    psi = V.vqs.NQS(V.nets.CpxRBM(2, False), orbit=orbit, precision="fp32")
    psi(np.zeros((1, 1, L), np.int32))
    psi.set_parameters(np.array(fixtures["rbm_L4_M2_weights"]))
    es = V.sampler.ExactSampler(psi, L)
    _, _, pex = es.sample()
    mc = V.sampler.MCSampler(psi, (L,), 0, updateProposer=V.sampler.propose_spin_flip, numChains=777)
    smc, lp, p = mc.sample(numSamples=500000)
    assert smc.shape[1] >= 500000
    ints = (smc[0].long() * (2 ** torch.arange(L, device=cuda))).sum(-1)
    pmc = torch.bincount(ints, weights=p[0], minlength=16)
    pmc = pmc / pmc.sum()
    assert torch.max(torch.abs(pmc - pex[0])) < 2e-3
    assert torch.max(torch.abs((lp - psi(smc)) / lp)) < 1e-14


def test_autograd_backward(cuda):
    import vmc_jax_gb300 as V
    from vmc_jax_gb300.autograd import log_psi
    L, M = 6, 3
    orbit = _orbit(L, "translation", "reflection")
    psi, opsi = _sym_pair(L, M, True, orbit, "exp", seed=13)
    s = _configs(50, L, seed=14)
    theta = psi.get_parameters().clone().requires_grad_(True)
    out = log_psi(psi, theta, s)
    c = torch.randn_like(out)
    (out * c).sum().backward()
    G = opsi.gradients(s)[0]                    # (N, 2P): d log psi / d theta_real
    cc = c.detach().cpu().numpy()
    ref = cc[:, 0] @ G.real + cc[:, 1] @ G.imag
    assert _rel(theta.grad.cpu().numpy(), ref) < 1e-11


@pytest.mark.parametrize("makeReal,rhs", [("real", 1.0), ("imag", 1.j)])
def test_tdvp_exact_step(cuda, makeReal, rhs):
    """One Euler step of a SymNet state with the ExactSampler: the complex
    P x P pipeline fed from the materialised O (FP64) against the oracle's
    2P real solve."""
    import vmc_jax_gb300 as V
    L, M = 8, 4
    orbit = _orbit(L, "translation", "reflection")
    psi, opsi = _sym_pair(L, M, True, orbit, "exp", seed=15, scale=0.8)
    H, Ho = _tfim(L, 0.8)
    es, eso = V.sampler.ExactSampler(psi, L), O.ExactSampler(opsi, L)
    td = V.util.TDVP(es, makeReal=makeReal, rhsPrefactor=rhs, pinvCutoff=1e-8)
    tdo = O.TDVP(eso, makeReal=makeReal, rhsPrefactor=rhs, pinvCutoff=1e-8)
    th, tho = psi.get_parameters(), opsi.get_parameters()
    new, _ = V.util.stepper.Euler(timeStep=0.01).step(0, td, th, hamiltonian=H, psi=psi)
    newo, _ = O.Euler(timeStep=0.01).step(0, tdo, tho, hamiltonian=Ho, psi=opsi)
    assert abs(complex(td.ElocMean0) - tdo.ElocMean0) / abs(tdo.ElocMean0) < 1e-10
    assert _rel((new - th).cpu().numpy(), newo - tho) < 1e-8
    assert _rel(td.get_metadata()["spectrum"].cpu().numpy(), tdo.metaData["spectrum"]) < 1e-8
    # S0 v in the reference layout (tdvp.py:215-216), S0 of the last RHS call
    v = np.random.default_rng(0).normal(size=th.numel())
    assert _rel(td.S_dot(torch.as_tensor(v, device=cuda)).cpu().numpy(), tdo.S0 @ v) < 1e-10


def test_tdvp_mc_same_samples(cuda):
    """MCSampler (same Philox chains on both sides) + SNR regulariser."""
    import vmc_jax_gb300 as V
    L, M = 8, 4
    orbit = _orbit(L, "translation")
    psi, opsi = _sym_pair(L, M, True, orbit, "exp", seed=16, scale=0.8)
    H, Ho = _tfim(L, 0.8)
    mc = V.sampler.MCSampler(psi, (L,), 99, updateProposer=V.sampler.propose_spin_flip, numChains=64,
                             numSamples=2048, thermalizationSweeps=4, sweepSteps=L)
    mco = O.MCSampler(opsi, (L,), 99, numChains=64, numSamples=2048, thermalizationSweeps=4, sweepSteps=L)
    td = V.util.TDVP(mc, makeReal="imag", rhsPrefactor=1.j, pinvCutoff=1e-8, snrTol=2)
    tdo = O.TDVP(mco, makeReal="imag", rhsPrefactor=1.j, pinvCutoff=1e-8, snrTol=2)
    u = td(psi.get_parameters(), 0., psi=psi, hamiltonian=H, intStep=0).cpu().numpy()
    uo = tdo(opsi.get_parameters(), 0., psi=opsi, hamiltonian=Ho, intStep=0)
    assert abs(complex(td.ElocMean0) - tdo.ElocMean0) / abs(tdo.ElocMean0) < 1e-10
    assert _rel(u, uo) < 1e-8


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_tdvp_reduced_precision(cuda, precision):
    """The FP32 and mixed (BF16x3 tcgen05) S/SNR builds from the dense data
    producers against the FP64 step on the same samples: energy within 1e-5,
    update within 1e-3 relative (well-conditioned state)."""
    import vmc_jax_gb300 as V
    L, M = 16, 8
    orbit = _orbit(L, "translation", "reflection")
    H, _ = _tfim(L, 1.0)
    out = {}
    for prec in ("fp64", precision):
        psi, _ = _sym_pair(L, M, True, orbit, "exp", seed=17, scale=0.8,
                           precision="fp64" if prec == "fp64" else "fp32")
        mc = V.sampler.MCSampler(psi, (L,), 5, updateProposer=V.sampler.propose_spin_flip, numChains=128,
                                 numSamples=4096, thermalizationSweeps=4, sweepSteps=L)
        # the same chains for both: sample with FP64 kernels
        psi.precision = "fp64"
        psi._touch()
        configs, lp, p = mc.sample()
        psi.precision = "fp64" if prec == "fp64" else "fp32"
        psi._touch()
        td = V.util.TDVP(mc, makeReal="imag", rhsPrefactor=1.j, pinvCutoff=1e-8, snrTol=2, precision=prec)
        Eloc = H.get_O_loc(configs, psi, None)
        upd, res, cut = td._complex_rhs(psi, configs, Eloc, p)
        out[prec] = (upd.cpu().numpy(), complex(td.ElocMean))
    u64, e64 = out["fp64"]
    u, e = out[precision]
    assert abs(e - e64) / abs(e64) < 1e-5
    assert _rel(u, u64) < 1e-3
