"""Parity of the CUDA path against the oracle (FP64 restatement of jVMC).

Bars: integer outputs (basis, s', nonzero counts, Metropolis chains for the
same random stream) bit-exact; FP64 values within 1e-10 relative (1e-12 where
noted); FP32 kernels within 2e-5 relative."""

import numpy as np
import pytest
import torch

from oracle import jvmc_oracle as O

pytestmark = pytest.mark.gpu


def _rbm_pair(L, M, bias, seed, scale=0.1):
    import vmc_jax_gb300 as V
    rng = np.random.default_rng(seed)
    prm = O.init_cpx_rbm(L, M, bias, rng, scale=scale)
    opsi = O.NQS(O.CpxRBM(M, bias), prm)
    psi = V.vqs.NQS(V.nets.CpxRBM(numHidden=M, bias=bias))
    psi(np.zeros((1, 1, L), np.int32))
    psi.set_parameters(opsi.get_parameters())
    return psi, opsi


def _configs(N, L, seed):
    return np.random.default_rng(seed).integers(0, 2, (1, N, L)).astype(np.int32)


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def _tfim_pair(L, J, h):
    import vmc_jax_gb300.operator as op
    H = op.BranchFreeOperator()
    for l in range(L):
        H.add(op.scal_opstr(-J, (op.Sz(l), op.Sz((l + 1) % L))))
        H.add(op.scal_opstr(-h, (op.Sx(l),)))
    return H, O.tfim(L, J, h)


def _xxz_pair(L, delta):
    import vmc_jax_gb300.operator as op
    H = op.BranchFreeOperator()
    for l in range(L):
        r = (l + 1) % L
        H.add(op.scal_opstr(1.0, (op.Sx(l), op.Sx(r))))
        H.add(op.scal_opstr(1.0, (op.Sy(l), op.Sy(r))))
        H.add(op.scal_opstr(delta, (op.Sz(l), op.Sz(r))))
    return H, O.xxz(L, delta)


# ------------------------------------------------------------------ basis
@pytest.mark.parametrize("L,ldim", [(10, 2), (1, 2), (5, 3)])
def test_exact_basis_bit_exact(cuda, L, ldim):
    import vmc_jax_gb300 as V
    psi = V.vqs.NQS(V.nets.CpxRBM(2, False))
    if ldim == 2:
        es = V.sampler.ExactSampler(psi, (L,), lDim=ldim)
        got = es.basis.cpu().numpy()[0]
    else:
        import vmc_jax_gb300._lib as Lb
        got = torch.empty((ldim ** L, L), dtype=torch.int32, device=cuda)
        Lb.call("vmc_exact_basis", Lb.ptr(got), 0, ldim ** L, L, ldim, Lb.stream())
        got = got.cpu().numpy()
    assert np.array_equal(got, O.exact_basis(L, ldim))


# ---------------------------------------------------------------- network
@pytest.mark.parametrize("L,M,bias", [(10, 20, True), (4, 2, False), (64, 256, True), (37, 13, True)])
def test_rbm_logpsi_and_gradients(cuda, L, M, bias):
    # weights scaled so that theta stays clear of the poles of tanh (i pi/2),
    # where summation-order rounding of theta is amplified
    psi, opsi = _rbm_pair(L, M, bias, seed=L * M, scale=0.3 / np.sqrt(L))
    s = _configs(300, L, seed=1)
    lp = psi(s).cpu().numpy()
    assert _rel(lp, opsi(s)) < 1e-12
    g = psi.gradients(s).cpu().numpy()
    assert g.shape == (1, 300, 2 * opsi.numParameters)
    assert _rel(g, opsi.gradients(s)) < 1e-12
    psi.precision = "fp32"
    psi._touch()
    assert _rel(psi(s).cpu().numpy(), opsi(s)) < 2e-5


def test_rbm_gradients_finite_difference(cuda):
    """tests/vqs_test.py:99-131 style check at delta = 1e-6, tolerance 1e-2."""
    psi, _ = _rbm_pair(3, 2, True, seed=3)
    s = np.zeros((1, 4, 3), np.int32)
    s[0, 1, 1] = 1
    s[0, 2, 2] = 1
    psi0 = psi(s)
    G = psi.gradients(s)
    params = psi.get_parameters()
    for j in range(G.shape[-1]):
        u = torch.zeros(G.shape[-1], dtype=torch.float64, device=cuda)
        u[j] = 1
        psi.update_parameters(1e-6 * u)
        psi1 = psi(s)
        psi.set_parameters(params)
        assert torch.max(torch.abs((psi1 - psi0) / 1e-6 - G[..., j])) < 1e-2


# -------------------------------------------------------------- operators
def _ops_cases():
    import vmc_jax_gb300.operator as op
    cases = []
    # S+ strings (operator_test.py:48-68)
    H = op.BranchFreeOperator()
    Ho = O.BranchFreeOperator()
    for i in range(3):
        H += 2. * op.Sp(i)
        Ho.add(O.scal_opstr(2., (O.Sp(i),)))
    cases.append(("sp", 4, H, Ho))
    Ht, Hto = _tfim_pair(10, 1.0, 0.7)
    cases.append(("tfim10", 10, Ht, Hto))
    Hx, Hxo = _xxz_pair(8, 1.5)
    cases.append(("xxz8", 8, Hx, Hxo))
    # mixed string lengths, a Y-Z-X string, an S- string and a cancelling X X on one site
    Hm = op.BranchFreeOperator()
    Hmo = O.BranchFreeOperator()
    for l in range(6):
        Hm.add(op.scal_opstr(0.5, (op.Sy(l), op.Sz((l + 2) % 6), op.Sx((l + 1) % 6))))
        Hmo.add(O.scal_opstr(0.5, (O.Sy(l), O.Sz((l + 2) % 6), O.Sx((l + 1) % 6))))
        Hm.add(op.scal_opstr(0.3, (op.Sm(l),)))
        Hmo.add(O.scal_opstr(0.3, (O.Sm(l),)))
        Hm.add((op.Sz(l),))
        Hmo.add((O.Sz(l),))
    Hm.add((op.Sx(2), op.Sx(2)))
    Hmo.add((O.Sx(2), O.Sx(2)))
    cases.append(("mixed6", 6, Hm, Hmo))
    return cases


@pytest.mark.parametrize("case", range(4))
def test_s_primes_bit_exact(cuda, case):
    name, L, H, Ho = _ops_cases()[case]
    s = _configs(200, L, seed=case)
    s[0, 0] = 0
    s[0, 1] = 1
    sp, m = H.get_s_primes(s)
    spo, mo = Ho.get_s_primes(s)
    assert sp.shape == spo.shape and m.shape == mo.shape
    assert np.array_equal(sp.cpu().numpy(), spo)
    assert np.array_equal(H.numNonzero.cpu().numpy()[0], Ho.numNonzero)
    assert np.max(np.abs(m.cpu().numpy() - mo)) < 1e-14


def test_s_primes_fermions_match_fixture(cuda, fixtures):
    """Jordan-Wigner signs: tests/operator_test.py:189-254 on the GPU expansion."""
    import vmc_jax_gb300.operator as op
    t, mu, Vv, L, fl = -1.0, -2.0, 4.0, 4, 2
    fL = fl * L
    H = op.BranchFreeOperator()
    Ho = O.BranchFreeOperator()
    up, do = 0, fL - 1
    for mod, h in ((op, H), (O, Ho)):
        for i in range(L):
            h.add(mod.scal_opstr(Vv, (mod.number(up + i), mod.number(do - i))))
            h.add(mod.scal_opstr(mu, (mod.number(up + i),)))
            h.add(mod.scal_opstr(mu, (mod.number(do - i),)))
            if i == L - 1:
                continue
            h.add(mod.scal_opstr(t, (mod.creation(up + i + 1), mod.annihilation(up + i))))
            h.add(mod.scal_opstr(t, (mod.creation(up + i), mod.annihilation(up + i + 1))))
            h.add(mod.scal_opstr(t, (mod.creation(do - i - 1), mod.annihilation(do - i))))
            h.add(mod.scal_opstr(t, (mod.creation(do - i), mod.annihilation(do - i - 1))))
    s = O.exact_basis(fL)[None]
    sp, m = H.get_s_primes(s)
    spo, mo = Ho.get_s_primes(s)
    assert np.array_equal(sp.cpu().numpy(), spo)
    assert np.max(np.abs(m.cpu().numpy() - mo)) < 1e-14
    tab = np.array(fixtures["fermion_table_re"]) + 1j * np.array(fixtures["fermion_table_im"])
    onet = O.LookupNet(fL)
    lp = onet.apply({"kernel": tab}, s[0])
    lps = onet.apply({"kernel": tab}, sp.cpu().numpy()[0])
    Eloc = H.get_O_loc_unbatched(torch.as_tensor(lp[None], device=cuda), torch.as_tensor(lps[None], device=cuda))
    p = np.exp(2 * lp.real)
    p /= p.sum()
    E = np.sum(p * Eloc.cpu().numpy()[0])
    assert abs(E - fixtures["fermion_energy"]) < 1e-7


@pytest.mark.parametrize("case", range(4))
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_fused_oloc(cuda, case, precision):
    name, L, H, Ho = _ops_cases()[case]
    psi, opsi = _rbm_pair(L, 7, True, seed=11 + case, scale=0.3)
    s = _configs(300, L, seed=case + 5)
    ref = Ho.get_O_loc(s, opsi)
    psi.precision = precision
    psi._touch()
    got = H.get_O_loc(s, psi).cpu().numpy()
    tol = 1e-11 if precision == "fp64" else 5e-5
    assert _rel(got, ref) < tol
    # with the caller's log psi(s) (base.py:162-164 semantics)
    lp = opsi(s) + 0.25 - 0.1j
    got2 = H.get_O_loc(s, psi, torch.as_tensor(lp, device=cuda)).cpu().numpy()
    ref2 = Ho.get_O_loc(s, opsi, lp)
    assert _rel(got2, ref2) < tol


def test_oloc_unfused_path(cuda):
    """get_s_primes + psi(s') + O_loc kernel (the path of non-RBM nets)."""
    import vmc_jax_gb300 as V
    H, Ho = _xxz_pair(8, 1.5)
    psi, opsi = _rbm_pair(8, 5, True, seed=2, scale=0.3)
    s = _configs(100, 8, seed=9)
    sp, _ = H.get_s_primes(s)
    got = H.get_O_loc_unbatched(psi(s), psi(sp)).cpu().numpy()
    assert _rel(got, Ho.get_O_loc(s, opsi)) < 1e-12
    H2 = V.operator.BranchFreeOperator(ElocBatchSize=13)
    for o in H.ops:
        H2.add(o)
    assert _rel(H2.get_O_loc(s, psi).cpu().numpy(), Ho.get_O_loc(s, opsi)) < 1e-11


def test_time_dependent_prefactor(cuda):
    """tests/operator_test.py:70-93."""
    import vmc_jax_gb300.operator as op
    s = _configs(24, 4, seed=3)
    h = op.BranchFreeOperator()

    def f(t):
        return 2.0 * t
    for i in range(3):
        h.add(op.scal_opstr(f, (op.Sp(i),)))
    for t in [0.5, 2, 13.9]:
        sp, m = h.get_s_primes(s, t)
        lp = torch.ones(s.shape[:-1], dtype=torch.complex128, device=cuda)
        lps = torch.ones(sp.shape[:-1], dtype=torch.complex128, device=cuda)
        tmp = h.get_O_loc_unbatched(lp, lps).cpu().numpy()
        assert np.sum(np.abs(tmp - f(t) * np.sum(-(s[..., :3] - 1), axis=-1))) < 1e-7


# ----------------------------------------------------------------- samplers
def test_exact_sampler_probabilities(cuda):
    import vmc_jax_gb300 as V
    psi, opsi = _rbm_pair(10, 20, True, seed=0, scale=0.3)
    es = V.sampler.ExactSampler(psi, (10,))
    eso = O.ExactSampler(opsi, (10,))
    for _ in range(3):  # lastNorm carries over between calls
        b, lp, p = es.sample()
        bo, lpo, po = eso.sample()
        assert np.array_equal(b.cpu().numpy(), bo)
        assert _rel(lp.cpu().numpy(), lpo) < 1e-12
        assert _rel(p.cpu().numpy(), po) < 1e-12
    assert abs(float(es.lastNorm) - eso.lastNorm) < 1e-12 * max(1, abs(eso.lastNorm))


@pytest.mark.parametrize("mu", [2, 1])
def test_metropolis_bit_exact(cuda, mu):
    """Same Philox stream on both sides: identical chains (FP64 kernel)."""
    import vmc_jax_gb300 as V
    L, M = 8, 4
    psi, opsi = _rbm_pair(L, M, True, seed=21, scale=0.4)
    mc = V.sampler.MCSampler(psi, (L,), 1234, updateProposer=V.sampler.propose_spin_flip, numChains=16,
                             numSamples=64, thermalizationSweeps=3, sweepSteps=L, mu=mu)
    mco = O.MCSampler(opsi, (L,), 1234, numChains=16, numSamples=64, thermalizationSweeps=3, sweepSteps=L, mu=mu)
    for _ in range(2):
        s, lp, p = mc.sample()
        so, lpo, po = mco.sample()
        assert np.array_equal(s.cpu().numpy(), so)
        assert _rel(lp.cpu().numpy(), lpo) < 1e-12
        assert _rel(p.cpu().numpy(), po) < 1e-12
        c = mc.counters.cpu().numpy()
        assert c[0] == mco.numProposed and c[1] == mco.numAccepted


def test_metropolis_histogram_vs_exact(cuda, fixtures):
    """tests/sampler_test.py:32-82: MCMC histogram vs exact probabilities
    (< 2e-3) for the fixed CpxRBM(L=4, M=2) weights; FP32 chains."""
    import vmc_jax_gb300 as V
    L = 4
    psi = V.vqs.NQS(V.nets.CpxRBM(2, False), precision="fp32")
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
