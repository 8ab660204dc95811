"""CNN ansatz (10x10 transverse-field Ising workload shapes) on the CUDA
path against the oracle: log psi and the hand-written O_k backward at 1e-12
relative (FP64), the backward against central finite differences
(eps = 1e-4), Metropolis chains bit-exact, and a TDVP step."""

import numpy as np
import pytest
import torch

from oracle import jvmc_oracle as O

pytestmark = pytest.mark.gpu


def _pair(shape, F, channels, act="poly4", seed=0, scale=0.3):
    import vmc_jax_gb300 as V
    onet = O.CNN(F=F, channels=channels, strides=(1,) * len(F), actFun=(act,))
    rng = np.random.default_rng(seed)
    prm = {k: rng.normal(0, scale, s) for k, s in onet.leaf_shapes(shape)}
    opsi = O.NQS(onet, prm)
    psi = V.vqs.NQS(V.nets.CNN(F=F, channels=channels, strides=(1,) * len(F), actFun=(act,)))
    psi(np.zeros((1, 1) + tuple(shape), np.int32))
    psi.set_parameters(opsi.get_parameters())
    return psi, opsi


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


@pytest.mark.parametrize("shape,F,channels,act", [((10, 10), (3, 3), (8, 8), "poly4"),
                                                  ((4, 4), (3, 3), (3, 2, 5), "poly6"),
                                                  ((9,), (4,), (3, 2), "poly4")])
def test_cnn_logpsi_and_gradients(cuda, shape, F, channels, act):
    psi, opsi = _pair(shape, F, channels, act)
    s = np.random.default_rng(1).integers(0, 2, (1, 200) + tuple(shape)).astype(np.int32)
    assert _rel(psi(s).cpu().numpy(), opsi(s)) < 1e-12
    g = psi.gradients(s).cpu().numpy()
    assert g.shape == (1, 200, opsi.numParameters)
    assert _rel(g, opsi.gradients(s)) < 1e-12
    assert np.all(g.imag == 0)
    psi.precision = "fp32"
    psi._touch()
    assert _rel(psi(s).cpu().numpy(), opsi(s)) < 1e-5


def test_cnn_translation_invariance(cuda):
    """tests/nets_test.py:16-46 on the CUDA kernel."""
    psi, _ = _pair((4, 4), (3, 3), (3, 2, 5), "poly6", seed=3)
    S0 = np.array([[1, 0, 1, 1], [0, 1, 1, 1], [0, 0, 1, 0], [1, 0, 0, 1]])
    S = np.array([np.roll(np.roll(S0, -i, 0), -j, 1) for i in range(4) for j in range(4)])[None].astype(np.int32)
    v = psi(S).cpu().numpy()
    assert np.max(np.abs(v - v[0, 0])) < 1e-12 * np.abs(v[0, 0])


def test_cnn_backward_vs_central_differences(cuda):
    """The 10x10 CNN: hand-written backward vs central finite differences
    (eps = 1e-4) of the CUDA forward pass."""
    psi, _ = _pair((10, 10), (3, 3), (8, 8), seed=5, scale=0.2)
    s = np.random.default_rng(2).integers(0, 2, (1, 16, 10, 10)).astype(np.int32)
    G = psi.gradients(s)[0].real
    theta = psi.get_parameters()
    eps = 1e-4
    for k in np.random.default_rng(0).choice(theta.numel(), 40, replace=False):
        u = torch.zeros_like(theta)
        u[k] = eps
        psi.set_parameters(theta + u)
        lp = psi(s)[0].real
        psi.set_parameters(theta - u)
        lm = psi(s)[0].real
        fd = (lp - lm) / (2 * eps)
        assert torch.max(torch.abs(fd - G[:, k])) < 1e-6 * max(1.0, float(torch.max(torch.abs(G[:, k]))))
    psi.set_parameters(theta)


def test_cnn_metropolis_bit_exact(cuda):
    import vmc_jax_gb300 as V
    psi, opsi = _pair((4, 4), (3, 3), (4, 4), seed=7)
    mc = V.sampler.MCSampler(psi, (4, 4), 99, updateProposer=V.sampler.propose_spin_flip, numChains=8,
                             numSamples=32, thermalizationSweeps=2, sweepSteps=16)
    mco = O.MCSampler(opsi, (4, 4), 99, numChains=8, numSamples=32, thermalizationSweeps=2, sweepSteps=16)
    for _ in range(2):
        s, lp, p = mc.sample()
        so, lpo, po = mco.sample()
        assert np.array_equal(s.cpu().numpy(), so)
        assert _rel(lp.cpu().numpy(), lpo) < 1e-12


def test_cnn_tdvp_exact(cuda):
    """One imaginary-time TDVP step of a 3x3 periodic TFIM with a CNN
    (ExactSampler, FP64): energy 1e-10, update 1e-8 relative."""
    import vmc_jax_gb300 as V
    psi, opsi = _pair((3, 3), (3, 3), (2, 2), seed=11, scale=0.3)
    L = 9
    H = V.operator.BranchFreeOperator()
    for y in range(3):
        for x in range(3):
            i = 3 * y + x
            H.add(V.operator.scal_opstr(-1.0, (V.operator.Sz(i), V.operator.Sz(3 * y + (x + 1) % 3))))
            H.add(V.operator.scal_opstr(-1.0, (V.operator.Sz(i), V.operator.Sz(3 * ((y + 1) % 3) + x))))
            H.add(V.operator.scal_opstr(-3.0, (V.operator.Sx(i),)))
    Ho = O.tfim(L, 1.0, 3.0, lattice=(3, 3))
    es = V.sampler.ExactSampler(psi, (3, 3))
    eso = O.ExactSampler(opsi, (3, 3))
    td = V.util.TDVP(es, makeReal="real", rhsPrefactor=1.)
    tdo = O.TDVP(eso, makeReal="real", rhsPrefactor=1.)
    u = td(psi.get_parameters(), 0., psi=psi, hamiltonian=H, intStep=0).cpu().numpy()
    uo = tdo(opsi.get_parameters(), 0., psi=opsi, hamiltonian=Ho, intStep=0)
    assert abs(complex(td.ElocMean0) - tdo.ElocMean0) / abs(tdo.ElocMean0) < 1e-10
    assert _rel(u, uo) < 1e-8
