"""Lattice symmetry orbits (CPU): the package's generators against the
oracle's restatement of util/symmetries.py, the element counts of the
reference's tests/symmetries_test.py:15-43, and the kernel codes."""

import numpy as np
import pytest

from oracle import jvmc_oracle as O
from vmc_jax_gb300.util import symmetries as S

FACTORS = dict(reflection_factor=-1., translation_factor=np.exp(0.7j), spinflip_factor=1j)


@pytest.mark.parametrize("L", [3, 6])
@pytest.mark.parametrize("use", [(), ("translation",), ("reflection",), ("spinflip",),
                                 ("translation", "reflection", "spinflip")])
def test_orbit_1d(L, use):
    ls = S.get_orbit_1D(L, *use, **FACTORS)
    o, f = O.get_orbit_1D(L, *use, **FACTORS)
    assert np.array_equal(ls.orbit, o) and np.array_equal(ls.factor, f)
    assert np.issubdtype(ls.dtype, np.integer)
    # symmetries_test.py:31-43 (L = 3: 2 reflections, 3 translations, 2 spin flips)
    if L == 3:
        n = (2 if "reflection" in use else 1) * (3 if "translation" in use else 1) * (2 if "spinflip" in use else 1)
        assert ls.shape[0] == n


@pytest.mark.parametrize("L", [3, 4])
@pytest.mark.parametrize("use", [("rotation",), ("reflection",), ("translation",), ("spinflip",),
                                 ("rotation", "reflection", "translation", "spinflip")])
def test_orbit_2d(L, use):
    kw = dict(FACTORS, rotation_factor=1j)
    ls = S.get_orbit_2D_square(L, *use, **kw)
    o, f = O.get_orbit_2D_square(L, *use, **kw)
    assert np.array_equal(ls.orbit, o) and np.array_equal(ls.factor, f)
    assert np.issubdtype(ls.dtype, np.integer)


def test_orbit_codes_reproduce_transformed_configs():
    ls = S.get_orbit_2D_square(4, "rotation", "reflection", "translation", "spinflip")
    codes, inv = S.orbit_codes(ls)
    s = np.random.default_rng(1).integers(0, 2, (7, 16))
    ref = O.SymNet(O.CpxRBM(2), ls.orbit, ls.factor).transformed(s)  # (S, N, L)
    got = (s[:, codes >> 1] ^ (codes & 1)[None]).transpose(1, 0, 2)
    assert np.array_equal(got, ref)
    assert np.array_equal(np.take_along_axis(codes >> 1, inv, axis=1), np.tile(np.arange(16), (len(codes), 1)))


def test_orbit_codes_reject_non_permutations():
    o = np.zeros((1, 3, 3), np.int32)
    o[0, 0, 0] = o[0, 1, 0] = o[0, 2, 2] = 1
    with pytest.raises(ValueError):
        S.orbit_codes(o)


def test_oracle_symnet_sector_signs():
    """symmetries_test.py:46-85 on the oracle: in the odd sector of a
    reflection / translation / spin flip, psi(g s) = -psi(s)."""
    L = 10
    rng = np.random.default_rng(0)
    prm = O.init_cpx_rbm(L, 2, True, rng, scale=0.3)
    c1 = rng.permutation(np.array([0, 1] * (L // 2)))
    for use, c2 in (("reflection", c1[::-1]), ("translation", np.roll(c1, 1)), ("spinflip", 1 - c1)):
        o, f = O.get_orbit_1D(L, use, reflection_factor=-1., translation_factor=np.exp(1j * np.pi),
                              spinflip_factor=-1.)
        net = O.SymNet(O.CpxRBM(2, True), o, f)
        a = net.apply(prm, c1[None])[0]
        b = net.apply(prm, c2[None].copy())[0]
        assert abs(1 + np.exp(a - b)) < 1e-10


def test_oracle_symnet_gradient_finite_difference():
    """The oracle's SymNet gradient (weights f exp(lp_tau - lp)) against
    central differences of its log psi (vqs_test.py:104-125)."""
    L = 6
    rng = np.random.default_rng(1)
    prm = O.init_cpx_rbm(L, 3, True, rng, scale=0.3)
    o, f = O.get_orbit_1D(L, "translation", "reflection", translation_factor=np.exp(0.4j))
    for avg in (O.avgFun_Coefficients_Exp, O.avgFun_Coefficients_Log):
        psi = O.NQS(O.SymNet(O.CpxRBM(3, True), o, f, avg), prm)
        s = rng.integers(0, 2, (1, 5, L))
        G = psi.gradients(s)[0]
        th = psi.get_parameters()
        eps = 1e-6
        for j in range(0, th.size, 7):
            u = np.zeros(th.size)
            u[j] = eps
            psi.set_parameters(th + u)
            up = psi(s)[0]
            psi.set_parameters(th - u)
            dn = psi(s)[0]
            psi.set_parameters(th)
            assert np.max(np.abs((up - dn) / (2 * eps) - G[:, j])) < 1e-6
