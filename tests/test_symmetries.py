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
