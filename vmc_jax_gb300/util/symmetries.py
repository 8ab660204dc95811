"""Lattice symmetry orbits (mirror of jVMC/util/symmetries.py).

An orbit is a stack of signed permutation matrices o_tau (|S|, L, L) int32
and one factor per element (the character of the chosen symmetry sector).
The symmetrised network evaluates the plain network on
tau(s) = (o_tau (2s - 1) + 1) // 2.  The matrices are generated and
de-duplicated exactly as in the reference (products translation x
reflection [x rotation], optional spin flip as -o, then ``np.unique`` over
the flattened matrices, which fixes the element order).
"""

import numpy as np


class LatticeSymmetry:
    """Orbit matrices and their factors (symmetries.py:9-38).

    Initializer arguments:
        * ``orbit``: (|S|, L, L) integer array, one signed permutation matrix
          per symmetry operation.
        * ``factor``: (|S|,) phase factor of each operation.
    """

    def __init__(self, orbit, factor):
        self._orbit = np.asarray(orbit)
        self._factor = np.asarray(factor)

    @property
    def factor(self):
        return self._factor

    @property
    def orbit(self):
        return self._orbit

    @property
    def shape(self):
        return self._orbit.shape

    @property
    def dtype(self):
        return self._orbit.dtype


def get_2D_index(L):
    return np.arange(L ** 2).reshape((L, L))


def get_1D_index(L):
    return np.arange(L)


def _matrix(site_map, idx):
    o = np.zeros((idx.size, idx.size), dtype=np.int32)
    o[idx.ravel(), site_map.ravel()] = 1
    return o


def _unique(orbits, factors, n):
    uo, first = np.unique(orbits.reshape((-1, n * n)), return_index=True, axis=0)
    return LatticeSymmetry(uo.reshape(-1, n, n).astype(np.int32), np.asarray(factors)[first])


def get_orbits_from_maps_1D(L, translation, reflection):
    """symmetries.py:146-165."""
    idx = get_1D_index(L)
    orbits, factors = [], []
    for mt, ft in zip(translation["maps"], translation["factor"]):
        for mr, fr in zip(reflection["maps"], reflection["factor"]):
            orbits.append(_matrix(mt, idx) @ _matrix(mr, idx))
            factors.append(ft * fr)
    return np.array(orbits), np.array(factors)


def get_maps_1D(L, **kwargs):
    """symmetries.py:168-188."""
    idx = get_1D_index(L)
    reflection = {"maps": [idx], "factor": [1.]}
    translation = {"maps": [idx], "factor": [1.]}
    if kwargs["reflection"]["use"]:
        reflection["maps"].append(idx[::-1])
        reflection["factor"].append(kwargs["reflection"]["factor"])
    if kwargs["translation"]["use"]:
        for x in range(1, L):
            translation["maps"].append(np.roll(idx, x, axis=(0,)))
            translation["factor"].append(kwargs["translation"]["factor"] ** x)
    return translation, reflection


def get_orbit_1D(L, *args, translation_factor=1., reflection_factor=1., spinflip_factor=1.):
    """Group of lattice symmetries of a chain of L sites (symmetries.py:191-212).

    ``*args``: any of "reflection", "translation", "spinflip";
    ``*_factor``: the factor of the corresponding generator."""
    kwargs = {"reflection": {"use": "reflection" in args, "factor": reflection_factor},
              "translation": {"use": "translation" in args, "factor": translation_factor},
              "spinflip": {"use": "spinflip" in args, "factor": spinflip_factor}}
    translation, reflection = get_maps_1D(L, **kwargs)
    orbits, factors = get_orbits_from_maps_1D(L, translation, reflection)
    if kwargs["spinflip"]["use"]:
        orbits = np.concatenate([orbits, -orbits], axis=0)
        factors = np.concatenate([factors, spinflip_factor * factors])
    return _unique(orbits, factors, L)


def get_orbits_from_maps_2D(L, translation, rotation, reflection):
    """symmetries.py:51-75: products T @ A @ B over translation (outer),
    then the maps passed as ``reflection``, then those passed as
    ``rotation``.  ``get_orbit_2D_square`` passes (translation, reflection,
    rotation) to these parameters, as the reference does
    (symmetries.py:134), so the elements are T @ Rot @ Refl."""
    idx = get_2D_index(L)
    orbits, factors = [], []
    for mt, ft in zip(translation["maps"], translation["factor"]):
        for ma, fa in zip(reflection["maps"], reflection["factor"]):
            for mb, fb in zip(rotation["maps"], rotation["factor"]):
                orbits.append(_matrix(mt, idx) @ _matrix(ma, idx) @ _matrix(mb, idx))
                factors.append(ft * fa * fb)
    return np.array(orbits), np.array(factors)


def get_maps_2D(L, **kwargs):
    """symmetries.py:78-111."""
    idx = get_2D_index(L)
    rotation = {"maps": [idx], "factor": [1.]}
    reflection = {"maps": [idx], "factor": [1.]}
    translation = {"maps": [idx], "factor": [1.]}
    if kwargs["rotation"]["use"]:
        f = kwargs["rotation"]["factor"]
        rotation["maps"] += [idx[::-1, :].T, idx[::-1, ::-1], idx[:, ::-1].T]
        rotation["factor"] += [f, f ** 2, f ** 3]
    if kwargs["reflection"]["use"]:
        f = kwargs["reflection"]["factor"]
        reflection["maps"] += [idx[::-1, :], idx[:, ::-1], idx[::-1, ::-1]]
        reflection["factor"] += [f, f, f ** 2]
    if kwargs["translation"]["use"]:
        for x in range(L):
            for y in range(L):
                if x == 0 and y == 0:
                    continue
                translation["maps"].append(np.roll(idx, (y, x), axis=(0, 1)))
                translation["factor"].append(kwargs["translation"]["factor"] ** (x + y))
    return translation, reflection, rotation


def get_orbit_2D_square(L, *args, translation_factor=1., reflection_factor=1., rotation_factor=1.,
                        spinflip_factor=1.):
    """Group of lattice symmetries of an L x L square lattice
    (symmetries.py:114-148).

    ``*args``: any of "reflection", "rotation", "translation", "spinflip"."""
    kwargs = {"reflection": {"use": "reflection" in args, "factor": reflection_factor},
              "translation": {"use": "translation" in args, "factor": translation_factor},
              "rotation": {"use": "rotation" in args, "factor": rotation_factor},
              "spinflip": {"use": "spinflip" in args, "factor": spinflip_factor}}
    translation, reflection, rotation = get_maps_2D(L, **kwargs)
    orbits, factors = get_orbits_from_maps_2D(L, translation, reflection, rotation)
    if kwargs["spinflip"]["use"]:
        orbits = np.concatenate([orbits, -orbits], axis=0)
        factors = np.concatenate([factors, spinflip_factor * factors])
    return _unique(orbits, factors, L ** 2)


def orbit_codes(orbit):
    """Kernel form of an orbit: codes (|S|, L) int32 = 2 src + flip with
    tau(s)_i = s_src xor flip, and the inverse (|S|, L) int32 (position of
    tau(s) that holds site j).  Raises ValueError unless every o_tau is a
    signed permutation matrix."""
    o = np.asarray(orbit.orbit if isinstance(orbit, LatticeSymmetry) else orbit)
    if o.ndim != 3 or o.shape[1] != o.shape[2]:
        raise ValueError("orbit must have shape (|S|, L, L)")
    S, L, _ = o.shape
    nz = o != 0
    if not np.all(nz.sum(axis=2) == 1) or not np.all(nz.sum(axis=1) == 1) or not np.all(np.abs(o[nz]) == 1):
        raise ValueError("every orbit element must be a signed permutation matrix")
    src = np.argmax(nz, axis=2)                           # (S, L)
    flip = (np.take_along_axis(o, src[:, :, None], axis=2)[:, :, 0] < 0).astype(np.int32)
    codes = (2 * src + flip).astype(np.int32)
    inverse = np.empty((S, L), dtype=np.int32)
    inverse[np.arange(S)[:, None], src] = np.arange(L)[None, :]
    return codes, inverse
