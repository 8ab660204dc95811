"""The integrators of vmc_jax_gb300.util.stepper (host logic: step-size
control, half-step comparison) follow the oracle's restatement of
stepper.py:6-182 step for step, on numpy arrays and on torch tensors."""

import numpy as np
import pytest
import torch

from oracle import jvmc_oracle as O
from vmc_jax_gb300.util import stepper as S


def _problem():
    rs = np.random.RandomState(7)
    mat = (rs.rand(5, 5) - 0.5) + 1.j * (rs.rand(5, 5) - 0.5)
    y0 = rs.rand(5) + 1.j * rs.rand(5)
    return mat, y0


@pytest.mark.parametrize("kind", ["Euler", "Heun", "AdaptiveHeun"])
@pytest.mark.parametrize("as_torch", [False, True])
def test_stepper_follows_oracle(kind, as_torch):
    mat, y0 = _problem()
    kw = {"timeStep": 0.05}
    if kind == "AdaptiveHeun":
        kw.update(tol=1e-6, maxStep=0.2)
    ref, mine = getattr(O, kind)(**kw), getattr(S, kind)(**kw)
    tm = torch.as_tensor(mat)

    def f_ref(y, t, **args):
        return mat.dot(y)

    def f_mine(y, t, **args):
        return tm @ y if as_torch else mat.dot(y)

    def norm_ref(y):
        return np.real(np.conj(y).dot(y))

    def norm_mine(y):
        return torch.real(torch.vdot(y, y)) if as_torch else norm_ref(y)

    yr, ym = y0.copy(), (torch.as_tensor(y0) if as_torch else y0.copy())
    tr = tmine = 0.0
    for _ in range(40):
        if kind == "AdaptiveHeun":
            yr, dtr = ref.step(tr, f_ref, yr, normFunction=norm_ref)
            ym, dtm = mine.step(tmine, f_mine, ym, normFunction=norm_mine)
        else:
            yr, dtr = ref.step(tr, f_ref, yr)
            ym, dtm = mine.step(tmine, f_mine, ym)
        tr += dtr
        tmine += float(dtm)
        got = ym.numpy() if as_torch else ym
        assert abs(tmine - tr) <= 1e-12 * max(1.0, tr)
        assert np.abs(got - yr).max() <= 1e-12 * np.abs(yr).max()
    if kind == "AdaptiveHeun":
        assert ref.dt == pytest.approx(mine.dt, rel=1e-12)
