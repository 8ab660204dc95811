"""ODE integrators (mirror of jVMC/util/stepper.py:6-182).  The state y is
a torch tensor (GPU) or a numpy array; every operation stays on its device."""

import numpy as np
import torch


def _copy(y):
    return y.clone() if isinstance(y, torch.Tensor) else np.array(y, copy=True)


def _norm(y):
    return torch.linalg.norm(y) if isinstance(y, torch.Tensor) else np.linalg.norm(y)


class Euler:
    """y_{n+1} = y_n + dt f(y_n, t_n) (stepper.py:6-42)."""

    def __init__(self, timeStep=1e-3):
        self.dt = timeStep

    def step(self, t, f, yInitial, **rhsArgs):
        dy = f(yInitial, t, **rhsArgs, intStep=0)
        return yInitial + self.dt * dy, self.dt


class Heun:
    """Second-order Heun step (stepper.py:45-95)."""

    def __init__(self, timeStep=1e-3):
        self.dt = timeStep

    def set_dt(self, timeStep):
        self.dt = timeStep

    def step(self, t, f, yInitial, **rhsArgs):
        dt = rhsArgs.get("dt", self.dt)
        k0 = f(yInitial, t, **rhsArgs, intStep=0)
        y = yInitial + dt * k0
        k1 = f(y, t + dt, **rhsArgs, intStep=1)
        dy0 = 0.5 * dt * (k0 + k1)
        return yInitial + dy0, dt


class AdaptiveHeun:
    """Heun step with step-size control from a half-step comparison
    (stepper.py:98-182)."""

    def __init__(self, timeStep=1e-3, tol=1e-8, maxStep=1):
        self.dt = timeStep
        self.tolerance = tol
        self.maxStep = maxStep

    def step(self, t, f, y, normFunction=_norm, **rhsArgs):
        fe = 0.5
        dt = self.dt
        yInitial = _copy(y)
        while fe < 1.:
            y = _copy(yInitial)
            k0 = f(y, t, **rhsArgs, intStep=0)
            y = y + dt * k0
            k1 = f(y, t + dt, **rhsArgs, intStep=1)
            dy0 = 0.5 * dt * (k0 + k1)
            # now with half step size
            y = y - 0.5 * dt * k0
            k10 = f(y, t + 0.5 * dt, **rhsArgs, intStep=2)
            dy1 = 0.25 * dt * (k0 + k10)
            y = yInitial + dy1
            k01 = f(y, t + 0.5 * dt, **rhsArgs, intStep=3)
            y = y + 0.5 * dt * k01
            k11 = f(y, t + dt, **rhsArgs, intStep=4)
            dy1 = dy1 + 0.25 * dt * (k01 + k11)
            # compute deviation
            updateDiff = float(normFunction(dy1 - dy0))
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
