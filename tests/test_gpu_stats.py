"""The public ``vmc_jax_gb300.stats.SampledObs`` on CUDA tensors against the
known answers of the reference's tests/stats_test.py:15-39 (extracted into
tests/golden/reference_fixtures.json), and against the oracle's SampledObs on
a random weighted complex sample."""

import numpy as np
import pytest
import torch

from oracle import jvmc_oracle as O

pytestmark = pytest.mark.gpu


def test_sampled_obs_known_answers(cuda, fixtures):
    from vmc_jax_gb300.stats import SampledObs
    p = torch.full((1, 3), 1.0 / 3, dtype=torch.float64, device=cuda)
    o1 = SampledObs(torch.tensor([fixtures["stats_obs1"]], dtype=torch.float64, device=cuda), p)
    o2 = SampledObs(torch.tensor([fixtures["stats_obs2"]], dtype=torch.float64, device=cuda), p)
    assert o1.mean().is_cuda
    assert abs(float(o1.mean()[0]) - fixtures["stats_mean1"]) < 1e-12
    assert abs(float(o1.var()[0]) - fixtures["stats_var1"]) < 1e-12
    np.testing.assert_allclose(o2.covar().cpu().numpy(), np.array(fixtures["stats_covar2"]), rtol=0, atol=1e-12)
    np.testing.assert_allclose(o2.mean().cpu().numpy(), np.array(fixtures["stats_mean2"]), rtol=0, atol=1e-12)
    np.testing.assert_allclose(o1.covar(o2).cpu().numpy().ravel(), np.array(fixtures["stats_covar12"]).ravel(),
                               rtol=0, atol=1e-12)
    np.testing.assert_allclose(o1.covar(o2).cpu().numpy().ravel(),
                               o1.covar_data(o2).mean().cpu().numpy().ravel(), rtol=0, atol=1e-12)
    np.testing.assert_allclose(o1.covar_var(o2).cpu().numpy().ravel(),
                               o1.covar_data(o2).var().cpu().numpy().ravel(), rtol=0, atol=1e-12)
    D = o2._data.reshape((-1, 2))
    np.testing.assert_allclose(o2.tangent_kernel().cpu().numpy(), (D @ torch.conj(D).T).cpu().numpy(), rtol=0,
                               atol=1e-12)


def test_sampled_obs_matches_oracle_on_weighted_complex_data(cuda):
    from vmc_jax_gb300.stats import SampledObs
    rng = np.random.default_rng(5)
    n, k = 257, 6
    x = rng.normal(size=(1, n, k)) + 1j * rng.normal(size=(1, n, k))
    y = rng.normal(size=(1, n)) + 1j * rng.normal(size=(1, n))
    w = rng.uniform(0.1, 1.0, size=(1, n))
    w /= w.sum()
    ox, oy = O.SampledObs(x, w), O.SampledObs(y, w)
    gx = SampledObs(torch.as_tensor(x, device=cuda), torch.as_tensor(w, device=cuda))
    gy = SampledObs(torch.as_tensor(y, device=cuda), torch.as_tensor(w, device=cuda))
    for got, want in [(gx.mean(), ox.mean()), (gx.var(), ox.var()), (gx.covar(), ox.covar()),
                      (gx.covar(gy), ox.covar(oy)), (gx.covar_var(gy), ox.covar_var(oy)),
                      (gx.tangent_kernel(), ox.tangent_kernel())]:
        g = got.resolve_conj().cpu().numpy()
        np.testing.assert_allclose(g.reshape(np.shape(want)), want, rtol=1e-12, atol=1e-14)
