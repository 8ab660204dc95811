"""Host logic of the two-stage eigensolver (util/tdvp.py): where the FP32
spectrum is split into the refined block and the rest, how many power steps
the refinement takes, and the share of the update the rest carries."""

import numpy as np

from vmc_jax_gb300.util import tdvp as T


def _spectrum(rng, null, bulk, top, top_lo=0.05):
    return np.sort(np.concatenate([np.full(null, -1e-9), 10.0 ** rng.uniform(-10, -5, bulk),
                                   rng.uniform(top_lo, 1.0, top)]))


def test_plan_splits_at_the_gap():
    rng = np.random.default_rng(0)
    ev = _spectrum(rng, 20, 780, 200)
    k, q = T.refine_plan(ev, None, None, 1e-8, 2)
    assert k == 200
    # rho = 1e-5 / 0.05: the FP32 error 1e-7 / 0.05 reaches 1e-16 in 3 steps
    assert q == 3


def test_plan_refuses_without_a_gap_or_with_a_large_top_block():
    rng = np.random.default_rng(1)
    assert T.refine_plan(np.sort(10.0 ** rng.uniform(-6, 0, 1000)), None, None, 1e-8, 2) is None
    # the gap lies below the top half of the spectrum
    assert T.refine_plan(_spectrum(rng, 0, 300, 700), None, None, 1e-8, 2) is None
    assert T.refine_plan(np.zeros(10), None, None, 1e-8, 2) is None


def test_plan_ignores_gaps_inside_the_fp32_noise():
    """A relative gap among eigenvalues below 10x the FP32 noise floor (here
    set by the most negative eigenvalue, 1e-4 of the largest) is not taken."""
    ev = np.sort(np.concatenate([[-1e-4], np.full(50, 1e-9), np.full(449, 5e-4), np.linspace(0.1, 1.0, 500)]))
    k, q = T.refine_plan(ev, None, None, 1e-8, 2)
    assert k == 500
    assert 1 <= q <= 16


def test_bulk_share_follows_the_snr_regulariser():
    rng = np.random.default_rng(2)
    ev = _spectrum(rng, 0, 800, 200)
    vtf = rng.normal(size=1000) + 1j * rng.normal(size=1000)
    snr = np.full(1000, 5.0)
    snr[:800] = 0.01
    quiet = T.bulk_weight(ev, vtf, snr, 200, 1e-8, 2)
    snr[:800] = 10.0
    loud = T.bulk_weight(ev, vtf, snr, 200, 1e-8, 2)
    assert quiet < T.REFINE_EXCLUDED_NORM < loud
    # with no bulk the share is zero; with no update at all, too
    assert T.bulk_weight(ev[800:], vtf[800:], snr[800:], 200, 1e-8, 2) == 0.0
    assert T.bulk_weight(ev, np.zeros(1000), snr, 200, 1e-8, 2) == 0.0


def test_solve_weights_match_the_regulariser():
    """solve_weights: |vtf| / lambda times the cutoff regulariser
    1 / (1 + (c / (lambda / lambda_max))^6) and the SNR regulariser
    1 / (1 + (snrTol / snr)^6) (tdvp.py:195-211)."""
    ev = np.array([1e-12, 1e-9, 1e-8, 1e-3, 1.0])
    vtf = np.array([1.0, 2.0, -3.0, 1j, 0.5])
    snr = np.array([1.0, 2.0, 4.0, 0.5, 8.0])
    w = T.solve_weights(ev, vtf, snr, 1e-8, 2)
    r = ev / ev.max()
    ref = np.abs(vtf) / ev / (1 + (1e-8 / r) ** 6) / (1 + (2 / snr) ** 6)
    ref[r <= 1e-14] = 0.0
    np.testing.assert_allclose(w, ref, rtol=1e-14, atol=0)


def test_plan_refuses_steps_that_collapse_the_block():
    """Eigenvalues 1e-4 .. 1 of lambda_max above a bulk below 1e-9: the
    largest relative gap above the FP32 noise floor (4e-6 here) lies inside
    the top block (~0.005 over 1e-4), whose 7 power steps (rho 0.02) would
    grow the FP32 mixing inside the block by ~200^7 = 1e16, beyond
    REFINE_MAX_GROWTH: the plan is refused.  A block spanning 0.05 .. 1 needs
    3 steps and grows it by 20^3 = 8000."""
    rng = np.random.default_rng(3)
    wide = np.sort(np.concatenate([10.0 ** rng.uniform(-10, -9, 800), [1e-4], rng.uniform(1e-4, 1.0, 199)]))
    assert T.refine_plan(wide, None, None, 1e-8, 2) is None
    narrow = _spectrum(rng, 0, 800, 200)
    k, q = T.refine_plan(narrow, None, None, 1e-8, 2)
    assert (k, q) == (200, 3) and (narrow.max() / narrow[800]) ** q < T.REFINE_MAX_GROWTH
