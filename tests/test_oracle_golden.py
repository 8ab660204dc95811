"""The oracle (numpy FP64 restatement of jVMC) against the numeric
fixtures of jVMC's own test-suite (tests/golden/reference_fixtures.json)."""

import numpy as np
import pytest
from scipy.interpolate import interp1d
from scipy.linalg import expm

from oracle import jvmc_oracle as O


def test_stats_known_answers(fixtures):
    """tests/stats_test.py:15-39."""
    p = np.ones((1, 3)) / 3
    o1 = O.SampledObs(np.array([fixtures["stats_obs1"]]), p)
    o2 = O.SampledObs(np.array([fixtures["stats_obs2"]]), p)
    assert abs(o1.mean()[0] - fixtures["stats_mean1"]) < 1e-12
    assert abs(o1.var()[0] - fixtures["stats_var1"]) < 1e-12
    assert np.allclose(o2.covar(), fixtures["stats_covar2"])
    assert np.allclose(o2.mean(), fixtures["stats_mean2"])
    assert np.allclose(o1.covar(o2), fixtures["stats_covar12"])
    assert np.allclose(o1.covar(o2), o1.covar_data(o2).mean())
    assert np.allclose(o1.covar_var(o2), o1.covar_data(o2).var())
    O_ = o2._data.reshape((-1, 2))
    assert np.allclose(o2.tangent_kernel(), O_ @ np.conj(O_.T))


def test_mpi_mean_var():
    """tests/mpi_wrapper_test.py:24-40 for one process."""
    data = np.arange(720 * 4).reshape(720, 4).astype(float)
    my, glob = O.distribute_sampling(720)
    p = np.ones((1, 720)) / glob
    assert np.sum(O.global_mean(data[None], p) - data.mean(0)) < 1e-10
    assert np.sum(O.global_variance(data[None], p) - data.var(0)) < 1e-9


def test_stepper_vs_expm():
    """tests/stepper_test.py:14-39: adaptive Heun on a linear ODE."""
    N = 4
    rs = np.random.RandomState(123)
    mat = rs.rand(N, N) + 1.j * rs.rand(N, N)
    y0 = rs.rand(N).astype(complex)

    def f(y, t, **args):
        return args["mat"].dot(y)

    def norm(y):
        return np.real(np.conj(y).dot(y))

    st = O.AdaptiveHeun()
    y = y0.copy()
    t = 0
    diffs = []
    for k in range(100):
        y, dt = st.step(t, f, y, normFunction=norm, mat=mat)
        t += dt
        diffs.append(norm(y - expm(t * mat).dot(y0)) / N)
    assert max(diffs) < 1e-5


def test_fermion_energy(fixtures):
    """tests/operator_test.py:189-254: Jordan-Wigner signs of the branch-free
    expansion pinned by the reference's fermion energy."""
    t, mu, V, L, flavour = -1.0, -2.0, 4.0, 4, 2
    fL = flavour * L
    H = O.BranchFreeOperator()
    up, do = 0, fL - 1
    for i in range(L):
        H.add(O.scal_opstr(V, (O.number(up + i), O.number(do - i))))
        H.add(O.scal_opstr(mu, (O.number(up + i),)))
        H.add(O.scal_opstr(mu, (O.number(do - i),)))
        if i == L - 1:
            continue
        H.add(O.scal_opstr(t, (O.creation(up + i + 1), O.annihilation(up + i))))
        H.add(O.scal_opstr(t, (O.creation(up + i), O.annihilation(up + i + 1))))
        H.add(O.scal_opstr(t, (O.creation(do - i - 1), O.annihilation(do - i))))
        H.add(O.scal_opstr(t, (O.creation(do - i), O.annihilation(do - i - 1))))
    tab = np.array(fixtures["fermion_table_re"]) + 1j * np.array(fixtures["fermion_table_im"])
    psi = O.NQS(O.LookupNet(fL), {"kernel": tab})
    es = O.ExactSampler(psi, (fL,))
    s, lp, p = es.sample()
    E = O.global_mean(H.get_O_loc(s, psi, lp)[..., None], p)[0]
    assert abs(E - fixtures["fermion_energy"]) < 1e-7


def test_nonzeros_closed_form():
    """tests/operator_test.py:48-68: S+ local estimator closed form."""
    rng = np.random.default_rng(3)
    s = rng.integers(0, 2, (1, 24, 4)).astype(np.int32)
    h = O.BranchFreeOperator()
    for i in range(3):
        h.add(O.scal_opstr(2., (O.Sp(i),)))
    sp, m = h.get_s_primes(s)
    tmp = h.get_O_loc_unbatched(np.ones(s.shape[:-1]), np.ones(sp.shape[:-1]))
    assert np.sum(np.abs(tmp - 2. * np.sum(-(s[..., :3] - 1), axis=-1))) < 1e-7


def _rbm_L4(weights):
    psi = O.NQS(O.CpxRBM(2, False), {"kernel": np.zeros((4, 2), complex)})
    psi.set_parameters(np.array(weights))
    return psi


def test_time_evolution_refZZ(fixtures):
    """tests/tdvp_test.py:59-128: exact-sampler real-time TDVP, ZZ(t) within 1e-3."""
    L = 4
    psi = _rbm_L4(fixtures["rbm_L4_M2_weights"])
    H = O.tfim(L, 1.0, 0.3)
    ZZ = O.BranchFreeOperator()
    for l in range(L):
        ZZ.add((O.Sz(l), O.Sz((l + 1) % L)))
    es = O.ExactSampler(psi, L)
    st = O.AdaptiveHeun(timeStep=1e-3, tol=1e-5)
    td = O.TDVP(es, snrTol=1, pinvTol=0.0, pinvCutoff=1e-8, rhsPrefactor=1.j, diagonalShift=0., makeReal='imag')
    t = 0
    times, obs = [0], []
    m = O.measure({'E': H, 'ZZ': ZZ}, psi, es)
    obs.append([m['E']['mean'][0], m['ZZ']['mean'][0]])
    while t < 0.5:
        dp, dt = st.step(0, td, psi.get_parameters(), hamiltonian=H, psi=psi, numSamples=0)
        psi.set_parameters(dp)
        t += dt
        times.append(t)
        m = O.measure({'E': [(H, t)], 'ZZ': ZZ}, psi, es)
        obs.append([m['E']['mean'][0], m['ZZ']['mean'][0]])
    obs = np.array(obs)
    assert np.max(np.abs((obs[:, 0] - obs[0, 0]) / obs[0, 0])) < 1e-3
    zz = interp1d(np.array(times), obs[:, 1])(np.arange(0, 0.5, 0.05))
    ref = np.array(fixtures["tdvp_refZZ"])
    assert np.max(np.abs(zz - ref[:len(zz)])) < 1e-3


@pytest.mark.parametrize("k", [0, 1])
def test_gs_search(fixtures, k):
    """tests/tdvp_test.py:26-56: ground-state search to the exact energy (1e-3)."""
    hx, exE = fixtures["tdvp_gs_hxs"][k], fixtures["tdvp_exEs"][k]
    rng = np.random.default_rng(1234)
    psi = O.NQS(O.CpxRBM(6, False), O.init_cpx_rbm(4, 6, False, rng, dist="uniform"))
    H = O.tfim(4, 1.0, -hx)
    es = O.ExactSampler(psi, 4)
    td = O.TDVP(es, snrTol=1, pinvTol=0.0, pinvCutoff=1e-8, rhsPrefactor=1., diagonalShift=2, makeReal='real')
    O.ground_state_search(psi, H, td, es, numSteps=100, stepSize=5e-2)
    E = O.measure({'energy': H}, psi, es)['energy']['mean'][0]
    assert abs((E - exE) / exE) < 1e-3
    assert abs(np.linalg.eigvalsh(O.hamiltonian_matrix(H, 4))[0] - exE) < 1e-7


def test_cnn_translation_invariance_and_gradient():
    """tests/nets_test.py:16-46 (periodic CNN) and a finite-difference check
    of the oracle's hand-written CNN gradient."""
    rng = np.random.default_rng(0)
    net = O.CNN(F=(3, 3), channels=(3, 2, 5), strides=(1, 1), actFun=("poly6",))
    params = {k: rng.normal(0, 0.3, s) for k, s in net.leaf_shapes((4, 4))}
    S0 = np.array([[1, 0, 1, 1], [0, 1, 1, 1], [0, 0, 1, 0], [1, 0, 0, 1]])
    S = np.array([np.roll(np.roll(S0, -i, 0), -j, 1) for i in range(4) for j in range(4)])
    v = net.apply(params, S)
    assert np.max(np.abs(v - v[0])) < 1e-12
    g = net.grad(params, S[:3])
    eps = 1e-6
    for k, p in params.items():
        for idx in [(0,) * p.ndim, tuple(d - 1 for d in p.shape)]:
            pp = {kk: vv.copy() for kk, vv in params.items()}
            pp[k][idx] += eps
            pm = {kk: vv.copy() for kk, vv in params.items()}
            pm[k][idx] -= eps
            fd = (net.apply(pp, S[:3]) - net.apply(pm, S[:3])) / (2 * eps)
            flat = np.ravel_multi_index(idx, p.shape)
            assert np.allclose(g[k][:, flat], fd, atol=1e-7)


def test_exact_sampler_energy_matches_ed():
    """ExactSampler energy of an RBM equals <psi|H|psi>/<psi|psi> from the
    dense Hamiltonian (independent check of the branch-free expansion)."""
    rng = np.random.default_rng(5)
    L = 6
    psi = O.NQS(O.CpxRBM(5, True), O.init_cpx_rbm(L, 5, True, rng, scale=0.3))
    for H in [O.tfim(L, 1.0, 0.7), O.xxz(L, 1.5)]:
        es = O.ExactSampler(psi, L)
        s, lp, p = es.sample()
        E = O.global_mean(H.get_O_loc(s, psi, lp)[..., None], p)[0]
        v = np.exp(lp[0])
        Hm = O.hamiltonian_matrix(H, L)
        assert abs(E - np.vdot(v, Hm @ v) / np.vdot(v, v)) < 1e-10


@pytest.mark.parametrize("k", [0, 1])
def test_minsr_gs_search(fixtures, k):
    """tests/minsr_test.py:15-43: MinSR ground-state search to exEs (1e-3)."""
    hx, exE = fixtures["tdvp_gs_hxs"][k], fixtures["tdvp_exEs"][k]
    rng = np.random.default_rng(1234)
    psi = O.NQS(O.CpxRBM(8, False), O.init_cpx_rbm(4, 8, False, rng, dist="uniform"))
    H = O.tfim(4, 1.0, -hx)
    es = O.ExactSampler(psi, 4)
    solver = O.MinSR(es, pinvTol=1e-6, diagonalShift=0.)
    O.ground_state_search(psi, H, solver, es, numSteps=200, stepSize=1e-2)
    E = O.measure({'energy': H}, psi, es)['energy']['mean'][0]
    assert abs((E - exE) / exE) < 1e-3
