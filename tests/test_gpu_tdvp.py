"""TDVP right-hand side of the CUDA path against the oracle and against the
reference test-suite's fixtures.

Energy and variance: 1e-10 relative (FP64).  Update dtheta: 1e-10 relative,
or 10x the conditioning floor of the solve where that is larger.  The floor
is measured, not assumed: the oracle's own update is recomputed with every
entry of S changed by one unit in the last place (relative 2^-52, two random
symmetric patterns) and the larger relative change of dtheta is the floor.
For the 10-site workload with N(0, 0.01^2) weights the floor is ~1e-7
(eigenvalues span 4e-11..1.8e-2 and the cutoff loop runs to 1e-8), so no
FP64 implementation can hold 1e-10 there."""

import numpy as np
import pytest
import torch
from scipy.interpolate import interp1d

from oracle import jvmc_oracle as O

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def _pair(L, M, bias, scale, seed=0):
    import vmc_jax_gb300 as V
    rng = np.random.default_rng(seed)
    prm = {}
    if bias:
        prm["bias"] = rng.normal(0, scale, M) + 1j * rng.normal(0, scale, M)
    prm["kernel"] = rng.normal(0, scale, (L, M)) + 1j * rng.normal(0, scale, (L, M))
    opsi = O.NQS(O.CpxRBM(M, bias), prm)
    psi = V.vqs.NQS(V.nets.CpxRBM(numHidden=M, bias=bias))
    psi(np.zeros((1, 1, L), np.int32))
    psi.set_parameters(opsi.get_parameters())
    return psi, opsi


def _tfim(V, L, J, h):
    H = V.operator.BranchFreeOperator()
    for l in range(L):
        H.add(V.operator.scal_opstr(-J, (V.operator.Sz(l), V.operator.Sz((l + 1) % L))))
        H.add(V.operator.scal_opstr(-h, (V.operator.Sx(l),)))
    return H


def _conditioning_floor(opsi, Ho, L, makeReal, rhs, tho):
    """Largest relative change of the oracle's Euler update when S is
    perturbed by one ulp (two patterns)."""
    eso = O.ExactSampler(opsi, L)
    base = O.Euler(timeStep=0.01).step(0, O.TDVP(eso, makeReal=makeReal, rhsPrefactor=rhs, pinvCutoff=1e-8), tho,
                                       hamiltonian=Ho, psi=opsi)[0] - tho
    floor = 0.0
    for seed in (1, 2):
        td = O.TDVP(eso, makeReal=makeReal, rhsPrefactor=rhs, pinvCutoff=1e-8, perturbS=(2.0 ** -52, seed))
        moved = O.Euler(timeStep=0.01).step(0, td, tho, hamiltonian=Ho, psi=opsi)[0] - tho
        floor = max(floor, _rel(moved, base))
    opsi.set_parameters(tho)
    return floor


@pytest.mark.parametrize("scale", [0.01, 0.1, 0.3])
@pytest.mark.parametrize("makeReal,rhs", [("real", 1.0), ("imag", 1.j)])
def test_exact_euler_step(cuda, scale, makeReal, rhs):
    """The 10-site TFIM workload: ExactSampler, FP64, one Euler step of 0.01."""
    import vmc_jax_gb300 as V
    L, M = 10, 20
    psi, opsi = _pair(L, M, True, scale)
    H = _tfim(V, L, 1.0, 0.7)
    Ho = O.tfim(L, 1.0, 0.7)
    es = V.sampler.ExactSampler(psi, L)
    eso = O.ExactSampler(opsi, L)
    td = V.util.TDVP(es, makeReal=makeReal, rhsPrefactor=rhs, pinvCutoff=1e-8)
    tdo = O.TDVP(eso, makeReal=makeReal, rhsPrefactor=rhs, pinvCutoff=1e-8)
    stp, stpo = V.util.stepper.Euler(timeStep=0.01), O.Euler(timeStep=0.01)
    th, tho = psi.get_parameters(), opsi.get_parameters()
    new, _ = stp.step(0, td, th, hamiltonian=H, psi=psi)
    newo, _ = stpo.step(0, tdo, tho, hamiltonian=Ho, psi=opsi)
    assert abs(complex(td.ElocMean0) - tdo.ElocMean0) / abs(tdo.ElocMean0) < 1e-10
    assert abs(float(td.ElocVar0) - tdo.ElocVar0) / abs(tdo.ElocVar0) < 1e-10
    dth = (new - th).cpu().numpy()
    floor = _conditioning_floor(opsi, Ho, L, makeReal, rhs, tho)
    tol = max(1e-10, 10.0 * floor)
    err = _rel(dth, newo - tho)
    print("scale %g %s: dtheta error %.2e, conditioning floor %.2e, bar %.2e" % (scale, makeReal, err, floor, tol))
    assert err <= tol
    md, mdo = td.get_metadata(), tdo.metaData
    assert _rel(md["spectrum"].cpu().numpy(), mdo["spectrum"]) < 1e-9
    assert abs(float(md["tdvp_residual"]) - mdo["tdvp_residual"]) <= 1e-6 * max(mdo["tdvp_residual"], 1e-12) + 1e-14
    assert abs(float(md["pinv_cutoff"]) - mdo["pinv_cutoff"]) < 1e-20
    assert abs(float(md["tdvp_error"]) - mdo["tdvp_error"]) < 1e-6 * max(1.0, abs(mdo["tdvp_error"]))


def test_time_evolution_refZZ(cuda, fixtures):
    """tests/tdvp_test.py:59-128 through the CUDA path: ZZ(t) within 1e-3 of
    the reference series, energy drift < 1e-3, and 1e-7 of the oracle."""
    import vmc_jax_gb300 as V
    L = 4
    w = np.array(fixtures["rbm_L4_M2_weights"])
    psi = V.vqs.NQS(V.nets.CpxRBM(2, False))
    psi(np.ones((1, 1, 4), np.int32))
    psi.set_parameters(w)
    H = _tfim(V, L, 1.0, 0.3)
    ZZ = V.operator.BranchFreeOperator()
    for l in range(L):
        ZZ.add((V.operator.Sz(l), V.operator.Sz((l + 1) % L)))
    es = V.sampler.ExactSampler(psi, L)
    st = V.util.stepper.AdaptiveHeun(timeStep=1e-3, tol=1e-5)
    td = V.util.TDVP(es, snrTol=1, pinvTol=0.0, pinvCutoff=1e-8, rhsPrefactor=1.j, diagonalShift=0., makeReal='imag')
    t = 0
    times, obs = [0], []
    m = V.util.measure({'E': H, 'ZZ': ZZ}, psi, es)
    obs.append([float(m['E']['mean'][0]), float(m['ZZ']['mean'][0])])
    while t < 0.5:
        dp, dt = st.step(0, td, psi.get_parameters(), hamiltonian=H, psi=psi, numSamples=0)
        psi.set_parameters(dp)
        t += dt
        times.append(t)
        m = V.util.measure({'E': [(H, t)], 'ZZ': ZZ}, psi, es)
        obs.append([float(m['E']['mean'][0]), float(m['ZZ']['mean'][0])])
    obs = np.array(obs)
    assert np.max(np.abs((obs[:, 0] - obs[0, 0]) / obs[0, 0])) < 1e-3
    zz = interp1d(np.array(times), obs[:, 1])(np.arange(0, 0.5, 0.05))
    ref = np.array(fixtures["tdvp_refZZ"])
    assert np.max(np.abs(zz - ref[:len(zz)])) < 1e-3


@pytest.mark.parametrize("k", [0, 1])
def test_gs_search(cuda, fixtures, k):
    """tests/tdvp_test.py:26-56: ground-state energy within 1e-3."""
    import vmc_jax_gb300 as V
    hx, exE = fixtures["tdvp_gs_hxs"][k], fixtures["tdvp_exEs"][k]
    psi = V.vqs.NQS(V.nets.CpxRBM(numHidden=6, bias=False))
    H = _tfim(V, 4, 1.0, -hx)
    es = V.sampler.ExactSampler(psi, 4)
    td = V.util.TDVP(es, snrTol=1, pinvTol=0.0, pinvCutoff=1e-8, rhsPrefactor=1., diagonalShift=2, makeReal='real')
    V.util.ground_state_search(psi, H, td, es, numSteps=100, stepSize=5e-2)
    E = float(V.util.measure({'energy': H}, psi, es)['energy']['mean'][0])
    assert abs((E - exE) / exE) < 1e-3


@pytest.mark.parametrize("makeReal,rhs,mode", [("imag", 1.j, "reference"), ("real", 1.0, "pair")])
def test_mc_rhs_same_samples(cuda, makeReal, rhs, mode):
    """MCSampler + SNR regulariser: the same Philox chains on both sides, so
    both solve the same sampled equation (FP64)."""
    import vmc_jax_gb300 as V
    L, M = 8, 6
    psi, opsi = _pair(L, M, True, 0.2, seed=4)
    H = _tfim(V, L, 1.0, 0.7)
    Ho = O.tfim(L, 1.0, 0.7)
    mc = V.sampler.MCSampler(psi, (L,), 77, updateProposer=V.sampler.propose_spin_flip, numChains=64,
                             numSamples=2048, thermalizationSweeps=4, sweepSteps=L)
    mco = O.MCSampler(opsi, (L,), 77, numChains=64, numSamples=2048, thermalizationSweeps=4, sweepSteps=L)
    td = V.util.TDVP(mc, makeReal=makeReal, rhsPrefactor=rhs, pinvCutoff=1e-8, snrTol=2)
    tdo = O.TDVP(mco, makeReal=makeReal, rhsPrefactor=rhs, pinvCutoff=1e-8, snrTol=2, snrMode=mode)
    u = td(psi.get_parameters(), 0., psi=psi, hamiltonian=H, intStep=0).cpu().numpy()
    uo = tdo(opsi.get_parameters(), 0., psi=opsi, hamiltonian=Ho, intStep=0)
    assert abs(complex(td.ElocMean0) - tdo.ElocMean0) / abs(tdo.ElocMean0) < 1e-10
    assert _rel(u, uo) < 1e-8
    assert _rel(td.get_snr().cpu().numpy(), tdo.metaData["SNR"]) < 1e-6 if mode == "reference" else True


def test_cross_validation_runs(cuda):
    import vmc_jax_gb300 as V
    L, M = 8, 6
    psi, opsi = _pair(L, M, True, 0.2, seed=4)
    H = _tfim(V, L, 1.0, 0.7)
    mc = V.sampler.MCSampler(psi, (L,), 5, updateProposer=V.sampler.propose_spin_flip, numChains=64,
                             numSamples=2048, thermalizationSweeps=4, sweepSteps=L)
    td = V.util.TDVP(mc, makeReal="imag", rhsPrefactor=1.j, crossValidation=True)
    td(psi.get_parameters(), 0., psi=psi, hamiltonian=H, intStep=0)
    md = td.get_metadata()
    assert np.isfinite(float(md["tdvp_residual_cross_validation_ratio"]))
    assert np.isfinite(float(md["tdvp_error_cross_validation_ratio"]))


@pytest.mark.parametrize("k", [0, 1])
def test_minsr_gs_search(cuda, fixtures, k):
    """tests/minsr_test.py:15-43 through the CUDA path (exEs within 1e-3)."""
    import vmc_jax_gb300 as V
    hx, exE = fixtures["tdvp_gs_hxs"][k], fixtures["tdvp_exEs"][k]
    psi = V.vqs.NQS(V.nets.CpxRBM(numHidden=8, bias=False), seed=1234)
    H = _tfim(V, 4, 1.0, -hx)
    es = V.sampler.ExactSampler(psi, 4)
    solver = V.util.MinSR(es, pinvTol=1e-6, diagonalShift=0.)
    V.util.ground_state_search(psi, H, solver, es, numSteps=200, stepSize=1e-2)
    E = float(V.util.measure({'energy': H}, psi, es)['energy']['mean'][0])
    assert abs((E - exE) / exE) < 1e-3


def test_minsr_update_matches_oracle(cuda):
    import vmc_jax_gb300 as V
    psi, opsi = _pair(8, 6, True, 0.2, seed=9)
    H = _tfim(V, 8, 1.0, 0.9)
    es = V.sampler.ExactSampler(psi, 8)
    eso = O.ExactSampler(opsi, 8)
    u = V.util.MinSR(es, pinvTol=1e-8)(psi.get_parameters(), 0., psi=psi, hamiltonian=H, intStep=0)
    uo = O.MinSR(eso, pinvTol=1e-8)(opsi.get_parameters(), 0., psi=opsi, hamiltonian=O.tfim(8, 1.0, 0.9),
                                    intStep=0)
    assert _rel(u.cpu().numpy(), uo) < 1e-8


def test_checkpoint_resume_reproduces_the_run(cuda, tmp_path):
    """save_checkpoint after two steps; the resumed run (fresh objects) makes
    the same next two steps as the uninterrupted one, bit for bit (chains and
    random-stream position restored)."""
    import vmc_jax_gb300 as V

    def make():
        psi, _ = _pair(8, 6, True, 0.2, seed=31)
        mc = V.sampler.MCSampler(psi, (8,), 5, updateProposer=V.sampler.propose_spin_flip, numChains=32,
                                 numSamples=512, thermalizationSweeps=2, sweepSteps=8)
        td = V.util.TDVP(mc, makeReal="real", rhsPrefactor=1., pinvCutoff=1e-8, snrTol=2)
        return psi, mc, td, V.util.stepper.AdaptiveHeun(timeStep=1e-3, tol=1e-3)

    H = _tfim(V, 8, 1.0, 0.7)

    def steps(psi, td, st, n):
        out = []
        for _ in range(n):
            th, dt = st.step(0, td, psi.get_parameters(), hamiltonian=H, psi=psi, numSamples=512)
            psi.set_parameters(th)
            out.append(th.cpu().numpy())
        return out

    psi, mc, td, st = make()
    steps(psi, td, st, 2)
    path = str(tmp_path / "ckpt.pt")
    V.util.save_checkpoint(path, psi, mc, st, t=0.5)
    ref = steps(psi, td, st, 2)
    psi2, mc2, td2, st2 = make()
    assert V.util.load_checkpoint(path, psi2, mc2, st2) == 0.5
    got = steps(psi2, td2, st2, 2)
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)


def test_minsr_mixed_tangent_kernel(cuda):
    """MinSR with the tangent kernel on the tcgen05 BF16x3 Gram kernel: the
    kernel matrix against the FP64 product of the same samples (2e-5
    relative to its largest entry, the FP32-accumulation bar of the Gram
    kernel's own test), and the update against the FP64 MinSR at the same
    pseudo-inverse tolerance (1e-3: the pseudo-inverse amplifies the S-level
    error by the spread of the retained eigenvalues, 1e3 here)."""
    import vmc_jax_gb300 as V
    from vmc_jax_gb300.util.minsr import tangent_kernel_mixed
    g = torch.Generator(device=cuda).manual_seed(2)
    X = (torch.randn(300, 700, dtype=torch.complex64, device=cuda, generator=g) * 0.1)
    T = tangent_kernel_mixed(X)
    Xd = X.to(torch.complex128)
    ref = Xd @ Xd.mH
    assert ((T - ref).abs().max() / ref.abs().max()).item() < 2e-5
    psi, opsi = _pair(8, 6, True, 0.2, seed=9)
    H = _tfim(V, 8, 1.0, 0.9)
    es = V.sampler.ExactSampler(psi, 8)
    u64 = V.util.MinSR(es, pinvTol=1e-3)(psi.get_parameters(), 0., psi=psi, hamiltonian=H, intStep=0)
    psi.precision = "fp32"
    psi._touch()
    um = V.util.MinSR(es, pinvTol=1e-3, precision="mixed")(psi.get_parameters(), 0., psi=psi, hamiltonian=H,
                                                          intStep=0)
    assert _rel(um.cpu().numpy(), u64.cpu().numpy()) < 1e-3
