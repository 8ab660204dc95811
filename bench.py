#!/usr/bin/env python
"""Benchmark: TDVP steps/s of the per-step VMC hot path on one GB300.

Workload (default): transverse-field Ising chain L = 64, periodic, J = 1,
h = 1.0; CpxRBM with 256 hidden units and bias (16,640 complex parameters),
parameters N(0, 0.01^2) from seed 0; MCSampler with 1024 chains, single
spin flips, 64 thermalisation sweeps of L proposals, 16 samples per chain
(N_s = 16,384); TDVP imaginary time (makeReal='real', rhsPrefactor=1,
pinvCutoff=1e-8, snrTol=2) in the mixed form (FP32 sampling / E_loc
kernels, BF16x3 tcgen05 S and SNR contractions, FP64 statistics, FP32
eigendecomposition with the eigenpairs that carry the solve refined to FP64
accuracy, FP64 solve); one Euler step dtau = 0.01 per step.  Inputs are
synthetic and seeded; there is no dataset.

``--impl reference`` times the CPU restatement of jVMC's algorithm (the
oracle; jVMC itself needs JAX, which is not installed) on the host cores on a
bounded sample of the same step, extrapolated to one full step.
"""

import argparse
import atexit
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

WORKLOADS = {
    "ising64_rbm256_mcmc16k": dict(L=64, M=256, J=1.0, h=1.0, chains=1024, therm=64, per_chain=16, dt=0.01,
                                   sampler="mc"),
    "ising10_rbm20_exact": dict(L=10, M=20, J=1.0, h=0.7, dt=0.01, sampler="exact"),
    "ising10x10_cnn8x8_mcmc32k": dict(Lx=10, Ly=10, J=1.0, h=3.0, chains=4096, therm=10, per_chain=8, dt=0.01,
                                       sampler="mc", net="cnn"),
    "ising64_symrbm64_mcmc16k": dict(L=64, M=64, J=1.0, h=1.0, chains=1024, therm=64, per_chain=16, dt=0.01,
                                     sampler="mc", net="symrbm", symmetries=("translation",)),
}
DEFAULT_WORKLOAD = "ising64_rbm256_mcmc16k"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp32", "fp64"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the FP64 / plain-FP32 comparison on the same samples after the timed region")
    ap.add_argument("--plain-steps", type=int, default=1,
                    help="timed steps of the plain-FP32 form (after one warm-up step) for mixed_over_fp32")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--serve", action="store_true",
                    help="serving load: Poisson stream of independent Ising jobs through vmc_jax_gb300.serving")
    ap.add_argument("--jobs", type=int, default=16)
    ap.add_argument("--rate", type=float, default=2.0, help="job arrivals per second (--serve)")
    ap.add_argument("--job-steps", type=int, default=10)
    ap.add_argument("--serve-L", default="16,24,32,48,64", help="lattice sizes of the served jobs")
    ap.add_argument("--serve-m-over-l", default="1,2,4", help="hidden units per site of the served jobs")
    ap.add_argument("--serve-ns-exp", default="11,14", help="log2 of the smallest and largest sample count")
    ap.add_argument("--slots", type=int, default=8, help="resident jobs at most (serving)")
    ap.add_argument("--quench", type=float, default=None,
                    help="XXZ L=48 real-time quench with the adaptive Heun integrator up to this time: energy drift "
                         "of the mixed form and of the FP64 form")
    ap.add_argument("--quench-steps", type=int, default=100, help="step cap of each quench integration")
    ap.add_argument("--quench-wall", type=float, default=600.0, help="wall-clock cap (s) of each quench integration")
    ap.add_argument("--kernel", default=None,
                    choices=["gram", "snr", "eloc", "metropolis", "data", "hermitian", "gemv", "stats"],
                    help="time one kernel on a fixed synthetic case instead of the TDVP step (profiling)")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


# ---------------------------------------------------------------- workload
def initial_parameters(cfg):
    rng = np.random.default_rng(0)
    L, M = cfg["L"], cfg["M"]
    b = rng.normal(0, 0.01, M) + 1j * rng.normal(0, 0.01, M)
    W = rng.normal(0, 0.01, (L, M)) + 1j * rng.normal(0, 0.01, (L, M))
    return np.concatenate([b.real, b.imag, W.real.ravel(), W.imag.ravel()])


def build_cnn(cfg, precision):
    """10x10 TFIM with a real CNN (3x3 filters, 8 and 8 channels, x^2/2 - x^4/12,
    bias on the second layer), He-normal parameters from seed 0, MCSampler."""
    import vmc_jax_gb300 as V
    Lx, Ly = cfg["Lx"], cfg["Ly"]
    net = V.nets.CNN(F=(3, 3), channels=(8, 8), strides=(1, 1), actFun=(V.nets.activation_functions.poly4,))
    psi = V.vqs.NQS(net, precision="fp64" if precision == "fp64" else "fp32")
    psi(np.zeros((1, 1, Lx, Ly), np.int32))
    rng = np.random.default_rng(0)
    theta = []
    for name, shape in net.leaf_shapes((Lx, Ly)):
        if name.endswith("bias"):
            theta.append(np.zeros(shape).ravel())
        else:
            fan_in = int(np.prod(shape[:-1]))
            theta.append(rng.normal(0, np.sqrt(2.0 / fan_in), shape).ravel())
    psi.set_parameters(np.concatenate(theta))
    H = V.operator.BranchFreeOperator()
    for y in range(Ly):
        for x in range(Lx):
            i = y * Lx + x
            H.add(V.operator.scal_opstr(-cfg["J"], (V.operator.Sz(i), V.operator.Sz(y * Lx + (x + 1) % Lx))))
            H.add(V.operator.scal_opstr(-cfg["J"], (V.operator.Sz(i), V.operator.Sz(((y + 1) % Ly) * Lx + x))))
            H.add(V.operator.scal_opstr(-cfg["h"], (V.operator.Sx(i),)))
    ns = cfg["chains"] * cfg["per_chain"]
    sampler = V.sampler.MCSampler(psi, (Lx, Ly), 0, updateProposer=V.sampler.propose_spin_flip,
                                  numChains=cfg["chains"], numSamples=ns, thermalizationSweeps=cfg["therm"],
                                  sweepSteps=Lx * Ly)
    tdvp = V.util.TDVP(sampler, makeReal="real", rhsPrefactor=1., pinvCutoff=1e-8, snrTol=2, precision=precision)
    stepper = V.util.stepper.Euler(timeStep=cfg["dt"])
    P = sum(int(np.prod(sh)) for _, sh in net.leaf_shapes((Lx, Ly)))
    return dict(V=V, psi=psi, H=H, sampler=sampler, tdvp=tdvp, stepper=stepper, ns=ns, P=P)


def build(cfg, precision):
    import vmc_jax_gb300 as V
    if cfg.get("net") == "cnn":
        return build_cnn(cfg, precision)
    L, M = cfg["L"], cfg["M"]
    orbit = None
    if cfg.get("net") == "symrbm":
        orbit = V.util.symmetries.get_orbit_1D(L, *cfg["symmetries"])
    psi = V.vqs.NQS(V.nets.CpxRBM(numHidden=M, bias=True), orbit=orbit,
                    precision="fp64" if precision == "fp64" else "fp32")
    psi(np.zeros((1, 1, L), np.int32))
    psi.set_parameters(initial_parameters(cfg))
    H = V.operator.BranchFreeOperator()
    for l in range(L):
        H.add(V.operator.scal_opstr(-cfg["J"], (V.operator.Sz(l), V.operator.Sz((l + 1) % L))))
        H.add(V.operator.scal_opstr(-cfg["h"], (V.operator.Sx(l),)))
    if cfg["sampler"] == "mc":
        ns = cfg["chains"] * cfg["per_chain"]
        sampler = V.sampler.MCSampler(psi, (L,), 0, updateProposer=V.sampler.propose_spin_flip,
                                      numChains=cfg["chains"], numSamples=ns, thermalizationSweeps=cfg["therm"],
                                      sweepSteps=L)
    else:
        ns = 2 ** L
        sampler = V.sampler.ExactSampler(psi, L)
    tdvp = V.util.TDVP(sampler, makeReal="real", rhsPrefactor=1., pinvCutoff=1e-8, snrTol=2, precision=precision)
    stepper = V.util.stepper.Euler(timeStep=cfg["dt"])
    return dict(V=V, psi=psi, H=H, sampler=sampler, tdvp=tdvp, stepper=stepper, ns=ns, P=L * M + M)


def one_step(ctx, theta):
    new, _ = ctx["stepper"].step(0, ctx["tdvp"], theta, hamiltonian=ctx["H"], psi=ctx["psi"],
                                 numSamples=ctx["ns"])
    ctx["psi"].set_parameters(new)
    return new


def accuracy_block(ctx):
    """Relative errors of the mixed form (BF16x3 S/SNR; and, as a study, plain
    BF16 S/SNR: "mixed_bf16x1") and of the plain-FP32 form against the FP64
    form on one common sample: energy and variance of E_loc, S (the complex
    P x P matrix A, Frobenius norm), F (covar(O, E)), and the update dtheta
    (l2 norm and largest entry).  Every form runs its own E_loc kernels
    (FP64 or FP32) and its own S build, eigendecomposition and solve on the
    same configurations and weights."""
    import torch
    V, psi, H, smp = ctx["V"], ctx["psi"], ctx["H"], ctx["sampler"]
    configs, _, p = smp.sample()
    keep = psi.precision
    ref, errs = None, {}

    def rel(a, b):
        return float(torch.linalg.norm((a - b).reshape(-1)) / torch.linalg.norm(b.reshape(-1)))

    for form in ("fp64", "mixed", "mixed_bf16x1", "fp32"):
        prec = "mixed" if form.startswith("mixed") else form
        td = V.util.TDVP(smp, makeReal="real", rhsPrefactor=1., pinvCutoff=1e-8, snrTol=2, precision=prec)
        if form == "mixed_bf16x1":
            td.splitProducts = 1
        psi.precision = "fp64" if prec == "fp64" else "fp32"
        psi._touch()
        E = V.operator.BranchFreeOperator.get_O_loc_fused(H, configs, psi, None, 0.)
        u, res, cut = td._complex_rhs(psi, configs, E, p)
        cur = {"u": u.detach().clone(), "A": td._A, "f": td._covOE.clone(), "E": complex(td.ElocMean),
               "var": float(td.ElocVar), "cutoff": float(cut), "residual": float(res)}
        if ref is None:
            ref = cur
            continue
        errs[form] = {"energy": abs(cur["E"] - ref["E"]) / abs(ref["E"]),
                      "variance": abs(cur["var"] - ref["var"]) / abs(ref["var"]),
                      "S": rel(cur["A"], ref["A"]), "F": rel(cur["f"], ref["f"]),
                      "dtheta": rel(cur["u"], ref["u"]),
                      "dtheta_max": float((cur["u"] - ref["u"]).abs().max() / ref["u"].abs().max()),
                      "pinv_cutoff": cur["cutoff"]}
        if prec == "mixed":
            errs[form]["eigensolver"] = td.refineInfo
        del cur
        torch.cuda.empty_cache()
    psi.precision = keep
    psi._touch()
    errs["fp64_pinv_cutoff"] = ref["cutoff"]
    return errs


def plain_fp32_steps_per_s(cfg, steps):
    """Steps/s of the plain-FP32 form (FP32 kernels, cuBLAS complex64 GEMMs,
    FP64 eigendecomposition by cuSOLVER) on the same workload, CUDA events
    over ``steps`` steps after one warm-up step."""
    import torch
    ctx = build(cfg, "fp32")
    theta = ctx["psi"].get_parameters()
    theta = one_step(ctx, theta)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        theta = one_step(ctx, theta)
    e1.record()
    torch.cuda.synchronize()
    return steps / (e0.elapsed_time(e1) / 1000.0)


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clock / throttle samples every 200 ms while active."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
            # the sampler never outlives this process, also when a step raises
            atexit.register(self._kill)
        except Exception:
            self.proc = None

    def _kill(self):
        if self.proc is not None and self.proc.poll() is None:
            self.proc.kill()

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.file.flush()
        rows = []
        with open(self.file.name) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ----------------------------------------------------------- CPU baseline
def cpu_step_seconds(cfg, budget_note):
    """Seconds of one full TDVP step of the oracle (CPU FP64 restatement of
    jVMC's algorithm), measured on bounded samples and extrapolated:
    Metropolis by chain-steps, E_loc and gradients by samples, the S build
    and SNR contraction by N_s * n^2 (GEMM rate at a smaller n), the 2P
    eigendecomposition by n^3 (LAPACK at a smaller n)."""
    from oracle import jvmc_oracle as O
    if cfg.get("net") == "cnn":
        return cnn_cpu_step_seconds(cfg)
    L, M = cfg["L"], cfg["M"]
    rng = np.random.default_rng(0)
    prm = O.init_cpx_rbm(L, M, True, rng, scale=0.01)
    sym = cfg.get("net") == "symrbm"
    if sym:
        orbit, factor = O.get_orbit_1D(L, *cfg["symmetries"])
        psi = O.NQS(O.SymNet(O.CpxRBM(M, True), orbit, factor), prm)
    else:
        psi = O.NQS(O.CpxRBM(M, True), prm)
    H = O.tfim(L, cfg["J"], cfg["h"])
    P2 = 2 * (L * M + M)
    out = {}
    if cfg["sampler"] == "mc":
        Ns = cfg["chains"] * cfg["per_chain"]
        chain_steps = cfg["chains"] * (cfg["therm"] + cfg["per_chain"]) * L
        C = 64 if sym else cfg["chains"]
        mc = O.MCSampler(psi, (L,), 0, numChains=C, numSamples=C, thermalizationSweeps=0, sweepSteps=L)
        t0 = time.perf_counter()
        mc.sample(numSamples=C)
        out["sampling"] = (time.perf_counter() - t0) / (C * L) * chain_steps
    else:
        Ns = 2 ** L
        out["sampling"] = 0.0
    n_s = (64 if sym else 512) if cfg["sampler"] == "mc" else min(Ns, 256)
    s = rng.integers(0, 2, (1, n_s, L)).astype(np.int32)
    t0 = time.perf_counter()
    H.get_O_loc(s, psi)
    out["eloc"] = (time.perf_counter() - t0) / n_s * Ns
    t0 = time.perf_counter()
    psi.gradients(s)
    out["gradients"] = (time.perf_counter() - t0) / n_s * Ns
    # complex GEMM rate (S0 = conj(O)^T O over samples) at n' = 4096, K' = 2048
    a = rng.normal(size=(2048, 4096)) + 1j * rng.normal(size=(2048, 4096))
    t0 = time.perf_counter()
    np.tensordot(np.conj(a), a, axes=(0, 0))
    rate = 8.0 * 2048 * 4096 * 4096 / (time.perf_counter() - t0)
    out["s_build"] = 8.0 * Ns * P2 * P2 / rate
    out["snr"] = 8.0 * Ns * P2 * P2 / rate
    # real symmetric eigh of the 2P representation, n^3 scaling from n' = 4096
    x = rng.normal(size=(4096, 4096))
    S = x @ x.T
    t0 = time.perf_counter()
    np.linalg.eigh(S)
    out["eigh"] = (time.perf_counter() - t0) * (P2 / 4096.0) ** 3
    total = sum(out.values())
    return total, out


def cnn_cpu_step_seconds(cfg):
    """Oracle CNN step on bounded samples: Metropolis with 64 chains x one sweep,
    E_loc and gradients of 64 samples, a 656^2 x N_s S build (GEMM rate) and a
    656^2 eigh, extrapolated to the full step."""
    from oracle import jvmc_oracle as O
    Lx, Ly = cfg["Lx"], cfg["Ly"]
    net = O.CNN(F=(3, 3), channels=(8, 8), strides=(1, 1), actFun=("poly4",))
    rng = np.random.default_rng(0)
    prm = {k: rng.normal(0, 0.3, sh) for k, sh in net.leaf_shapes((Lx, Ly))}
    psi = O.NQS(net, prm)
    H = O.tfim(Lx * Ly, cfg["J"], cfg["h"], lattice=(Lx, Ly))
    Ns = cfg["chains"] * cfg["per_chain"]
    n = Lx * Ly
    chain_steps = cfg["chains"] * (cfg["therm"] + cfg["per_chain"]) * n
    out = {}
    C = 64
    mc = O.MCSampler(psi, (Lx, Ly), 0, numChains=C, numSamples=C, thermalizationSweeps=0, sweepSteps=n)
    t0 = time.perf_counter()
    mc.sample(numSamples=C)
    out["sampling"] = (time.perf_counter() - t0) / (C * n) * chain_steps
    s = rng.integers(0, 2, (1, 64, Lx, Ly)).astype(np.int32)
    t0 = time.perf_counter()
    H.get_O_loc(s, psi)
    out["eloc"] = (time.perf_counter() - t0) / 64 * Ns
    t0 = time.perf_counter()
    g = psi.gradients(s)
    out["gradients"] = (time.perf_counter() - t0) / 64 * Ns
    P = g.shape[-1]
    a = rng.normal(size=(4096, P)) + 0j
    t0 = time.perf_counter()
    np.tensordot(np.conj(a), a, axes=(0, 0))
    out["s_build"] = (time.perf_counter() - t0) * Ns / 4096
    out["snr"] = out["s_build"]
    x = rng.normal(size=(P, P))
    t0 = time.perf_counter()
    np.linalg.eigh(x @ x.T)
    out["eigh"] = time.perf_counter() - t0
    return sum(out.values()), out


def cpu_sample_desc(cfg):
    if cfg.get("net") == "cnn":
        return ("oracle timed on: CNN Metropolis with 64 chains x one sweep, E_loc and gradients of 64 samples, "
                "a 656-wide complex GEMM over 4096 samples and the 656^2 eigh; extrapolated to one full step")
    if cfg.get("net") == "symrbm":
        return ("oracle (numpy FP64 restatement of jVMC, SymNet over %d translations) timed on: Metropolis with 64 "
                "chains x one sweep, E_loc and gradients of 64 samples, a 4096^2 x 2048 complex GEMM and a 4096^2 "
                "eigh; extrapolated to one full step" % cfg["L"])
    if cfg["sampler"] == "mc":
        return ("oracle (numpy FP64 restatement of jVMC) timed on: Metropolis of all %d chains for one sweep, "
                "E_loc and gradients of 512 samples, a 4096^2 x 2048 complex GEMM and a 4096^2 eigh; "
                "extrapolated to one full step (5.24M chain-steps, 16384 samples, 2P = 33280 GEMMs and eigh)"
                % cfg["chains"])
    return "oracle timed on 256 exact-basis samples, a 4096^2 x 2048 complex GEMM and a 4096^2 eigh, extrapolated"


# ---------------------------------------------------------- replicas (N>1)
def reduce_max_ms(ms, device=None):
    """Max over ranks of the timed region (ms); identity without a process group."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(ms)
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t[0])


def aggregate_steps_per_s(steps, world, max_ms):
    """Whole-job throughput of independent replicas: every rank ran ``steps``
    steps; the job took the slowest rank's time."""
    return world * steps / (max_ms / 1000.0)


# ------------------------------------------------------------------- main
def emit(obj):
    print(json.dumps(obj), flush=True)


EXTRAPOLATED = {
    "sampling": "all chains timed for one sweep of L proposals; the step's thermalisation + sampling sweeps are "
                "that time multiplied by the sweep count (linear work per sweep)",
    "eloc": "512 samples timed, multiplied by N_s / 512 (linear work per sample)",
    "gradients": "512 samples timed, multiplied by N_s / 512 (linear work per sample)",
    "s_build": "complex FP64 GEMM rate measured at 4096^2 x 2048, applied to the step's 8 N_s (2P)^2 flop",
    "snr": "same GEMM rate applied to the SNR transform's 8 N_s (2P)^2 flop",
    "eigh": "LAPACK real symmetric eigh timed at n = 4096, scaled by (2P / 4096)^3",
}


def gpu_config(cfg, workload, precision):
    """The config keys of the GPU arm's line for the same workload."""
    if cfg.get("net") == "cnn":
        ns = cfg["chains"] * cfg["per_chain"]
        P = 656
    else:
        ns = cfg["chains"] * cfg["per_chain"] if cfg["sampler"] == "mc" else 2 ** cfg["L"]
        P = cfg["L"] * cfg["M"] + cfg["M"]
    return {"workload": workload, "precision": precision, "num_samples": ns, "num_params_complex": P,
            "l2": "inputs larger than L2 (O_k bf16 planes %.2f GB)" % (8.0 * P * ns / 1e9),
            "parallelism": "single GPU", **cfg}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    cfg = WORKLOADS[args.workload]
    # one warm-up sample loads BLAS thread pools and pages; further ones only
    # lengthen the run (the CPU path has nothing to compile)
    for _ in range(min(args.warmup, 1)):
        cpu_step_seconds(cfg, "")
    secs, walls = [], []
    for _ in range(args.steps):
        w0 = time.perf_counter()
        t, parts = cpu_step_seconds(cfg, "")
        walls.append(time.perf_counter() - w0)
        secs.append(t)
    sec = float(np.mean(secs))
    val = 1.0 / sec
    emit({"metric": "TDVP steps/s", "value": val, "unit": "steps/s", "n_gpus": args.gpus, "steps": args.steps,
          "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak",
          "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "impl": "reference",
          "config": gpu_config(cfg, args.workload, args.precision), "warmup_samples_run": min(args.warmup, 1),
          "measured_wall_s_per_step": float(np.mean(walls)),
          "extrapolated": {"note": "jVMC (JAX) is not installed on the GPU host; the numpy FP64 restatement of its "
                                   "algorithm is timed on bounded parts of each phase; ms_per_step is the sum of the "
                                   "phase estimates, measured_wall_s_per_step the time actually spent per step",
                           "phases": EXTRAPOLATED},
          "cpu_baseline": {"value": val, "unit": "steps/s", "cores": os.cpu_count(), "kind": "port",
                           "sample": cpu_sample_desc(cfg)},
          "e2e": {"value": val, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
          "phase_seconds": parts})


def kernel_bench(args):
    """One kernel on a fixed synthetic case, timed with CUDA events:
    gram  tcgen05 BF16x3 Gram, rows 8192 x K 16384 (planes 537 MB > L2)
    snr   tcgen05 BF16x3 colsq GEMM, 16384 x 8192 x 8192
    eloc  fused E_loc of the L=64, M=256 Ising workload, 16384 samples
    metropolis  RBM Metropolis, 1024 chains, L=64, M=256, 64 sweeps
    data  centred O_k as transposed BF16 hi/lo planes, N=16384, L=64, M=256
    hermitian, gemv, stats  the TDVP solve's FP32 -> Hermitian fill, U^H x / U x,
          and the FP64 O_k statistics"""
    import torch
    import vmc_jax_gb300 as V
    L_ = V._lib
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    st = L_.stream()
    g = torch.Generator(device=dev).manual_seed(0)
    if args.kernel in ("gram", "snr"):
        if args.kernel == "gram":
            rows, K = 8192, 16384
            x = torch.randn(rows, K, device=dev, generator=g)
            hi = x.to(torch.bfloat16)
            lo = (x - hi.float()).to(torch.bfloat16)
            del x
            G = torch.empty((rows, rows), dtype=torch.float32, device=dev)
            fn = lambda: L_.call("vmc_gram_bf16x3", L_.ptr(hi), L_.ptr(lo), rows, K, K, L_.ptr(G), rows, 3, None, st)
            alg = float(rows) * (rows + 1) * K
            hw = 3.0 * rows * rows * K
            shape = {"rows": rows, "k": K}
        else:
            m, n, K = 16384, 8192, 8192
            a = torch.randn(m, K, device=dev, generator=g)
            b = torch.randn(n, K, device=dev, generator=g) / 90.0
            ah, bh = a.to(torch.bfloat16), b.to(torch.bfloat16)
            al, bl = (a - ah.float()).to(torch.bfloat16), (b - bh.float()).to(torch.bfloat16)
            del a, b
            cs = torch.empty(n, dtype=torch.float32, device=dev)
            ws = torch.empty(L_.query("vmc_gemm_bf16x3_colsq_workspace_bytes", m, n), dtype=torch.uint8, device=dev)
            fn = lambda: L_.call("vmc_gemm_bf16x3_colsq", L_.ptr(ah), L_.ptr(al), m, K, L_.ptr(bh), L_.ptr(bl), n, K,
                                 K, L_.ptr(cs), L_.ptr(ws), ws.numel(), 3, None, st)
            alg = 2.0 * m * n * K
            hw = 3.0 * alg
            shape = {"m": m, "n": n, "k": K}
        unit, bound = "TFLOP/s", "tensor"
    elif args.kernel in ("data", "hermitian", "gemv", "stats"):
        unit, bound = "GB/s", "hbm"
        alg = hw = None
        if args.kernel == "data":
            # centred O_k -> transposed BF16 hi/lo planes of the 64-site step:
            # N=16384, L=64, M=256 (P=16640; planes 2.18 GB)
            N, L, M = 16384, 64, 256
            P = L * M + M
            cfg_ = torch.randint(0, 2, (N, L), dtype=torch.int32, device=dev, generator=g)
            W = (0.05 * torch.randn(L, M, dtype=torch.complex64, device=dev, generator=g)).contiguous()
            b = (0.05 * torch.randn(M, dtype=torch.complex64, device=dev, generator=g)).contiguous()
            w = torch.full((N,), 1.0 / N, dtype=torch.float64, device=dev)
            mean = torch.zeros(P, dtype=torch.complex128, device=dev)
            hi = torch.empty((2 * P, N), dtype=torch.bfloat16, device=dev)
            lo = torch.empty_like(hi)
            fn = lambda: L_.call("vmc_rbm_centered_gradients", 1, L_.ptr(cfg_), N, L, M, L_.ptr(W), L_.ptr(b),
                                 L_.ptr(w), L_.ptr(mean), 2, L_.ptr(hi), L_.ptr(lo), N, st)
            nbytes = 2 * (2 * P * N * 2) + N * L * 4 + P * 16 + N * 8
            shape = {"N": N, "L": L, "M": M, "P": P}
        elif args.kernel == "hermitian":
            P = 4096
            G = torch.randn((2 * P, 2 * P), dtype=torch.float32, device=dev, generator=g)
            A = torch.empty((P, P), dtype=torch.complex128, device=dev)
            fn = lambda: L_.call("vmc_gram_to_hermitian", 1, L_.ptr(G), 2 * P, P, 0.0, L_.ptr(A), st)
            nbytes = 4 * P * P * 4 + P * P * 16   # each needed G entry once (4 per output), A once
            shape = {"P": P}
        elif args.kernel == "gemv":
            P = 8192
            U = torch.randn((P, P), dtype=torch.complex128, device=dev, generator=g)
            x = torch.randn(P, dtype=torch.complex128, device=dev, generator=g)
            y = torch.empty_like(x)
            wsg = torch.empty(L_.query("vmc_zgemv_workspace_bytes", P), dtype=torch.uint8, device=dev)
            fn = lambda: (L_.call("vmc_zgemv", 1, L_.ptr(U), P, P, L_.ptr(x), L_.ptr(y), None, 0, st),
                          L_.call("vmc_zgemv", 0, L_.ptr(U), P, P, L_.ptr(x), L_.ptr(y), L_.ptr(wsg), wsg.numel(), st))
            nbytes = 2 * (P * P * 16 + 2 * P * 16)   # adjoint and forward product
            shape = {"P": P, "products": "U^H x and U x"}
        else:
            N, L, M = 16384, 64, 256
            P = L * M + M
            cfg_ = torch.randint(0, 2, (N, L), dtype=torch.int32, device=dev, generator=g)
            W = (0.05 * torch.randn(L, M, dtype=torch.complex64, device=dev, generator=g)).contiguous()
            b = (0.05 * torch.randn(M, dtype=torch.complex64, device=dev, generator=g)).contiguous()
            w = torch.full((N,), 1.0 / N, dtype=torch.float64, device=dev)
            E = torch.randn(N, dtype=torch.complex128, device=dev, generator=g)
            em = torch.zeros(1, dtype=torch.complex128, device=dev)
            om = torch.empty(P, dtype=torch.complex128, device=dev)
            fo = torch.empty(P, dtype=torch.complex128, device=dev)
            ws = torch.empty(L_.query("vmc_rbm_grad_stats_workspace_bytes", N, L, M), dtype=torch.uint8, device=dev)
            fn = lambda: L_.call("vmc_rbm_grad_stats", 1, L_.ptr(cfg_), N, L, M, L_.ptr(W), L_.ptr(b), L_.ptr(w),
                                 L_.ptr(E), L_.ptr(em), L_.ptr(om), L_.ptr(fo), L_.ptr(ws), ws.numel(), st)
            nbytes = N * L * 4 + N * 16 + N * 8 + 2 * P * 16
            shape = {"N": N, "L": L, "M": M, "P": P}
            bound = "FP64 reduction (compute)"
    else:
        cfg = WORKLOADS[DEFAULT_WORKLOAD]
        ctx = build(cfg, "mixed")
        psi, H = ctx["psi"], ctx["H"]
        if args.kernel == "eloc":
            s = torch.randint(0, 2, (1, 16384, cfg["L"]), dtype=torch.int32, device=dev, generator=g)
            psi.rbm_tables()
            fn = lambda: H.get_O_loc_fused(s, psi, None)
            shape = {"samples": 16384, "L": cfg["L"], "M": cfg["M"], "strings": 2 * cfg["L"]}
        else:
            smp = ctx["sampler"]
            fn = lambda: smp._run_chains(psi, 0)
            smp.thermalizationSweeps = 64
            shape = {"chains": cfg["chains"], "sweeps": 64, "L": cfg["L"], "M": cfg["M"]}
        alg = hw = None
        unit, bound = "ms", "latency/compute (FP32 + MUFU)"
    for _ in range(max(args.warmup, 1)):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    out = {"kernel": args.kernel, "ms_per_launch": ms, "shape": shape, "bound": bound}
    if unit == "GB/s":
        out["algorithmic_bytes"] = nbytes
        out["achieved_gbs"] = nbytes / ms / 1e6
    if alg:
        out["algorithmic_tflops"] = alg / ms / 1e9
        out["executed_tflops"] = hw / ms / 1e9
    emit(out)


def quench_bench(args):
    """XXZ chain H = sum X X + Y Y + 1.5 Z Z (Pauli), L = 48, periodic; CpxRBM
    M = 96 with bias, started from a Neel-peaked state (hidden unit 0 couples
    to the staggered magnetisation with weight 1.0 and bias 1.0, the rest
    N(0, 0.01^2)); N_s = 8192 (1024 chains x 8); real-time TDVP
    (makeReal='imag', rhsPrefactor=1j) with AdaptiveHeun(tol=1e-4).  Reports
    the energy drift max_t |E(t) - E(0)| / |E(0)| of each form."""
    import torch
    import vmc_jax_gb300 as V
    torch.cuda.set_device(0)
    L, M, delta = 48, 96, 1.5
    rng = np.random.default_rng(0)
    b = rng.normal(0, 0.01, M) + 1j * rng.normal(0, 0.01, M)
    W = rng.normal(0, 0.01, (L, M)) + 1j * rng.normal(0, 0.01, (L, M))
    W[:, 0] = np.array([(-1) ** i for i in range(L)], dtype=float)
    b[0] = 1.0
    theta0 = np.concatenate([b.real, b.imag, W.real.ravel(), W.imag.ravel()])
    H = V.operator.BranchFreeOperator()
    for l in range(L):
        r = (l + 1) % L
        H.add(V.operator.scal_opstr(1.0, (V.operator.Sx(l), V.operator.Sx(r))))
        H.add(V.operator.scal_opstr(1.0, (V.operator.Sy(l), V.operator.Sy(r))))
        H.add(V.operator.scal_opstr(delta, (V.operator.Sz(l), V.operator.Sz(r))))
    res = {}
    for prec in ["mixed", "fp64"]:
        psi = V.vqs.NQS(V.nets.CpxRBM(numHidden=M, bias=True), precision="fp64" if prec == "fp64" else "fp32")
        psi(np.zeros((1, 1, L), np.int32))
        psi.set_parameters(theta0)
        smp = V.sampler.MCSampler(psi, (L,), 7, updateProposer=V.sampler.propose_spin_flip, numChains=1024,
                                  numSamples=8192, thermalizationSweeps=32, sweepSteps=L)
        td = V.util.TDVP(smp, makeReal="imag", rhsPrefactor=1.j, pinvCutoff=1e-8, snrTol=2, precision=prec)
        st = V.util.stepper.AdaptiveHeun(timeStep=1e-3, tol=1e-4)
        theta = psi.get_parameters()
        t, times, E = 0.0, [], []
        t0 = time.perf_counter()

        # integration error in the metric of S (the norm_fun of the
        # reference's time-evolution examples: Re v^dagger S v)
        def s_norm(v):
            return float(torch.real(torch.vdot(v.to(torch.complex128), td.S_dot(v))))

        class _WallClock(Exception):
            pass

        def rhs(y, tt, **kw):  # the step-size control may retry: bound the wall clock per RHS
            if time.perf_counter() - t0 > args.quench_wall:
                raise _WallClock()
            return td(y, tt, **kw)

        while t < args.quench and len(E) < args.quench_steps:
            try:
                theta, dt = st.step(t, rhs, theta, hamiltonian=H, psi=psi, numSamples=8192, normFunction=s_norm)
            except _WallClock:
                break
            psi.set_parameters(theta)
            times.append(t)
            E.append(float(torch.real(td.ElocMean0)))
            t += dt
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        E = np.array(E)
        if prec == "mixed":
            # estimator error of the FP32 kernels: E on the same samples at the
            # final parameters with FP32 and with FP64 kernels
            smp_chk = V.sampler.MCSampler(psi, (L,), 11, updateProposer=V.sampler.propose_spin_flip,
                                          numChains=1024, numSamples=8192, thermalizationSweeps=8, sweepSteps=L)
            psi.precision = "fp64"
            psi._touch()
            cfgs, _, pw = smp_chk.sample()
            e_pair = {}
            for kp in ("fp32", "fp64"):
                psi.precision = kp
                psi._touch()
                el = H.get_O_loc(cfgs, psi, None)
                e_pair[kp] = float(torch.real(torch.sum(el * pw)))
            psi.precision = "fp32"
            psi._touch()
            same_sample_err = abs(e_pair["fp32"] - e_pair["fp64"]) / abs(e_pair["fp64"])
        res[prec] = {"steps": len(E), "t_end": t, "wall_s": wall, "E0": float(E[0]), "stopped_early": t < args.quench,
                     "drift": float(np.max(np.abs(E - E[0])) / abs(E[0])), "E": E.tolist(), "t": times}
    emit({"metric": "XXZ quench energy drift, mixed vs FP64 solve", "workload": "xxz48_rbm96_quench",
          "config": {"L": L, "M": M, "delta": delta, "num_samples": 8192,
                     "integrator": "AdaptiveHeun tol 1e-4, S-metric error norm", "t_end": args.quench,
                     "max_steps": args.quench_steps, "max_wall_s": args.quench_wall},
          "data": "synthetic (seeded)",
          "energy_rel_err_fp32_vs_fp64_same_samples": same_sample_err, **res})


def serve_bench(args):
    """Poisson arrivals of independent jobs served by the continuous-batching
    loop: the serving workload's distributions (L uniform over --serve-L,
    h ~ U[0.5, 1.5], M = L times a draw from --serve-m-over-l, N_s = 2^e with
    e uniform in --serve-ns-exp, 1 in 4 a real-time quench), --job-steps
    TDVP steps each; p50/p99 per-step and per-job latency and steps/s."""
    import torch
    from vmc_jax_gb300.serving import JobSpec, Server
    torch.cuda.set_device(0)
    Ls = [int(x) for x in args.serve_L.split(",")]
    mol = [int(x) for x in args.serve_m_over_l.split(",")]
    e0, e1 = (int(x) for x in args.serve_ns_exp.split(","))
    rng = np.random.default_rng(123)
    t = 0.0
    specs = []
    for j in range(args.jobs):
        t += rng.exponential(1.0 / args.rate)
        L = int(rng.choice(Ls))
        specs.append(JobSpec(L=L, h=float(rng.uniform(0.5, 1.5)), M=int(rng.choice(mol)) * L,
                             num_samples=int(2 ** rng.integers(e0, e1 + 1)), steps=args.job_steps, seed=j,
                             kind="quench" if j % 4 == 3 else "ground_state",
                             dt=0.005 if j % 4 == 3 else 0.01, arrival=t, precision=args.precision))
    # warm-up: one small job pages in the libraries
    w = Server(max_slots=1)
    w.submit(JobSpec(L=8, h=1.0, M=8, num_samples=256, steps=2))
    w.run()
    srv = Server(max_slots=args.slots)
    for sp in specs:
        srv.submit(sp)
    rep = srv.run()
    emit({"metric": "served TDVP steps/s and p50/p99 latency", "value": rep["steps_per_s"], "unit": "steps/s",
          "n_gpus": 1, "higher_is_better": True, "data": "synthetic (seeded job stream)",
          "config": {"workload": "poisson_ising_jobs", "jobs": args.jobs, "rate_per_s": args.rate,
                     "steps_per_job": args.job_steps, "L": Ls, "M_over_L": mol,
                     "N_s": [2 ** e0, 2 ** e1], "precision": args.precision, "slots": args.slots},
          **rep})


def main():
    args = parse()
    if args.quench is not None:
        quench_bench(args)
        return
    if args.serve:
        serve_bench(args)
        return
    if args.kernel:
        kernel_bench(args)
        return
    if args.impl == "reference":
        run_reference(args)
        return
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    cfg = WORKLOADS[args.workload]
    ctx = build(cfg, args.precision)
    V = ctx["V"]
    from vmc_jax_gb300.util.timing import TIMER
    theta = ctx["psi"].get_parameters()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    for _ in range(max(args.warmup, 3) if args.warmup >= 3 else args.warmup):
        theta = one_step(ctx, theta)
    torch.cuda.synchronize()

    # timed region: K steps, device-resident inputs
    clocks = ClockSampler(local)
    TIMER.reset()
    TIMER.enabled = True
    TIMER.nvtx = True
    V._lib.launch_count = 0
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record()
    for _ in range(args.steps):
        theta = one_step(ctx, theta)
    t_end.record()
    torch.cuda.synchronize()
    barrier()
    clock = clocks.stop()
    TIMER.enabled = False
    TIMER.nvtx = False
    TIMER.close()
    launches = V._lib.launch_count
    ms = reduce_max_ms(t_start.elapsed_time(t_end), device=torch.device("cuda", local))
    ms_per_step = ms / args.steps
    phases = {k: v / args.steps for k, v in TIMER.durations().items()}
    gram_ms = TIMER.spans("gram_kernel")
    snr_ms = TIMER.spans("snr_kernel")
    energy = float(torch.real(ctx["tdvp"].ElocMean0))

    # e2e: the public API with host buffers (pinned), copies inside the timed region
    e2e = None
    if not args.no_e2e:
        host_theta = theta.cpu().pin_memory()
        host_out = torch.empty_like(host_theta).pin_memory()
        host_e = torch.empty(1, dtype=torch.float64).pin_memory()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dev_theta = host_theta.to("cuda", non_blocking=True)
        new = one_step(ctx, dev_theta)
        host_out.copy_(new, non_blocking=True)
        host_e.copy_(torch.real(ctx["tdvp"].ElocMean0).reshape(1), non_blocking=True)
        torch.cuda.synchronize()
        e2e_s = time.perf_counter() - t0
        e2e = {"value": 1.0 / e2e_s, "unit": "steps/s", "h2d_bytes_per_step": host_theta.numel() * 8,
               "d2h_bytes_per_step": host_out.numel() * 8 + 8}

    accuracy, plain = None, None
    if not args.no_accuracy and args.precision == "mixed" and cfg.get("net") != "cnn":
        accuracy = accuracy_block(ctx)
        if args.plain_steps > 0:
            plain = plain_fp32_steps_per_s(cfg, args.plain_steps)

    if rank != 0:
        return
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except Exception:
        pass
    Ns, P = ctx["ns"], ctx["P"]
    roofline = None
    if gram_ms:
        t = float(np.mean(gram_ms)) * 1e-3
        flops = 4.0 * Ns * P * (P + 1)  # Hermitian S build, 8 flop per complex MAC
        peak = peaks.get("bf16_tflops_sustained", 1700.0)
        ach = flops / t / 1e12
        # DRAM traffic of one launch, scaled from the ncu capture of the same
        # kernel at rows 8192, K 16384 (2.065 GB read + 0.123 GB written over
        # 1056 tiles of 128 x 256, grouped tile order): per tile the operand
        # panels grow with K, the FP32 tile write does not
        R = 2 * P
        tilesM, tilesN = (R + 127) // 128, (R + 255) // 256
        tiles = sum(min(tilesM, 2 * tn + 2) for tn in range(tilesN))
        traffic = tiles * (2.065120e9 / 1056 * (Ns / 16384.0) + 0.122942e9 / 1056)
        roofline = {"kernel": "tc_gemm_kernel (S build, BF16x3 split, tcgen05)", "bound": "tensor",
                    "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": ach / peak,
                    "peak_source": "MEASURED_PEAKS.json bf16_tflops_sustained (of measured)",
                    "traffic": traffic,
                    "traffic_source": "ncu dram__bytes_read+write of the rows-8192 K-16384 capture, scaled by tiles "
                                      "and K",
                    "algorithmic_flops_per_launch": flops,
                    "hardware_flops_per_launch": 3 * 2.0 * Ns * (2 * P) ** 2 / 2,
                    "launch_ms": t * 1e3}
    info = getattr(ctx["tdvp"], "refineInfo", None)
    refine_ms = TIMER.spans("eigh_refine")
    if info and info.get("refined") and refine_ms:
        # executed BF16 flop of the Ozaki-split products of one refinement
        # (csrc/eigh.cu): a complex m x n x K product with p slice pairs is
        # p * 8 m n K real flop; Hermitian products compute ~half the tiles
        n_, k_, q_ = info["n"], info["refined"], info["power_steps"]
        b_ = n_ - k_
        full, early, rest = 36, 21, 15
        per = 8.0 * n_ * k_ * n_
        flops = per * (early * max(q_ - 1, 0) + full * (1 if q_ >= 1 else 0) + full)   # power steps + A X
        flops += 2 * full * 0.5 * 8.0 * k_ * k_ * n_                                   # G, H (Hermitian)
        flops += full * 8.0 * n_ * k_ * k_                                              # X C
        flops += rest * 2 * 8.0 * k_ * b_ * n_                                          # orthogonalisation
        fp64eq = flops / full
        t = float(np.mean(refine_ms)) * 1e-3
        peak = peaks.get("bf16_tflops_sustained", 1700.0)
        # DRAM bytes per executed flop of the ncu capture of one 4096^3
        # complex product (8 slices, 36 pairs: 1.979e13 flop, 44.02 GB read +
        # 0.265 GB written), applied to the refinement's executed flop
        traffic = flops * (44.02e9 + 0.265e9) / (36 * 8.0 * 4096.0 ** 3)
        oz = {"kernel": "oz_gemm_kernel (Ozaki-split FP64-accurate complex products, tcgen05) in "
                        "vmc_eigh_refine_top", "bound": "tensor", "achieved": flops / t / 1e12, "peak": peak,
              "unit": "TFLOP/s", "frac": flops / t / 1e12 / peak, "traffic": traffic,
              "traffic_source": "ncu dram__bytes_read+write per executed flop of the 4096^3 capture, scaled to "
                                "the refinement's executed flop (all its Ozaki launches)",
              "peak_source": "MEASURED_PEAKS.json bf16_tflops_sustained (of measured)",
              "algorithmic_flops_per_refinement": flops, "fp64_equivalent_tflops": fp64eq / t / 1e12,
              "refinement_ms": t * 1e3,
              "note": "achieved counts the BF16 slice products the split scheme requires, timed over the whole "
                      "refinement call (slicing, assembly and the k x k FP64 zhegvd included)"}
        roofline, secondary = oz, roofline
    else:
        secondary = None
    out = {"metric": "TDVP steps/s", "value": aggregate_steps_per_s(args.steps, world, ms), "unit": "steps/s",
           "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32+bf16x3 (FP64 statistics and solve; FP64-accurate eigenpairs that carry the solve)",
           "data": "synthetic (seeded lattice and parameters)",
           "config": {**gpu_config(cfg, args.workload, args.precision),
                      "parallelism": "replicas" if world > 1 else "single GPU"},
           "energy": energy, "phase_ms": phases, "gram_kernel_ms": gram_ms, "snr_kernel_ms": snr_ms,
           "roofline": roofline, "clocks": clock, "gpu_launches": launches, "e2e": e2e,
           "notes": ["makeReal='real' SNR: each eigenvalue of S appears twice in the reference's 2P real "
                     "representation; both members of a pair get the rotation-invariant pair value "
                     "N |u^H f|^2 / sum_n w_n |u^H (h_n - f)|^2, where the reference's per-eigenvector value "
                     "depends on LAPACK's basis inside the degenerate pair (tdvp.py:173-181)"]}
    if secondary is not None:
        out["roofline_s_build"] = secondary
    if getattr(ctx["tdvp"], "refineInfo", None) is not None:
        out["eigensolver"] = ctx["tdvp"].refineInfo
    if accuracy is not None:
        out["accuracy"] = {"vs": "FP64 form (FP64 kernels, S, eigendecomposition and solve) on the same samples",
                           "relative_errors": accuracy}
    if plain is not None:
        out["plain_fp32_steps_per_s"] = plain
        out["mixed_over_fp32"] = out["value"] / plain
    if not args.no_cpu_baseline and world == 1:
        sec, parts = cpu_step_seconds(cfg, "")
        out["cpu_baseline"] = {"value": 1.0 / sec, "unit": "steps/s", "cores": os.cpu_count(), "kind": "port",
                               "sample": cpu_sample_desc(cfg), "phase_seconds": parts,
                               "extrapolated": EXTRAPOLATED}
    emit(out)


if __name__ == "__main__":
    main()
