"""Continuous-batching server for independent TDVP jobs on one GPU.

A job is a transverse-field Ising chain (L sites, couplings J and h) with a
CpxRBM of M hidden units, N_s Monte Carlo samples per step and a number of
TDVP steps: either an imaginary-time ground-state search (makeReal='real',
x = 1) or a real-time quench (makeReal='imag', x = i), Euler-integrated.

* Jobs arrive at any time (``submit``).  A job is admitted when a slot is
  free and its estimated HBM footprint fits the budget; until then it waits.
* An admitted job's parameters, Markov chains, random-stream counter and
  integrator state stay on the device in persistent per-slot buffers.
* Each tick launches the sampling + E_loc phase of every job that is ready
  for its next step from CUDA graphs: a set of ready jobs that recurs gets
  ONE shared graph (each job's kernels on its own branch), a set seen for
  the first time replays the jobs' own graphs (captured once per job) back
  to back, so that a mix of short and long steps, whose ready sets rarely
  repeat, captures nothing per tick.  Captures run in thread-local mode
  without a device-wide synchronisation: the solves in flight keep running.
  Then each job's solve runs on its own stream from its own host thread, so
  the solves of different jobs overlap on the GPU, and the next tick
  samples whichever jobs are ready again.
* Per-step latency (graph launch to update applied) and per-job latency
  (arrival to last step) are recorded for p50/p99 reporting.
* Failures stay with their job: an invalid spec is refused at ``submit``, a
  job whose footprint exceeds the whole budget is rejected at admission, a
  job whose step raises (including its ``on_step`` callback) is marked
  failed, a shared sampling launch that fails is retried job by job and only
  the jobs whose own launch fails are marked failed, and ``cancel``
  withdraws a queued job or stops an active one after its current step; the
  other jobs continue.  ``status`` reports each job's
  state.

A job computes exactly what it computes alone: its kernels, inputs and
random stream do not depend on the other jobs, and every reduction adds in
a fixed order.
"""

import dataclasses
import math
import threading
import time

import numpy as np
import torch

from . import _lib
from . import global_defs
from . import mpi_wrapper as mpi
from .nets.rbm import CpxRBM
from .operator.branch_free import BranchFreeOperator, Sx, Sz, scal_opstr
from .sampler import MCSampler, propose_spin_flip
from .util.tdvp import TDVP
from .vqs import NQS


class ReplayError(RuntimeError):
    """A shared graph replay failed after it may have enqueued work."""


@dataclasses.dataclass
class JobSpec:
    L: int
    h: float
    M: int
    num_samples: int
    steps: int = 50
    kind: str = "ground_state"   # or "quench"
    J: float = 1.0
    dt: float = 0.01
    seed: int = 0
    chains: int = 0              # 0: min(1024, num_samples // 4)
    precision: str = "mixed"
    arrival: float = 0.0         # seconds after the server starts
    on_step: object = None       # callable(job_id, step, energy) after every step

    def validate(self):
        if self.L < 2 or self.M < 1 or self.num_samples < 1 or self.steps < 0:
            raise ValueError("job spec needs L >= 2, M >= 1, num_samples >= 1, steps >= 0")
        if self.kind not in ("ground_state", "quench"):
            raise ValueError("job kind must be 'ground_state' or 'quench', not %r" % (self.kind,))
        if self.precision not in ("fp64", "fp32", "mixed"):
            raise ValueError("precision must be 'fp64', 'fp32' or 'mixed'")

    @property
    def num_params(self):
        return self.L * self.M + self.M

    def num_chains(self):
        return self.chains or max(1, min(1024, self.num_samples // 4))


def footprint_bytes(spec):
    """Conservative HBM estimate of one job's step (all buffers of the mixed
    pipeline alive at once)."""
    P, N, L = spec.num_params, spec.num_samples, spec.L
    P2 = 2 * P
    b = 0
    b += 2 * P2 * N * 2          # centred O_k planes (bf16 hi/lo)
    b += P2 * P2 * 4             # FP32 Gram
    b += 4 * P * P * 16          # A, eigenvectors, eigh workspace (estimate)
    b += 2 * N * P2 * 2          # SNR data planes
    b += 2 * P2 * P2 * 2         # eigenvector planes
    if P >= 2048:                # two-stage eigensolver: complex64 copy, cuSOLVER and Ozaki-slice workspaces
        b += 48 * P * P
    b += N * L * 4 * 2 + N * 64  # configs, per-sample scalars
    b += 64 << 20                # statistics workspace, tables, slack
    return b


def percentile(x, q):
    if not x:
        return None
    return float(np.percentile(np.asarray(x), q))


class _Slot:
    """Device-resident state of one admitted job."""

    def __init__(self, job_id, spec, arrival_wall):
        self.id = job_id
        self.spec = spec
        self.arrival_wall = arrival_wall
        self.steps_done = 0
        self.step_latencies = []
        self.energies = []
        self.stream = torch.cuda.Stream()
        self.graph = None            # this job's own sampling + E_loc graph
        L, M = spec.L, spec.M
        dev = global_defs.device()
        rng = np.random.default_rng(spec.seed)
        theta = np.concatenate([rng.normal(0, 0.01, M), rng.normal(0, 0.01, M),
                                rng.normal(0, 0.01, L * M), rng.normal(0, 0.01, L * M)])
        if spec.kind == "quench":
            theta = theta * 20.0
        self.psi = NQS(CpxRBM(numHidden=M, bias=True), precision="fp64" if spec.precision == "fp64" else "fp32")
        self.psi(np.zeros((1, 1, L), np.int32))
        self.psi.set_parameters(theta)
        self.H = BranchFreeOperator()
        for l in range(L):
            self.H.add(scal_opstr(-spec.J, (Sz(l), Sz((l + 1) % L))))
            self.H.add(scal_opstr(-spec.h, (Sx(l),)))
        C = spec.num_chains()
        self.sampler = MCSampler(self.psi, (L,), spec.seed, updateProposer=propose_spin_flip, numChains=C,
                                 numSamples=spec.num_samples, thermalizationSweeps=8, sweepSteps=L)
        if spec.kind == "quench":
            self.tdvp = TDVP(self.sampler, makeReal="imag", rhsPrefactor=1.j, pinvCutoff=1e-8,
                             precision=spec.precision)
        else:
            self.tdvp = TDVP(self.sampler, makeReal="real", rhsPrefactor=1., pinvCutoff=1e-8,
                             precision=spec.precision)
        # persistent buffers read by the captured sampling / E_loc graph
        self.kprec = "fp64" if spec.precision == "fp64" else "fp32"
        pr = self.psi.params_for(self.kprec)
        self.W = pr["kernel"].clone().contiguous()
        self.b = pr["bias"].clone().contiguous()
        self.tables = self.psi.net.tables({"kernel": self.W}, self.kprec).clone()
        self.perChain = int(math.ceil(spec.num_samples / C))
        self.N = self.perChain * C
        self.configs = torch.empty((self.N, L), dtype=torch.int32, device=dev)
        self.logpsi = torch.empty(self.N, dtype=torch.complex128, device=dev)
        self.p = torch.empty(self.N, dtype=torch.float64, device=dev)
        self.eloc = torch.empty(self.N, dtype=torch.complex128, device=dev)
        self.ws = torch.empty(_lib.query("vmc_reduce_workspace_bytes", 1), dtype=torch.uint8, device=dev)
        self.call = torch.zeros(1, dtype=torch.int32, device=dev)
        self.counters = torch.zeros(2, dtype=torch.int64, device=dev)
        self.op = self.H._device_operator()
        self.sampler.globNumSamples = self.N
        self.theta = self.psi.get_parameters()

    # ---- phase 1: captured into the job's own and the shared graphs
    def launch_sampling(self):
        spec = self.spec
        prec = CpxRBM._prec(self.kprec)
        L, M, C = spec.L, spec.M, self.sampler.numChains
        st = _lib.stream()
        _lib.call("vmc_rbm_prepare", prec, L, M, _lib.ptr(self.W), _lib.ptr(self.tables), st)
        _lib.call("vmc_rbm_metropolis_devcall", prec, _lib.ptr(self.sampler.states), C, L, M, _lib.ptr(self.W),
                  _lib.ptr(self.b), _lib.ptr(self.tables), float(self.sampler.mu), self.sampler.seed,
                  _lib.ptr(self.call), int(self.sampler.thermalizationSweeps * self.sampler.sweepSteps),
                  int(self.sampler.sweepSteps), self.perChain, _lib.ptr(self.configs), _lib.ptr(self.counters), st)
        _lib.call("vmc_rbm_logpsi", prec, _lib.ptr(self.configs), self.N, L, M, _lib.ptr(self.W), _lib.ptr(self.b),
                  _lib.ptr(self.logpsi), st)
        _lib.call("vmc_mc_probabilities", _lib.ptr(self.logpsi), self.N,
                  float(1.0 / self.sampler.logProbFactor - self.sampler.mu), _lib.ptr(self.p), _lib.ptr(self.ws),
                  self.ws.numel(), st)
        _lib.call("vmc_rbm_oloc_fused", prec, _lib.ptr(self.configs), self.N, L, M, _lib.ptr(self.W),
                  _lib.ptr(self.b), _lib.ptr(self.tables), self.op, None, _lib.ptr(self.eloc), st)

    # ---- phase 2: the job's own stream and host thread
    def solve(self, ready_event, t_launch):
        with torch.cuda.stream(self.stream):
            self.stream.wait_event(ready_event)
            configs = self.configs.reshape(1, self.N, self.spec.L)
            update, _, _ = self.tdvp._rbm_rhs(self.psi, configs, self.eloc.reshape(1, -1), self.p.reshape(1, -1))
            self.energies.append(self.tdvp.ElocMean.real.clone())
            self.theta = self.theta + self.spec.dt * update
            self.psi.set_parameters(self.theta)
            pr = self.psi.params_for(self.kprec)
            self.W.copy_(pr["kernel"])
            self.b.copy_(pr["bias"])
            self.stream.synchronize()
        self.steps_done += 1
        self.step_latencies.append(time.perf_counter() - t_launch)
        if self.spec.on_step is not None:
            self.spec.on_step(self.id, self.steps_done, float(self.energies[-1]))

    @property
    def finished(self):
        return self.steps_done >= self.spec.steps


class Server:
    """Persistent request loop over one GPU (see the module docstring).

    ``hbm_budget``: bytes the admitted jobs' footprints may sum to (default:
    80% of the free device memory); ``max_slots``: jobs resident at once;
    ``batch_window``: seconds a tick waits for more jobs to become ready."""

    def __init__(self, hbm_budget=None, max_slots=8, batch_window=0.002):
        self.sample_stream = self._open_device()
        if hbm_budget is None:
            free, _ = torch.cuda.mem_get_info()
            hbm_budget = int(0.8 * free)
        self.hbm_budget = hbm_budget
        self.max_slots = max_slots
        self.batch_window = batch_window
        self.queue = []
        self.active = {}
        self.done = {}
        self.graphs = {}             # shared graphs of recurring ready sets
        self.seen = {}               # ready sets launched so far (several jobs), count
        self.graph_replays = 0
        self.shared_replays = 0
        self.lock = threading.Condition()
        self.ready = set()
        self.next_id = 0
        self.t0 = None
        self.max_resident = 0
        self.graph_launches = 0
        self.states = {}        # job id -> queued / active / done / failed / rejected / cancelled
        self.errors = {}
        self.cancelled = set()

    def submit(self, spec):
        """Queue a job; raises ValueError for an invalid spec."""
        spec.validate()
        with self.lock:
            jid = self.next_id
            self.next_id += 1
            self.queue.append((jid, spec))
            self.states[jid] = "queued"
            self.lock.notify_all()
            return jid

    def cancel(self, job_id):
        """Withdraw a queued job, or stop an active one after its current step."""
        with self.lock:
            for item in list(self.queue):
                if item[0] == job_id:
                    self.queue.remove(item)
                    self.states[job_id] = "cancelled"
                    self.lock.notify_all()
                    return
            if job_id in self.active:
                self.cancelled.add(job_id)

    def status(self, job_id):
        return self.states.get(job_id)

    # ---- the device side of the loop (the scheduling above and below is
    # host logic only)
    def _open_device(self):
        """Check for the CUDA library and return the stream the shared graphs run on."""
        _lib.require_cuda()
        return torch.cuda.Stream()

    def _new_slot(self, job_id, spec, arrival_wall):
        return _Slot(job_id, spec, arrival_wall)

    def _launch(self, ids):
        """Replay the sampling + E_loc graphs of the ready jobs ``ids``
        (``_launch_plan``); returns the event the jobs' solves wait on and the
        launch time.  A failure while a graph is captured has enqueued nothing
        and raises as it is; a failure of a replay may have enqueued part of
        the jobs' work and raises ``ReplayError``."""
        shared, key = self._launch_plan(ids)
        if shared:
            if key not in self.graphs:
                self.graphs[key] = self._capture(key)
            graphs = [self.graphs[key]]
        else:
            graphs = []
            for jid in key:
                slot = self.active[jid]
                if slot.graph is None:
                    slot.graph = self._capture((jid,))
                graphs.append(slot.graph)
        t_launch = time.perf_counter()
        try:
            cap = self.sample_stream
            if shared:
                with torch.cuda.stream(cap):
                    graphs[0].replay()
            else:  # each job's graph from its own (idle) stream, so they run side by side
                for jid, g in zip(key, graphs):
                    st = self.active[jid].stream
                    st.wait_stream(cap)
                    with torch.cuda.stream(st):
                        g.replay()
                for jid in key:
                    cap.wait_stream(self.active[jid].stream)
            ev = torch.cuda.Event()
            ev.record(cap)
        except Exception as e:
            raise ReplayError("%s: %s" % (type(e).__name__, e)) from e
        self.graph_replays += len(graphs)
        self.shared_replays += int(shared)
        return ev, t_launch

    def _launch_plan(self, ids):
        """(shared, key): one shared graph for a set of several jobs seen
        before (its graph is kept while all its jobs stay), else the jobs'
        own graphs.  Host logic only."""
        key = tuple(sorted(ids))
        if len(key) < 2:
            return False, key
        if key in self.graphs:
            return True, key
        self.seen[key] = self.seen.get(key, 0) + 1
        return self.seen[key] >= 2, key

    def _capture(self, ids):
        """One graph of the sampling + E_loc kernels of the jobs ``ids``,
        each job on its own stream as a branch of the shared sample stream.
        Every job in ``ids`` is between steps, so its stream is idle; the
        capture is thread-local and takes no device-wide synchronisation."""
        g = torch.cuda.CUDAGraph()
        cap = self.sample_stream
        with torch.cuda.stream(cap):
            g.capture_begin(capture_error_mode="thread_local")
            try:
                branches = []
                for jid in ids:
                    br = self.active[jid].stream
                    br.wait_stream(cap)
                    with torch.cuda.stream(br):
                        self.active[jid].counters.zero_()
                        self.active[jid].launch_sampling()
                    branches.append(br)
                for br in branches:
                    cap.wait_stream(br)
            finally:
                g.capture_end()
        return g

    def _used(self):
        return sum(footprint_bytes(s.spec) for s in self.active.values())

    def _admit(self, now):
        admitted = []
        for item in list(self.queue):
            jid, spec = item
            if spec.arrival > now:
                continue
            if len(self.active) >= self.max_slots:
                break
            if footprint_bytes(spec) > self.hbm_budget:
                self.queue.remove(item)
                self.states[jid] = "rejected"
                self.errors[jid] = "needs %.1f GB, more than the HBM budget of %.1f GB" % (
                    footprint_bytes(spec) / 1e9, self.hbm_budget / 1e9)
                continue
            if self._used() + footprint_bytes(spec) > self.hbm_budget:
                continue
            self.queue.remove(item)
            try:
                slot = self._new_slot(jid, spec, self.t0 + spec.arrival)
            except Exception as e:  # e.g. device memory exhausted while allocating the slot
                self.states[jid] = "failed"
                self.errors[jid] = "admission: %s" % (e,)
                continue
            self.active[jid] = slot
            self.states[jid] = "active"
            self.ready.add(jid)
            admitted.append(jid)
        self.max_resident = max(self.max_resident, len(self.active))
        return admitted

    def run(self):
        """Serve until every submitted job has finished; returns the report."""
        self.t0 = time.perf_counter()
        workers = {}
        while True:
            with self.lock:
                now = time.perf_counter() - self.t0
                self._admit(now)
                if not self.queue and not self.active:
                    break
                if not self.ready:
                    # wait for a solve to finish or the next arrival
                    nxt = min([s.arrival for _, s in self.queue], default=None)
                    timeout = 0.05 if nxt is None else max(1e-4, min(0.05, nxt - now))
                    self.lock.wait(timeout)
                    continue
            time.sleep(self.batch_window)  # let more jobs become ready
            with self.lock:
                ids = sorted(self.ready)
                self.ready.clear()
                for jid in [i for i in ids if i in self.cancelled]:  # cancelled between steps
                    del self.active[jid]
                    self.states[jid] = "cancelled"
                ids = [i for i in ids if i not in self.cancelled]
                self.graphs = {k: v for k, v in self.graphs.items() if all(i in self.active for i in k)}
                self.seen = {k: v for k, v in self.seen.items() if all(i in self.active for i in k)}
                if not ids:
                    continue
            try:
                ev, t_launch = self._launch(ids)
                self.graph_launches += 1
                batch = [(jid, ev, t_launch) for jid in ids]
            except ReplayError as e:
                # part of the jobs' sampling may already have run: re-running it
                # would advance their chains twice, so every job of the launch fails
                self._fail(ids, "replay: %s" % (e,))
                batch = []
            except Exception:  # capture failed, nothing was enqueued: find the job(s) at fault
                batch = self._launch_each(ids)
            for jid, ev, t_launch in batch:
                slot = self.active[jid]
                th = threading.Thread(target=self._work, args=(slot, ev, t_launch), daemon=True)
                workers[jid] = th
                th.start()
        for th in workers.values():
            th.join()
        return self.report()

    def _launch_each(self, ids):
        """After a shared launch failed: launch each ready job alone.  A job
        whose own launch fails is marked failed and releases its slot; the
        others run this step from their own graphs."""
        batch = []
        for jid in ids:
            try:
                ev, t_launch = self._launch([jid])
            except ReplayError as e:
                self._fail([jid], "replay: %s" % (e,))
                continue
            except Exception as e:
                self._fail([jid], "launch: %s: %s" % (type(e).__name__, e))
                continue
            self.graph_launches += 1
            batch.append((jid, ev, t_launch))
        return batch

    def _fail(self, ids, why):
        """Mark the jobs ``ids`` failed and release their slots."""
        with self.lock:
            for jid in ids:
                slot = self.active.pop(jid, None)
                if slot is not None:
                    slot.job_latency = time.perf_counter() - slot.arrival_wall
                self.states[jid] = "failed"
                self.errors[jid] = why
            self.lock.notify_all()

    def _work(self, slot, ev, t_launch):
        err = None
        try:
            slot.solve(ev, t_launch)
        except Exception as e:  # the job fails alone; its slot is released
            err = "%s: %s" % (type(e).__name__, e)
        finally:
            _lib.Workspace.release()  # this step's thread ends: its scratch goes with it
        with self.lock:
            if err is not None or slot.id in self.cancelled or slot.finished:
                slot.job_latency = time.perf_counter() - slot.arrival_wall
                del self.active[slot.id]
                if err is not None:
                    self.states[slot.id] = "failed"
                    self.errors[slot.id] = err
                elif slot.finished:
                    self.done[slot.id] = slot
                    self.states[slot.id] = "done"
                else:
                    self.states[slot.id] = "cancelled"
            else:
                self.ready.add(slot.id)
            self.lock.notify_all()

    def report(self):
        steps = [x for s in self.done.values() for x in s.step_latencies]
        jobs = [s.job_latency for s in self.done.values()]
        wall = time.perf_counter() - self.t0
        return {"jobs": len(self.done), "steps": len(steps), "wall_s": wall,
                "steps_per_s": len(steps) / wall if wall > 0 else None,
                "step_latency_s": {"p50": percentile(steps, 50), "p99": percentile(steps, 99)},
                "job_latency_s": {"p50": percentile(jobs, 50), "p99": percentile(jobs, 99)},
                "max_resident_jobs": self.max_resident, "graph_launches": self.graph_launches,
                "graph_replays": self.graph_replays, "shared_graph_replays": self.shared_replays,
                "not_completed": {jid: st for jid, st in self.states.items() if st != "done"},
                "errors": {jid: str(msg) for jid, msg in self.errors.items()}}

    def result(self, job_id):
        """Final flat parameters and per-step energies of a finished job."""
        if job_id not in self.done:
            raise KeyError("job %d is %s%s" % (job_id, self.states.get(job_id, "unknown"),
                                               (": " + self.errors[job_id]) if job_id in self.errors else ""))
        s = self.done[job_id]
        return s.theta, torch.stack(s.energies)
