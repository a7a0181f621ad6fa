"""Many CASCI solves in flight on one GPU: batched instances and a continuous-batching server.

Every solve is a step generator (``CASCISolver.run_steps``): it enqueues device work on its CUDA
stream and yields the small device tensors it must read next (nothing, when its iterations run
from a captured graph that leaves its state in pinned host memory). ``StepScheduler`` gives each
job in flight a stream of its own, records an event after each step, and resumes a job as soon as
its event has completed, so a job never waits for another job's work: a slow solve (a large
active space) does not hold back the small ones. New jobs can be admitted whenever the
scheduler polls (``admit`` callback): the serving loop admits arriving requests while their
estimated HBM footprint fits the budget.

Streams of different jobs share the device's hardware queues (CUDA_DEVICE_MAX_CONNECTIONS, 8 by
default); an application with many jobs in flight should raise it (up to 32) before CUDA starts.
"""

from __future__ import annotations

import time
from dataclasses import dataclass
from math import comb

import numpy as np

from ._lib import check, lib
from .ci import CASCISolver
from .davidson import GraphPhase
from .params import CIParams, DavidsonLiuParams
from .synthetic import make_integrals


def _torch():
    import torch

    return torch


@dataclass
class Job:
    key: object
    gen: object
    stream: object
    event: object = None  # recorded after each step; completed = the step's device work is done
    request: list = None
    result: object = None
    t_admit: float = 0.0
    t_done: float = 0.0
    footprint: int = 0
    steps: int = 0


class StepScheduler:
    """Event-driven driver of step generators, one CUDA stream per job in flight.

    With one_launch=True, jobs whose graph-captured iterations wait for a collective launch
    (GraphPhase, CASCISolver(one_launch=True)) are parked; when every job in flight is parked, the
    iterations of all of them run in ONE graph launch (f2g_dgraph_batch_*: one branch per solve,
    each a device-side while loop that stops at its own convergence), after which they resume."""

    def __init__(self, nstreams: int = 16, poll_sleep: float = 2e-5, one_launch: bool = False):
        torch = _torch()
        self.one_launch = one_launch
        self.batch_launches = 0   # collective launches
        self.batch_solves = 0     # solve phases run inside them
        self.batch_nodes = 0      # graph nodes of the largest collective launch
        self._batches = {}        # (serials of the member graphs) -> batch handle
        self._batch_stream = None
        # free streams by priority class: 0 normal, 1 high (lower CUDA priority value); more are
        # made on demand
        self._free = {0: [torch.cuda.Stream() for _ in range(nstreams)], 1: []}
        self.max_streams = nstreams
        self.rounds = 0  # resumptions of jobs after a completed step
        self.polls = 0
        self.poll_sleep = poll_sleep
        self.host_s = {"start": 0.0, "resume": 0.0, "admit": 0.0}  # host time by activity

    def _stream(self, high=False):
        torch = _torch()
        free = self._free[1 if high else 0]
        if free:
            return free.pop()
        self.max_streams += 1
        return torch.cuda.Stream(priority=-1) if high else torch.cuda.Stream()

    def _resume(self, job, values):
        torch = _torch()
        with torch.cuda.stream(job.stream):
            try:
                job.request = job.gen.send(values) if values is not None else next(job.gen)
                job.steps += 1
                if job.event is None:
                    job.event = torch.cuda.Event()
                job.event.record(job.stream)
                return False
            except StopIteration as e:
                # no host wait: the work the job enqueued last (its final vectors) is ordered by
                # the event; a consumer on another stream waits for it (CASCISolver does)
                job.result = e.value
                if job.event is None:
                    job.event = torch.cuda.Event()
                job.event.record(job.stream)
                if isinstance(job.result, CASCISolver):
                    job.result._ready_event = job.event
                job.t_done = time.perf_counter()
                self._free[1 if job.stream.priority < 0 else 0].append(job.stream)
                return True

    def _launch_parked(self, parked):
        """One graph launch for the iterations of every parked job; each job resumes when it ends."""
        import ctypes as C

        torch = _torch()
        if self._batch_stream is None:
            self._batch_stream = torch.cuda.Stream()
        s = self._batch_stream
        for job in parked:
            s.wait_event(job.event)  # the job's reset and set-up work comes first
        handles = [job.request.handle for job in parked]
        with torch.cuda.stream(s):
            if len(handles) == 1:
                check(lib().f2g_dgraph_launch(handles[0], s.cuda_stream))
            else:
                serials = []
                for h in handles:
                    v = C.c_uint64()
                    check(lib().f2g_dgraph_serial(h, C.addressof(v)))
                    serials.append(v.value)
                key = tuple(serials)
                b = self._batches.get(key)
                if b is None:
                    arr = (C.c_void_p * len(handles))(*[h.value for h in handles])
                    b = C.c_void_p()
                    check(lib().f2g_dgraph_batch_create(C.addressof(arr), len(handles), C.byref(b)))
                    self._batches[key] = b
                    nodes = C.c_int()
                    check(lib().f2g_dgraph_batch_nodes(b, C.addressof(nodes)))
                    self.batch_nodes = max(self.batch_nodes, nodes.value)
                check(lib().f2g_dgraph_batch_launch(b, s.cuda_stream))
        ev = torch.cuda.Event()
        ev.record(s)
        for job in parked:
            job.stream.wait_event(ev)
            job.event = ev
            job.request = []
        self.batch_launches += 1
        self.batch_solves += len(parked)

    def close(self):
        """Destroy the collective launches' graphs (their member solves must still exist)."""
        for b in self._batches.values():
            lib().f2g_dgraph_batch_destroy(b)
        self._batches = {}

    @staticmethod
    def _read(job):
        if not job.request:
            return []
        torch = _torch()
        with torch.cuda.stream(job.stream):
            return [t.cpu().numpy() for t in job.request]

    def run(self, jobs=(), admit=None, on_done=None, idle_wait=None):
        """Run jobs (iterable of (key, generator)) plus whatever ``admit(now, active)`` returns
        ((key, generator, footprint[, high]) tuples), until nothing is active and ``admit`` reports
        no more work (returns None). Jobs admitted with high=True run on high-priority streams, so
        the block scheduler serves their small kernels before waiting blocks of long kernels."""
        torch = _torch()
        active = []
        done = []

        def finish(job):
            done.append(job)
            if on_done:
                on_done(job)

        def start(key, gen, footprint=0, high=False):
            t0 = time.perf_counter()
            job = Job(key, gen, self._stream(high), t_admit=t0, footprint=footprint)
            if self._resume(job, None):
                finish(job)
            else:
                active.append(job)
            self.host_s["start"] += time.perf_counter() - t0

        for key, gen in jobs:
            start(key, gen)
        while True:
            if admit is not None:
                t0 = time.perf_counter()
                new = admit(t0, active)
                self.host_s["admit"] += time.perf_counter() - t0
                if new is None and not active:
                    break
                for item in new or ():
                    start(*item)
            elif not active:
                break
            if not active:
                if idle_wait:
                    idle_wait()
                continue
            self.polls += 1
            still = []
            progressed = False
            for job in active:
                if isinstance(job.request, GraphPhase):
                    still.append(job)  # parked until the collective launch
                    continue
                if not job.event.query():
                    still.append(job)
                    continue
                progressed = True
                self.rounds += 1
                t0 = time.perf_counter()
                fin = self._resume(job, self._read(job))
                self.host_s["resume"] += time.perf_counter() - t0
                if fin:
                    finish(job)
                else:
                    still.append(job)
            active = still
            parked = [job for job in active if isinstance(job.request, GraphPhase)]
            if parked and len(parked) == len(active):
                self._launch_parked(parked)
                progressed = True
            if not progressed and self.poll_sleep:
                time.sleep(self.poll_sleep)
        torch.cuda.synchronize()
        self.close()
        return done


# ---- workload definitions ------------------------------------------------------------------

def batched_instances(n_inst: int = 64, seed: int = 4000):
    """The batched workload: active spaces (8e,8o), (10e,10o), (12e,12o) drawn uniformly,
    Ms = 0, multiplicity 1 or 3, 1-4 roots, each instance with its own seeded integrals."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_inst):
        n = int(rng.choice([8, 10, 12]))
        mult = int(rng.choice([1, 3]))
        nroot = int(rng.integers(1, 5))
        out.append(dict(norb=n, na=n // 2, nb=n // 2, multiplicity=mult, nroot=nroot, iseed=seed + 1 + i))
    return out


LARGE_NDET = 200_000  # spaces from here on are bound by sigma arithmetic, not by launches


def make_solver(inst, precision="fp64", e_tol=1e-10, maxiter=2000, autotune=True, ints=None, one_launch=False,
                sigma_variants=None):
    """One instance's solver; its sigma kernel variants are autotuned once per shape. Spaces of at
    least LARGE_NDET determinants get the larger Davidson subspace (12 vectors per root, collapse
    to 6, at most 64) in both precisions: the same energies in about a third of the iterations
    (the plain drop-in path keeps the reference's 4 and 2)."""
    ints = make_integrals(inst["norb"], inst["iseed"]) if ints is None else ints
    dl = DavidsonLiuParams(e_tol=e_tol, maxiter=maxiter)
    if comb(inst["norb"], inst["na"]) * comb(inst["norb"], inst["nb"]) >= LARGE_NDET:
        bpr = min(12, 64 // inst["nroot"])
        dl = DavidsonLiuParams(e_tol=e_tol, maxiter=maxiter, basis_per_root=bpr, collapse_per_root=min(6, bpr - 1))
    return CASCISolver(norb=inst["norb"], na=inst["na"], nb=inst["nb"], multiplicity=inst["multiplicity"],
                       nroot=inst["nroot"], E=ints.E, H=ints.H, V=ints.V, ci_params=CIParams(precision=precision),
                       davidson_liu_params=dl, autotune=autotune, one_launch=one_launch,
                       sigma_variants=sigma_variants)


def footprint_bytes(norb: int, na: int, nb: int, nroot: int, basis_per_root: int = 0) -> int:
    """Estimated device bytes of one CASCI solve (vectors, scratch, string Hamiltonian, CSF maps);
    basis_per_root 0 = the subspace make_solver gives this space."""
    n0a, n0b = comb(norb, na), comb(norb, nb)
    ndet = n0a * n0b
    if not basis_per_root:
        basis_per_root = min(12, 64 // nroot) if ndet >= LARGE_NDET else 4
    m = basis_per_root * nroot
    nnz_a = 1 + na * (norb - na) + comb(na, 2) * comb(norb - na, 2)
    nnz_b = 1 + nb * (norb - nb) + comb(nb, 2) * comb(norb - nb, 2)
    ss = 12 * (n0a * nnz_a + n0b * nnz_b) * 3 // 2  # FP64 + FP32 values, int32 columns
    det_vectors = 8 * ndet * (6 + 2 * m)  # C/sigma staging, transposes, closure buffers
    csf = 4 * ndet + 8 * ndet  # permutation + configuration tables (upper bound)
    davidson = 8 * ndet * (3 * m + 2)  # basis, sigma, residual rows (ncsf <= ndet)
    return int(ss + det_vectors + csf + davidson + (64 << 20))


def solve_batched(instances, precision="fp64", nstreams=16, one_launch=False, stats=None):
    """Solve all instances concurrently; returns (results by index, seconds, rounds). With
    one_launch=True the instances' Davidson iterations run in collective graph launches (one per
    solve phase: set-up and any host-side steps of each instance stay on its own stream); stats,
    a dict, receives the scheduler's launch counts."""
    torch = _torch()
    sched = StepScheduler(nstreams, one_launch=one_launch)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    jobs = [(i, make_solver(inst, precision, one_launch=one_launch).run_steps()) for i, inst in enumerate(instances)]
    done = sched.run(jobs)
    dt = time.perf_counter() - t0
    if stats is not None:
        stats.update(batch_launches=sched.batch_launches, batch_solves=sched.batch_solves,
                     batch_nodes=sched.batch_nodes)
    return {j.key: j.result for j in done}, dt, sched.rounds


def solve_loop(instances, precision="fp64"):
    """The baseline: one plain solve after the other."""
    torch = _torch()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = {i: make_solver(inst, precision).run() for i, inst in enumerate(instances)}
    torch.cuda.synchronize()
    return out, time.perf_counter() - t0
