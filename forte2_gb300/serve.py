"""Continuous-batching CASCI solve server on one GPU.

Requests (active space, multiplicity, roots, integrals) arrive over time. Each round of the step
scheduler admits waiting requests in arrival order while the estimated HBM footprint of all
solves in flight stays within the budget, so requests that arrive while others run join as soon
as memory frees up, and their kernels overlap on the device with the others'. Latency is measured
from a request's arrival to its result.
"""

from __future__ import annotations

import time
from collections import deque
from dataclasses import dataclass
from math import comb

import numpy as np

from .batch import StepScheduler, footprint_bytes, make_solver
from .synthetic import make_integrals


@dataclass
class Request:
    idx: int
    arrival: float  # seconds after the start of the stream
    norb: int
    multiplicity: int
    nroot: int
    iseed: int

    ints: object = None  # the request's integrals (the client sends them with the request)

    @property
    def inst(self):
        return dict(norb=self.norb, na=self.norb // 2, nb=self.norb // 2, multiplicity=self.multiplicity,
                    nroot=self.nroot, iseed=self.iseed)

    def integrals(self):
        if self.ints is None:
            self.ints = make_integrals(self.norb, self.iseed)
        return self.ints


def poisson_stream(n_requests=10000, rate=200.0, seed=5, sizes=(6, 8, 10, 12, 14, 16)):
    """The serving workload: Poisson arrivals at `rate` per second; active spaces (n e, n o), Ms = 0,
    drawn with weight 1/Ndet(n); multiplicity 1 or 3; 1-3 roots; per-request seeded integrals."""
    rng = np.random.default_rng(seed)
    w = np.array([1.0 / comb(n, n // 2) ** 2 for n in sizes])
    w /= w.sum()
    t = np.cumsum(rng.exponential(1.0 / rate, n_requests))
    n = rng.choice(sizes, size=n_requests, p=w)
    mult = rng.choice([1, 3], size=n_requests)
    roots = rng.integers(1, 4, size=n_requests)
    return [Request(i, float(t[i]), int(n[i]), int(mult[i]), int(roots[i]), 7_000_000 + i) for i in range(n_requests)]


def request_precision(r, precision, mixed_min_ndet=200_000):
    """Precision a request runs in. In mixed mode only spaces of at least mixed_min_ndet
    determinants use FP32 sigma builds: below that a solve is bound by launches and host steps,
    not by sigma arithmetic, and plain FP64 is both faster and exact."""
    if precision == "mixed" and comb(r.norb, r.norb // 2) ** 2 < mixed_min_ndet:
        return "fp64"
    return precision


class SolverPool:
    """Idle solvers by shape (orbitals, multiplicity, roots, precision). A request of a shape seen
    before takes an idle solver and only uploads its integrals: strings, spin adapter, sigma-builder
    buffers, eigensolver buffers and captured iteration graphs are all reused. Idle solvers keep
    their device memory, so they count against the HBM budget and the least recently used ones are
    dropped when an admission needs the room."""

    def __init__(self, precision, e_tol, mixed_min_ndet=200_000):
        self.precision, self.e_tol, self.mixed_min_ndet = precision, e_tol, mixed_min_ndet
        self.idle = {}  # key -> list of (solver, footprint), most recent last
        self.order = deque()  # keys of idle solvers, least recent first
        self.idle_bytes = 0
        self.created = 0
        self.reused = 0
        self.prewarmed = 0

    def prec(self, r):
        return request_precision(r, self.precision, self.mixed_min_ndet)

    def key(self, r):
        return (r.norb, r.multiplicity, r.nroot, self.prec(r))

    def take(self, r):
        lst = self.idle.get(self.key(r))
        if lst:
            solver, fp = lst.pop()
            self.order.remove(self.key(r))
            self.idle_bytes -= fp
            ints = r.integrals()
            solver.new_problem(ints.E, ints.H, ints.V)
            self.reused += 1
            return solver
        self.created += 1
        return make_solver(r.inst, self.prec(r), e_tol=self.e_tol, ints=r.integrals(),
                           sigma_variants=self.variants(r))

    def variants(self, r):
        """Kernel variants of a new solver made while the server runs: the FP32 options whose
        operands are allocated on first use (TMA-fed B tiles, dense same-spin GEMMs) stay off, since
        allocating device memory synchronises the device under every solve in flight."""
        return {"tma_b": 0, "dense_same_spin": 0} if self.prec(r) == "mixed" else None

    def has_idle(self, r):
        return bool(self.idle.get(self.key(r)))

    def give(self, r, solver, fp):
        self.idle.setdefault(self.key(r), []).append((solver, fp))
        self.order.append(self.key(r))
        self.idle_bytes += fp

    def prewarm(self, shapes, nstreams=16):
        """Create idle solvers before requests arrive: for each (norb, multiplicity, nroot, count)
        `count` solvers, each run once on seeded integrals so that its tables, buffers and
        captured iteration graphs exist (creating them synchronises the device, which a running
        server should not do per request). Returns the number created."""
        jobs = []
        for norb, mult, nroot, count in shapes:
            for _ in range(count):
                r = Request(-1, 0.0, norb, mult, nroot, 9_000_000 + len(jobs))
                solver = make_solver(r.inst, self.prec(r), e_tol=self.e_tol)
                jobs.append(((r, solver), solver.run_steps()))
        StepScheduler(nstreams).run(jobs)
        for (r, solver), _ in jobs:
            self.give(r, solver, footprint_bytes(r.norb, r.norb // 2, r.norb // 2, r.nroot))
        self.created += len(jobs)
        self.prewarmed = len(jobs)
        return len(jobs)

    def evict_one(self):
        if not self.order:
            return False
        k = self.order.popleft()
        _, fp = self.idle[k].pop(0)
        self.idle_bytes -= fp
        return True


def default_prewarm(sizes=(6, 8, 10), per_size=(16, 6, 2)):
    """Idle solvers to create before a stream: for every multiplicity 1/3 and 1-3 roots, per_size[i]
    solvers of (sizes[i] e, sizes[i] o) (the small spaces that make up almost all requests)."""
    return [(n, mult, nroot, c) for n, c in zip(sizes, per_size) for mult in (1, 3) for nroot in (1, 2, 3)]


def sm_count():
    import torch

    return torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count


def serve(requests, precision="fp64", hbm_budget=200 << 30, nstreams=16, e_tol=1e-10, max_inflight=256,
          pool=True, small_norb=10, mixed_min_ndet=200_000, prewarm=None, reserve_sms=48):
    """Serve a request stream in real time; returns per-request latencies and summary stats.
    prewarm: (norb, multiplicity, nroot, count) shapes of idle solvers to create before the clock
    starts (see SolverPool.prewarm)."""
    sp = SolverPool(precision, e_tol, mixed_min_ndet)
    t0 = time.perf_counter()
    if pool and prewarm:
        sp.prewarm(prewarm, nstreams)
    prewarm_s = time.perf_counter() - t0
    for r in requests:  # the payload each client sends: made before the clock starts
        r.integrals()
    sched = StepScheduler(nstreams)
    pending = deque(sorted(requests, key=lambda r: r.arrival))
    waiting = deque()
    used = [0]  # footprint of the solves in flight
    lat = {}
    energies = {}
    t_start = time.perf_counter()
    peak = [0, 0]

    def admit(now, active):
        rel = now - t_start
        while pending and pending[0].arrival <= rel:
            waiting.append(pending.popleft())
        new = []
        while waiting and len(active) + len(new) < max_inflight:
            r = waiting[0]
            fp = footprint_bytes(r.norb, r.norb // 2, r.norb // 2, r.nroot)
            reuse = pool and sp.has_idle(r)
            extra = 0 if reuse else fp
            while used[0] + sp.idle_bytes + extra > hbm_budget and sp.evict_one():
                pass
            if used[0] + sp.idle_bytes + extra > hbm_budget and (active or new):
                break
            waiting.popleft()
            solver = sp.take(r) if pool else make_solver(r.inst, sp.prec(r), e_tol=e_tol, ints=r.integrals())
            if r.norb > small_norb:
                # a large solve leaves reserve_sms SMs to the small latency-bound ones
                solver.sigma_max_blocks = max(1, sm_count() - reserve_sms)
            used[0] += fp
            # small spaces (latency bound, many requests) on high-priority streams: a long kernel
            # of a large request then does not hold their short kernels back
            new.append(((r, solver), solver.run_steps(), fp, r.norb <= small_norb))
        peak[0] = max(peak[0], len(active) + len(new))
        peak[1] = max(peak[1], used[0] + sp.idle_bytes)
        if not new and not active and not waiting:
            if not pending:
                return None
            # idle until the next arrival
            time.sleep(max(0.0, pending[0].arrival - (time.perf_counter() - t_start)))
        return new

    def on_done(job):
        r, solver = job.key
        used[0] -= job.footprint
        lat[r.idx] = (job.t_done - t_start) - r.arrival
        energies[r.idx] = [float(e) for e in job.result.evals]
        if pool:
            sp.give(r, solver, job.footprint)

    sched.run(admit=admit, on_done=on_done)
    wall = time.perf_counter() - t_start
    L = np.array([lat[r.idx] for r in requests])
    return {
        "requests": len(requests), "precision": precision, "wall_s": wall,
        "solves_per_s": len(requests) / wall, "p50_latency_s": float(np.percentile(L, 50)),
        "p99_latency_s": float(np.percentile(L, 99)), "mean_latency_s": float(L.mean()),
        "max_inflight": peak[0], "peak_footprint_gb": peak[1] / 2**30, "rounds": sched.rounds,
        "solvers_created": sp.created, "solvers_reused": sp.reused, "solvers_prewarmed": sp.prewarmed,
        "prewarm_s": round(prewarm_s, 3), "streams": sched.max_streams,
        "host_s": {k: round(v, 3) for k, v in sched.host_s.items()}, "polls": sched.polls,
        "sizes": {int(n): int(sum(1 for r in requests if r.norb == n)) for n in sorted({r.norb for r in requests})},
    }, lat, energies
