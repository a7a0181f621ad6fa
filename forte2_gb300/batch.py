"""Many CASCI solves in flight on one GPU: batched instances and a continuous-batching server.

Every solve is a step generator (``CASCISolver.run_steps``): it enqueues device work on its
CUDA stream and yields the small device tensors it must read next. ``StepScheduler`` resumes
every runnable job once per round (each on its own stream from a pool, so their kernels overlap
on the device), then synchronises the device once, copies all requested values to the host in one
transfer, and hands them back. New jobs can be admitted between rounds (``admit`` callback): the
serving loop admits arriving requests while their estimated HBM footprint fits the budget.
"""

from __future__ import annotations

import heapq
import time
from dataclasses import dataclass, field
from math import comb

import numpy as np

from .ci import CASCISolver
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
    request: list = None
    result: object = None
    t_admit: float = 0.0
    t_done: float = 0.0
    footprint: int = 0
    steps: int = 0


class StepScheduler:
    """Round-robin driver of step generators with one device synchronisation per round."""

    def __init__(self, nstreams: int = 16):
        torch = _torch()
        self.streams = [torch.cuda.Stream() for _ in range(nstreams)]
        self._next_stream = 0
        self.rounds = 0

    def _stream(self):
        s = self.streams[self._next_stream % len(self.streams)]
        self._next_stream += 1
        return s

    def _resume(self, job, values):
        torch = _torch()
        with torch.cuda.stream(job.stream):
            try:
                job.request = job.gen.send(values) if values is not None else next(job.gen)
                job.steps += 1
                return False
            except StopIteration as e:
                job.result = e.value
                job.t_done = time.perf_counter()
                return True

    def run(self, jobs=(), admit=None, on_done=None, idle_wait=None):
        """Run jobs (iterable of (key, generator)) plus whatever ``admit(now, active)`` returns each
        round, until nothing is active and ``admit`` reports no more work (returns None)."""
        torch = _torch()
        active = []
        done = []

        def start(key, gen, footprint=0):
            job = Job(key, gen, self._stream(), t_admit=time.perf_counter(), footprint=footprint)
            if self._resume(job, None):
                done.append(job)
                if on_done:
                    on_done(job)
            else:
                active.append(job)

        for key, gen in jobs:
            start(key, gen)
        while True:
            if admit is not None:
                new = admit(time.perf_counter(), active)
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
            self.rounds += 1
            # one synchronisation and one D2H transfer for every value requested this round
            # (the jobs' streams are synchronised before the gather, which runs on this thread's
            # current stream and must see every job's results)
            reqs = [t for job in active for t in job.request]
            torch.cuda.synchronize()
            if reqs:
                flat = torch.cat([t.reshape(-1) for t in reqs]) if len(reqs) > 1 else reqs[0].reshape(-1)
                host = flat.cpu().numpy()
            else:
                host = np.zeros(0)
            pos = 0
            still = []
            for job in active:
                vals = []
                for t in job.request:
                    n = t.numel()
                    vals.append(host[pos : pos + n].reshape(t.shape))
                    pos += n
                if self._resume(job, vals):
                    done.append(job)
                    if on_done:
                        on_done(job)
                else:
                    still.append(job)
            active = still
        torch.cuda.synchronize()
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


def make_solver(inst, precision="fp64", e_tol=1e-10, maxiter=400):
    ints = make_integrals(inst["norb"], inst["iseed"])
    return CASCISolver(norb=inst["norb"], na=inst["na"], nb=inst["nb"], multiplicity=inst["multiplicity"],
                       nroot=inst["nroot"], E=ints.E, H=ints.H, V=ints.V, ci_params=CIParams(precision=precision),
                       davidson_liu_params=DavidsonLiuParams(e_tol=e_tol, maxiter=maxiter))


def footprint_bytes(norb: int, na: int, nb: int, nroot: int, basis_per_root: int = 4) -> int:
    """Estimated device bytes of one CASCI solve (vectors, scratch, string Hamiltonian, CSF maps)."""
    n0a, n0b = comb(norb, na), comb(norb, nb)
    ndet = n0a * n0b
    m = basis_per_root * nroot
    nnz_a = 1 + na * (norb - na) + comb(na, 2) * comb(norb - na, 2)
    nnz_b = 1 + nb * (norb - nb) + comb(nb, 2) * comb(norb - nb, 2)
    ss = 12 * (n0a * nnz_a + n0b * nnz_b) * 3 // 2  # FP64 + FP32 values, int32 columns
    det_vectors = 8 * ndet * (6 + 2 * m)  # C/sigma staging, transposes, closure buffers
    csf = 4 * ndet + 8 * ndet  # permutation + configuration tables (upper bound)
    davidson = 8 * ndet * (3 * m + 2)  # basis, sigma, residual rows (ncsf <= ndet)
    return int(ss + det_vectors + csf + davidson + (64 << 20))


def solve_batched(instances, precision="fp64", nstreams=16):
    """Solve all instances concurrently; returns (results by index, seconds, rounds)."""
    torch = _torch()
    sched = StepScheduler(nstreams)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    jobs = [(i, make_solver(inst, precision).run_steps()) for i, inst in enumerate(instances)]
    done = sched.run(jobs)
    dt = time.perf_counter() - t0
    return {j.key: j.result for j in done}, dt, sched.rounds


def solve_loop(instances, precision="fp64"):
    """The baseline: one plain solve after the other."""
    torch = _torch()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = {i: make_solver(inst, precision).run() for i, inst in enumerate(instances)}
    torch.cuda.synchronize()
    return out, time.perf_counter() - t0
