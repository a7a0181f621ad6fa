"""GPU-resident Davidson-Liu eigensolver with the reference's call surface and semantics
(forte2/helpers/davidsonliu.py:12-515).

Basis, sigma and residual vectors live on the device as rows of (m, size) FP64 tensors; the
subspace matrix, its eigendecomposition (Jacobi), residuals, preconditioner and Gram-Schmidt all
run in the library's CUDA kernels. The host only reads back the handful of scalars that decide
convergence (eigenvalues, residual norms, overlaps).

The algorithm is written as a step generator (``solve_steps``): it enqueues device work and
yields the list of small device tensors whose values it needs next; the driver copies them to
the host after one synchronisation and sends the numpy arrays back. ``solve()`` drives one
generator; ``forte2_gb300.batch`` interleaves many of them (batched and serving workloads), so
that all solves in flight share one device synchronisation per round.

Sigma builders: ``add_sigma_builder(f)`` takes ``f(basis_block, sigma_block)``. If ``f`` has the
attribute ``device_rows = True`` it receives CUDA tensors of shape (m, size) (rows are vectors)
and only enqueues work; otherwise it receives numpy arrays of shape (size, m) exactly as the
reference passes them.

Differences from the reference, all at the level of rounding or documented choices:
  * Gram-Schmidt projects against all accepted vectors at once (classical Gram-Schmidt applied
    repeatedly) instead of one vector at a time; the acceptance tests (discard below 1e-8,
    orthonormal to 1e-12, at most 10 cycles) are the reference's (davidsonliu.py:438-484);
  * random vectors (no guesses, or refill after discards) come from a seeded generator, so
    solves are reproducible (the reference uses an unseeded default_rng, davidsonliu.py:114);
  * the initial guesses are orthonormalised by the same Gram-Schmidt instead of a Householder QR.
"""

from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from ._lib import check, lib, stream_handle
from .params import DavidsonLiuParams


def _torch():
    import torch

    return torch


def _ptr(t):
    return t.data_ptr()


def to_device(a):
    """Small host array -> device tensor without a host wait: staged in pinned memory (torch's
    caching host allocator) and copied in stream order."""
    torch = _torch()
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64)).pin_memory().to("cuda", non_blocking=True)


class GraphPhase:
    """Yielded by a graph-captured solve whose iterations wait for a collective launch: a
    scheduler launches the iterations of all waiting solves in one graph (f2g_dgraph_batch_*);
    resumed with [] once that launch has completed."""

    __slots__ = ("handle",)

    def __init__(self, handle):
        self.handle = handle


def drive(gen):
    """Run a step generator to completion on the current stream; returns its return value. A
    GraphPhase is launched alone."""
    torch = _torch()
    try:
        req = next(gen)
        while True:
            if isinstance(req, GraphPhase):
                check(lib().f2g_dgraph_launch(req.handle, stream_handle()))
                req = []
            torch.cuda.current_stream().synchronize()
            req = gen.send([t.cpu().numpy() for t in req])
    except StopIteration as e:
        return e.value


@dataclass
class DavidsonLiuSolver:
    size: int
    nroot: int
    davidson_liu_params: DavidsonLiuParams = field(default_factory=DavidsonLiuParams)
    energy_shift: float = None
    log_level: int = 3
    dtype: type = np.float64
    seed: int = 12345
    logger: object = None
    # stop (unconverged) when the largest residual norm has not halved over this many iterations;
    # 0 disables. Used by the FP32 phase of the mixed-precision driver, whose residuals stall at
    # the FP32 rounding level.
    stall_window: int = 0
    stall_floor: float = 0.0  # the stall rule applies only once the residual is below this
    # Graph-captured iterations (f2g_dgraph_*): None = whenever the sigma builder supports it and
    # size <= graph_max_size; True/False force it on/off.
    use_graph: bool = None
    graph_max_size: int = 1 << 40
    iters_per_launch: int = 8

    def __post_init__(self):
        p = self.davidson_liu_params
        self.collapse_per_root = p.collapse_per_root
        self.basis_per_root = p.basis_per_root
        self.maxiter = p.maxiter
        self.e_tol = p.e_tol
        self.r_tol = p.r_tol
        if self.size <= 0:
            raise ValueError("Davidson-Liu solver called with space of dimension smaller than 1.")
        if self.nroot <= 0:
            raise ValueError("Davidson-Liu solver called with zero roots.")
        if not np.issubdtype(np.dtype(self.dtype), np.floating):
            raise NotImplementedError("the GPU Davidson-Liu solver is real (float64) only")
        torch = _torch()
        self.collapse_size = min(self.collapse_per_root * self.nroot, self.size)
        self.max_subspace_size = min(self.basis_per_root * self.nroot, self.size)
        if self.max_subspace_size > 64:
            raise ValueError("the GPU Davidson-Liu solver supports at most 64 basis vectors")
        dev = "cuda"
        f64 = torch.float64
        m, n = self.max_subspace_size, self.size
        self.b = torch.zeros((m, n), dtype=f64, device=dev)
        self.sigma = torch.zeros((m, n), dtype=f64, device=dev)
        self.r = torch.zeros((max(self.nroot, m), n), dtype=f64, device=dev)
        self.tmp = torch.zeros((max(self.nroot, m), n), dtype=f64, device=dev)
        self.scratch = torch.zeros(int(lib().f2g_dav_scratch_size(n)), dtype=f64, device=dev)
        self.h_diag = None
        self.lam = np.zeros(m)
        self.lam_old = np.zeros(m)
        self.alpha = np.zeros((m, m))
        self.schmidt_discard_threshold = 1e-8
        self.schmidt_orthogonality_threshold = 1e-12
        self.preconditioner_denom_threshold = 1e-8
        self.basis_size = 0
        self.sigma_size = 0
        self._build_sigma = None
        self._executed = False
        self._gen = torch.Generator(device=dev)
        self._gen.manual_seed(int(self.seed))
        self.iter = 0
        self.converged = False
        self.sigma_builds = 0
        self.history = []
        self._graphs = {}
        self._tmp2 = None
        self.used_graph = False
        # graph iterations wait for a collective launch (GraphPhase) instead of launching themselves
        self.collective = False
        self._G = None  # subspace matrix B S^T, valid for the first _g_size rows and columns
        self._g_size = 0

    # ---- configuration (davidsonliu.py:116-182) ----
    def add_sigma_builder(self, sigma_builder):
        self._build_sigma = sigma_builder

    def add_h_diag(self, h_diag):
        torch = _torch()
        if not isinstance(h_diag, torch.Tensor):
            h_diag = torch.as_tensor(np.array(h_diag, dtype=np.float64))
        t = h_diag.to(torch.float64).reshape(-1)
        if t.shape != (self.size,):
            raise ValueError("h_diag must be shape (size,)")
        if self.h_diag is None:
            self.h_diag = t.to("cuda").contiguous().clone()
        else:  # same buffer: captured graphs keep its address
            self.h_diag.copy_(t)

    def add_guesses(self, guesses):
        torch = _torch()
        G = torch.as_tensor(guesses, dtype=torch.float64)
        if G.dim() != 2 or G.shape[0] != self.size:
            raise ValueError("guesses must be shape (size, n_guess)")
        self._guesses = G.to("cuda").T.contiguous()  # rows

    def add_guess_rows(self, rows):
        """Guesses as a device tensor of rows (n_guess, size); no host round trip."""
        if rows.dim() != 2 or rows.shape[1] != self.size:
            raise ValueError("guess rows must be shape (n_guess, size)")
        self._guesses = rows.contiguous()

    def add_project_out(self, project_out):
        """Vectors to project out (davidsonliu.py:150-172); shorter vectors are zero-padded."""
        torch = _torch()
        if len(project_out) == 0:
            return
        for v in project_out:
            if len(v) > self.size:
                raise ValueError(
                    f"Each project_out vector must have length at most {self.size}, but got {len(v)}")
        A = torch.zeros((len(project_out), self.size), dtype=torch.float64, device="cuda")
        for i, v in enumerate(project_out):
            A[i, : len(v)] = torch.as_tensor(np.asarray(v, dtype=np.float64), device="cuda")
        Q = torch.zeros_like(A)
        k = 0
        for i in range(A.shape[0]):
            ok, v = drive(self._orthonormalize_steps(Q[:k], A[i].clone()))
            if ok:
                Q[k] = v
                k += 1
        self._proj_out = Q[:k].contiguous()

    # ---- device primitives (enqueue only) ----
    def _dots_dev(self, A, B):
        """Device tensor (na, nb) of <A_i, B_j> for row blocks A, B."""
        torch = _torch()
        na, nb = A.shape[0], B.shape[0]
        out = torch.empty((max(na, 1), max(nb, 1)), dtype=torch.float64, device="cuda")
        if na and nb:
            check(lib().f2g_dav_dots(_ptr(A), na, A.stride(0), _ptr(B), nb, B.stride(0), self.size, _ptr(out),
                                     _ptr(self.scratch), stream_handle()))
        return out[:na, :nb]

    def _lincomb(self, X, coef, Y, beta):
        """Y_j = beta Y_j + sum_i coef[i, j] X_i; coef is numpy (nx, ny) or a device tensor."""
        torch = _torch()
        nx, ny = coef.shape
        if nx == 0 or ny == 0:
            if beta != 1.0 and ny:
                Y.mul_(beta)
            return
        if isinstance(coef, torch.Tensor):
            c = coef.contiguous()
        else:
            c = to_device(coef)
        check(lib().f2g_dav_lincomb(_ptr(X), nx, X.stride(0), _ptr(c), ny, _ptr(Y), Y.stride(0), float(beta),
                                    self.size, stream_handle()))

    def _dots(self, A, B):
        """Blocking <A_i, B_j> -> numpy (na, nb) (for callers outside a step generator)."""
        return drive(self._read_steps(self._dots_dev(A, B)))

    @staticmethod
    def _read_steps(t):
        (h,) = yield [t]
        return h

    # ---- step routines: enqueue device work, `yield [tensors]` to read values on the host ----
    def do_project_out(self, A):
        """A_i -> (1 - u u^T) A_i for every stored project-out vector u (davidsonliu.py:174-182).
        Enqueue only: the projections are consumed on the device."""
        if not hasattr(self, "_proj_out") or A.shape[0] == 0:
            return
        for k in range(self._proj_out.shape[0]):
            u = self._proj_out[k : k + 1]
            v = self._dots_dev(u, A)  # (1, nA)
            self._lincomb(u, -v, A, 1.0)

    def _orthonormality_steps(self, b, msg="Orthonormality check failed."):
        if b.shape[0] == 0:
            return
        (S,) = yield [self._dots_dev(b, b)]
        if not np.allclose(S, np.eye(S.shape[0]), atol=1e-11):
            raise ValueError(msg + f" Largest deviation from orthonormality: {np.max(np.abs(S - np.eye(S.shape[0])))}")

    def orthonormality_check(self, b, msg="Orthonormality check failed."):
        drive(self._orthonormality_steps(b, msg))

    def _orthonormalize_steps(self, A, v):
        """Orthonormalise v against the rows of A (davidsonliu.py:438-484). Returns (ok, v)."""
        vr = v[None, :]
        for _ in range(10):
            if A.shape[0]:
                d = self._dots_dev(A, vr)
                self._lincomb(A, -d, vr, 1.0)
                # the norm and the overlaps of the projected vector in one host read; the overlaps
                # of the normalised vector are these over the norm
                nrm2, ov = yield [self._dots_dev(vr, vr), self._dots_dev(A, vr)]
            else:
                (nrm2,) = yield [self._dots_dev(vr, vr)]
                ov = np.zeros(1)
            nrm = float(np.sqrt(max(nrm2[0, 0], 0.0)))
            if nrm < self.schmidt_discard_threshold:
                return False, v
            v.mul_(1.0 / nrm)
            max_overlap = float(np.abs(ov).max()) / nrm
            n2 = float(nrm2[0, 0]) / (nrm * nrm)
            if max_overlap < self.schmidt_orthogonality_threshold and abs(n2 - 1.0) < self.schmidt_orthogonality_threshold:
                return True, v
        return False, v

    def _add_rows_steps(self, n_existing, candidates):
        """Append orthonormalised candidate rows after the first n_existing basis rows."""
        added = 0
        cap = self.max_subspace_size - n_existing
        if candidates.shape[0] > cap:
            raise ValueError(f"Cannot add {candidates.shape[0]} candidates into {cap} slots")
        for j in range(candidates.shape[0]):
            v = candidates[j].clone()
            ok, v = yield from self._orthonormalize_steps(self.b[: n_existing + added], v)
            if ok:
                self.b[n_existing + added].copy_(v)
                added += 1
        return added

    def _random_rows(self, k):
        torch = _torch()
        return torch.rand((k, self.size), generator=self._gen, dtype=torch.float64, device="cuda") * 2.0 - 1.0

    def _sigma_steps(self, lo, hi):
        if getattr(self._build_sigma, "device_rows", False):
            self._build_sigma(self.b[lo:hi], self.sigma[lo:hi])
        else:
            torch = _torch()
            (B,) = yield [self.b[lo:hi]]
            B = np.ascontiguousarray(B.T)
            S = np.zeros_like(B)
            self._build_sigma(B, S)
            self.sigma[lo:hi].copy_(torch.as_tensor(np.ascontiguousarray(S.T)).to("cuda"))
        self.sigma_builds += hi - lo

    def _eigh_dev(self, m):
        """Enqueue the subspace matrix B S^T and its Jacobi eigendecomposition; returns (evals, evecs).

        Entries of rows and columns that were already in the previous subspace matrix are kept:
        only the pairs with a new basis or sigma row are computed (each pair's dot product is the
        same number however many pairs share a launch, so the matrix is bitwise the one a full
        recomputation gives). Anything that changes existing rows (collapse, a new solve, a
        projection) starts it afresh."""
        torch = _torch()
        k0 = self._g_size if (self._g_size <= m and not hasattr(self, "_proj_out")) else 0
        if self._G is None:
            self._G = torch.zeros((self.max_subspace_size, self.max_subspace_size), dtype=torch.float64,
                                  device="cuda")
        if k0 < m:
            self._G[:m, k0:m] = self._dots_dev(self.b[:m], self.sigma[k0:m])
            if k0 > 0:
                self._G[k0:m, :k0] = self._dots_dev(self.b[k0:m], self.sigma[:k0])
        self._g_size = m
        G = self._G[:m, :m].contiguous()
        ev = torch.empty(m, dtype=torch.float64, device="cuda")
        vec = torch.empty((m, m), dtype=torch.float64, device="cuda")
        check(lib().f2g_dav_eigh(m, _ptr(G), _ptr(ev), _ptr(vec), stream_handle()))
        return ev, vec

    def _collapse_steps(self, alpha):
        k = min(self.collapse_size, self.basis_size)
        m = self.basis_size
        yield from self._orthonormality_steps(self.b[:m], f"Before collapse: Checking orthonormality of Bblk with size {m}")
        self._lincomb(self.b[:m], alpha[:m, :k], self.tmp[:k], 0.0)
        self.b[:k].copy_(self.tmp[:k])
        self._lincomb(self.sigma[:m], alpha[:m, :k], self.tmp[:k], 0.0)
        self.sigma[:k].copy_(self.tmp[:k])
        self.basis_size = k
        self.sigma_size = k
        self._g_size = 0
        yield from self._orthonormality_steps(self.b[:k], f"After collapse: Checking orthonormality of newB with size {k}")

    def restart(self):
        """Forget the previous solution (the next solve starts from the guesses) but keep the
        buffers and captured graphs, for a new problem of the same size."""
        self._executed = False
        self.basis_size = self.sigma_size = 0
        self.lam_old[:] = 0.0
        if hasattr(self, "_guesses"):
            del self._guesses

    def __del__(self):
        try:
            for h in getattr(self, "_graphs", {}).values():
                lib().f2g_dgraph_destroy(h)
        except Exception:
            pass
        self._graphs = {}

    # ---- graph-captured iterations ----
    def _graph_spec(self):
        """(sigma builder, spin adapter, correction) when the graph path applies, else None."""
        spec = getattr(self._build_sigma, "graph", None)
        if spec is None or self.use_graph is False:
            return None
        if self.energy_shift is not None or hasattr(self, "_proj_out"):
            return None
        if self.use_graph is None and self.size > self.graph_max_size:
            return None
        return spec

    def _graph_for(self, spec):
        import ctypes as C

        torch = _torch()
        sb, sa, corr = spec
        key = (sb.h.value, sa.h.value, sb.get_precision(),
               None if corr is None else tuple(t.data_ptr() for t in corr[:3]) + (corr[3],))
        g = self._graphs.get(key)
        if g is not None and g[1] >= self.maxiter:
            return g[0]
        if g is not None:
            lib().f2g_dgraph_destroy(g[0])
        if self._tmp2 is None:
            self._tmp2 = torch.zeros((2 * self.collapse_size, self.size), dtype=torch.float64, device="cuda")
        thr = np.array([self.preconditioner_denom_threshold, self.schmidt_discard_threshold,
                        self.schmidt_orthogonality_threshold], dtype=np.float64)
        h = C.c_void_p()
        check(lib().f2g_dgraph_create(sb.h, sa.h, self.size, self.nroot, self.max_subspace_size, self.collapse_size,
                                      self.maxiter, int(self.seed), int(self.iters_per_launch), thr.ctypes.data,
                                      _ptr(self.b), _ptr(self.sigma), _ptr(self.r), _ptr(self._tmp2), self.b.stride(0),
                                      self.r.stride(0), self._tmp2.stride(0), _ptr(self.h_diag), C.byref(h)))
        if corr is not None:
            X, D, M, k = corr
            check(lib().f2g_dgraph_set_correction(h, _ptr(X), _ptr(D), X.stride(0), _ptr(M), int(k)))
        self._graphs[key] = (h, self.maxiter)
        return h

    def _solve_graph_steps(self, spec):
        """solve_steps with the iterations replayed from a captured graph: one host read per
        iters_per_launch iterations instead of several per iteration."""
        torch = _torch()
        L = lib()
        nroot, maxm = self.nroot, self.max_subspace_size
        self.used_graph = True
        g = self._graph_for(spec)
        dev_m = None
        if not self._executed:
            # Gram-Schmidt of the guesses decided on the device; the basis size stays on the device
            # until the first read, which overlaps the first launch of the iterations
            G = self._guesses if hasattr(self, "_guesses") else self._random_rows(nroot)
            ncand = min(G.shape[0], maxm)
            if getattr(self, "_added", None) is None:
                self._added = torch.zeros(1, dtype=torch.int32, device="cuda")
            dev_m = self._added
            check(L.f2g_dav_gs_append(_ptr(self.b), self.b.stride(0), maxm, 0, _ptr(G), G.stride(0), ncand, self.size,
                                      self.schmidt_discard_threshold, self.schmidt_orthogonality_threshold,
                                      min(nroot, maxm), int(self.seed), _ptr(dev_m), stream_handle()))
            m = max(ncand, min(nroot, maxm))  # rows that may hold a basis vector
            self.sigma_size = 0
            self.lam_old[:] = 0.0
        else:
            m = self.basis_size
        if m == 0:
            raise RuntimeError("Davidson-Liu solver: no basis vector survived orthonormalisation.")
        S = self._dots_dev(self.b[:m], self.b[:m]).contiguous()
        if m > self.sigma_size:
            # with a device basis size this covers every row the Gram-Schmidt may have filled;
            # rows beyond the accepted ones are computed needlessly and never used
            yield from self._sigma_steps(self.sigma_size, m)
        lam_old = np.ascontiguousarray(self.lam_old[:nroot])
        # the reset checks the starting overlap on the device; the first host read is the state
        # copied by the first launch
        check(L.f2g_dgraph_reset(g, m, -1 if dev_m is not None else m, _ptr(dev_m) if dev_m is not None else None,
                                 _ptr(S), S.stride(0), lam_old.ctypes.data, nroot, float(self.e_tol),
                                 float(self.r_tol), int(self.maxiter), int(self.stall_window), float(self.stall_floor),
                                 stream_handle()))
        self._graph_S = S  # kept alive until the reset has run
        ints = np.zeros(8, dtype=np.int32)
        dbl = np.zeros(131, dtype=np.float64)
        while True:
            if self.collective:
                # the scheduler launches the iterations of every waiting solve in one graph
                yield GraphPhase(g)
            else:
                check(L.f2g_dgraph_launch(g, stream_handle()))
                yield []
            check(L.f2g_dgraph_state(g, ints.ctypes.data, dbl.ctypes.data))
            if ints[3] != 0:
                break
        m, iters, status = int(ints[0]), int(ints[2]), int(ints[3])
        if status == 6:
            if m == 0:
                raise RuntimeError("Davidson-Liu solver: no basis vector survived orthonormalisation.")
            raise ValueError(f"Orthonormality check failed. Largest deviation from orthonormality: {dbl[130]}")
        if status == 4:
            raise ValueError(f"Before collapse: Checking orthonormality of Bblk with size {m}")
        if status == 5:
            raise ValueError(f"After collapse: Checking orthonormality of newB with size {self.collapse_size}")
        self.iter = iters - 1
        self.converged = status == 1
        self.sigma_builds += nroot * iters
        lamr = dbl[2 : 2 + nroot].copy()
        self.lam[:nroot] = lamr
        self.lam_old[:nroot] = dbl[66 : 66 + nroot]
        self.graph_status = status
        self._graph_last = (g, iters)
        check(L.f2g_dgraph_ritz(g, _ptr(self.tmp), self.tmp.stride(0), stream_handle()))
        self.b[:nroot].copy_(self.tmp[:nroot])
        self.basis_size = nroot
        self.sigma_size = 0
        self._executed = True
        self.evecs_rows = self.b[:nroot]
        return lamr, self.b[:nroot].T

    def graph_history(self):
        """Per-iteration (iteration, mean root energy, max |dE|, max |r|, basis size) of the last
        graph-captured solve (a blocking read)."""
        g, iters = self._graph_last
        h = np.zeros(4 * iters, dtype=np.float64)
        check(lib().f2g_dgraph_history(g, h.ctypes.data, iters))
        h = h.reshape(iters, 4)
        return [(i, h[i, 0], h[i, 1], h[i, 2], int(h[i, 3])) for i in range(iters)]

    def _log(self, msg):
        if self.logger is not None and self.log_level > 0:
            self.logger(msg)

    # ---- solve (davidsonliu.py:184-387) ----
    def solve_steps(self):
        """Step generator of solve(): yields lists of device tensors to read, returns (evals, evecs)."""
        if self._build_sigma is None:
            raise ValueError("Sigma builder function is not set.")
        if self.h_diag is None:
            raise ValueError("Hamiltonian diagonal is not set.")
        spec = self._graph_spec()
        if spec is not None:
            return (yield from self._solve_graph_steps(spec))
        self.used_graph = False
        self._g_size = 0  # rows may have been written since the last solve
        torch = _torch()
        if not self._executed:
            G = self._guesses.clone() if hasattr(self, "_guesses") else self._random_rows(self.nroot)
            self.do_project_out(G)
            k = 0
            for j in range(min(G.shape[0], self.max_subspace_size)):
                ok, v = yield from self._orthonormalize_steps(self.b[:k], G[j].clone())
                if ok:
                    self.b[k].copy_(v)
                    k += 1
            while k < min(self.nroot, self.max_subspace_size):  # dependent guesses: fill at random
                ok, v = yield from self._orthonormalize_steps(self.b[:k], self._random_rows(1)[0])
                if ok:
                    self.b[k].copy_(v)
                    k += 1
            self.basis_size = k
            self.sigma_size = 0
            self.lam_old[:] = 0.0
        yield from self._orthonormality_steps(self.b[: self.basis_size])
        self.iter = 0
        self.converged = False
        self.history = []
        nroot = self.nroot
        for self.iter in range(self.maxiter):
            t0 = time.perf_counter()
            if self.basis_size > self.sigma_size:
                yield from self._sigma_steps(self.sigma_size, self.basis_size)
                self.sigma_size = self.basis_size
            m = self.basis_size
            if hasattr(self, "_proj_out"):
                self.do_project_out(self.sigma[:m])
            ev, vec = self._eigh_dev(m)
            norms2 = torch.empty(nroot, dtype=torch.float64, device="cuda")

            def residual(d_alpha, d_lam):
                check(lib().f2g_dav_residual(_ptr(self.b), _ptr(self.sigma), m, self.b.stride(0), _ptr(d_alpha),
                                             _ptr(d_lam), nroot, _ptr(self.h_diag), self.size,
                                             self.preconditioner_denom_threshold, _ptr(self.r), self.r.stride(0),
                                             _ptr(norms2), _ptr(self.scratch), stream_handle()))

            if self.energy_shift is None:
                # the roots are the lowest eigenpairs, in the eigensolver's order: the residuals are
                # enqueued straight from its device output, one host read for both
                residual(vec[:, :nroot].contiguous(), ev[:nroot])
                lam, alpha, n2 = yield [ev, vec, norms2]
            else:
                lam, alpha = yield [ev, vec]
                idx = np.argsort(np.abs(lam - self.energy_shift))
                lam, alpha = lam[idx], alpha[:, idx]
                residual(to_device(alpha[:, :nroot]), to_device(lam[:nroot].copy()))
                (n2,) = yield [norms2]
            self.lam[:m] = lam
            self.alpha[:m, :m] = alpha
            lamr = lam[:nroot].copy()
            rnorms = np.sqrt(np.maximum(n2, 0.0))
            max_de = float(np.max(np.abs(lamr - self.lam_old[:nroot])))
            max_r = float(rnorms.max())
            self.history.append((self.iter, float(lamr.mean()), max_de, max_r, m, time.perf_counter() - t0))
            if (max_de < self.e_tol and max_r < self.r_tol) or self.basis_size == self.size:
                self.converged = True
                break
            w = self.stall_window
            if w and len(self.history) > w:
                recent = min(h[3] for h in self.history[-w:])
                before = min(h[3] for h in self.history[:-w])
                if recent > 0.5 * before and recent < self.stall_floor:
                    break
            if self.iter == self.maxiter - 1:
                break
            self.lam_old[:nroot] = lamr
            if self.basis_size + nroot > self.max_subspace_size:
                yield from self._collapse_steps(alpha)
            m = self.basis_size
            R0 = self.r[:nroot]
            d = self._dots_dev(self.b[:m], R0)  # R0 -= B (B^T R0), on the device
            self._lincomb(self.b[:m], -d, R0, 1.0)
            self.do_project_out(R0)
            to_add = min(nroot, self.max_subspace_size - self.basis_size)
            if to_add == 0:
                self.converged = True
                break
            added = yield from self._add_rows_steps(self.basis_size, R0[:to_add])
            self.basis_size += added
            if added < to_add:
                temp = self._random_rows(to_add - added)
                self.do_project_out(temp)
                added2 = yield from self._add_rows_steps(self.basis_size, temp)
                self.basis_size += added2
            self._log(f"iter {self.iter:4d} <E> {lamr.mean():20.12f} max(dE) {max_de:+.4e} max(r) {max_r:+.4e} "
                      f"basis {self.basis_size}")
        m = self.basis_size
        lamr = self.lam[:nroot].copy()
        self._lincomb(self.b[:m], self.alpha[:m, :nroot], self.tmp[:nroot], 0.0)
        self.b[:nroot].copy_(self.tmp[:nroot])
        self.basis_size = nroot
        self.sigma_size = 0
        self._executed = True
        self.evecs_rows = self.b[:nroot]
        return lamr, self.b[:nroot].T

    def solve(self):
        """Run to convergence (or maxiter) on the current stream; returns (evals, evecs (size, nroot))."""
        return drive(self.solve_steps())
