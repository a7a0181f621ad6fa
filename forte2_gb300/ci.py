"""CASCI driver with the reference's per-state solver semantics (forte2/ci/ci.py:30-836,
_CISingleStateSolver), device-resident end to end.

``CASCISolver.run()`` does what ``_CISingleStateSolver.run()`` does (ci.py:185-303): build the
strings and the CSF spin adapter, build the sigma builder with the current integrals, form the
CSF diagonal, build guess vectors from the lowest diagonal CSFs (ci.py:411-452), and run the
Davidson-Liu solver with the closure csf -> det -> H -> det -> csf (ci.py:221-235). Here every
vector stays on the GPU and each Davidson block is transformed and sigma-built in one call.

``precision="mixed"`` runs the Davidson iterations with FP32 sigma builds, then refines the
Ritz vectors by FP64 defect correction (``_solve_mixed``): a few FP64 sigma builds per root
instead of FP64 Davidson iterations. Orthogonalisation, residual norms and the subspace
eigensolves are FP64 throughout, and the reported energies come from an FP64 Rayleigh-Ritz step.
"""

from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from .ci_helpers import CISigmaBuilder, CISpinAdapter, CIStrings
from .davidson import DavidsonLiuSolver, drive
from .params import CIParams, DavidsonLiuParams


def _torch():
    import torch

    return torch


@dataclass
class CASCISolver:
    norb: int
    na: int
    nb: int
    multiplicity: int
    nroot: int
    E: float
    H: np.ndarray
    V: np.ndarray
    ci_params: CIParams = field(default_factory=CIParams)
    davidson_liu_params: DavidsonLiuParams = field(default_factory=DavidsonLiuParams)
    log_level: int = 0
    die_if_not_converged: bool = False
    # FP32 phase tolerances of the mixed mode (the FP64 phase uses davidson_liu_params)
    mixed_e_tol: float = 1e-7
    mixed_r_tol: float = 1e-4
    mixed_max_outer: int = 6
    # subspace of the mixed mode's Davidson (per root; the FP64 mode keeps the reference's
    # basis_per_root / collapse_per_root): a larger subspace needs fewer FP32 iterations
    mixed_basis_per_root: int = 12
    mixed_collapse_per_root: int = 6
    seed: int = 12345
    # the determinant space (CIStrings(na, nb, symmetry, orbital_symmetry, gas_min, gas_max),
    # ci.py:120-137): state irrep, orbital irreps per GAS space (None: one space of norb orbitals
    # in irrep 0) and the GAS electron bounds
    symmetry: int = 0
    orbital_symmetry: list = None
    gas_min: list = field(default_factory=list)
    gas_max: list = field(default_factory=list)
    # graph-captured Davidson iterations: None = automatic (small CSF spaces), True/False = force
    use_graph: bool = None
    # graph-captured iterations wait for a collective launch: run_steps yields GraphPhase and a
    # StepScheduler(one_launch=True) runs the iterations of many solves in one graph launch
    one_launch: bool = False
    # cap on the opposite-spin kernel's thread blocks (0 = none); see CISigmaBuilder.set_max_blocks
    sigma_max_blocks: int = 0
    # pick the fastest sigma kernel variants for this shape before solving (forte2_gb300.autotune)
    autotune: bool = False
    # kernel variants fixed for this solver ({name: value} of CISigmaBuilder.set_variant), applied
    # after the autotuner and over its choices
    sigma_variants: dict = None
    # after the solve, check every root's energy against its RDMs (ci.py:203-204, 323-403)
    do_test_rdms: bool = False

    def __post_init__(self):
        self._ready_event = None
        self.executed = False
        self.rebuild_guess = True
        self.eigensolver = None
        self.timings = {}

    @property
    def twice_ms(self):
        return self.na - self.nb

    def _startup(self):
        t0 = time.perf_counter()
        orbsym = self.orbital_symmetry if self.orbital_symmetry is not None else [[0] * self.norb]
        if sum(len(g) for g in orbsym) != self.norb:
            raise ValueError("orbital_symmetry must list the irreps of all norb active orbitals")
        self.ci_strings = CIStrings(self.na, self.nb, self.symmetry, orbsym, self.gas_min, self.gas_max)
        if self.ci_strings.ndet == 0:
            raise ValueError("No determinants could be generated for the given state and orbitals.")
        self.spin_adapter = CISpinAdapter(self.multiplicity - 1, self.twice_ms, self.norb)
        self.spin_adapter.prepare_couplings(self.ci_strings.make_determinants())
        self.ndet = self.ci_strings.ndet
        self.basis_size = self.spin_adapter.ncsf
        if self.basis_size == 0:
            raise ValueError("No CSFs with the requested multiplicity in this determinant space.")
        self.timings["startup"] = time.perf_counter() - t0

    def set_ints(self, E, H, V):
        """New integrals for the next run (ci.py:787-802); the eigensolver keeps its vectors."""
        self.E, self.H, self.V = E, H, V

    def reset_eigensolver(self):
        self.rebuild_guess = True
        self.eigensolver = None

    def new_problem(self, E, H, V):
        """Next solve of the same active space with other integrals, from fresh guesses. Keeps the
        strings, spin adapter, sigma builder, eigensolver buffers and captured graphs (no
        counterpart in the reference; a solver pool of the serving loop uses it)."""
        self.set_ints(E, H, V)
        self.rebuild_guess = True
        if self.eigensolver is not None:
            self.eigensolver.restart()

    def _make_sigma_closure(self):
        sa, sb = self.spin_adapter, self.sigma_builder

        def sigma_builder(B, S):
            # csf -> det -> H -> det -> csf in one native call (determinant scratch kept there)
            sb.apply_csf(sa, B, S)

        sigma_builder.device_rows = True
        sigma_builder.graph = (sb, sa, None)  # lets the eigensolver capture the same closure in a CUDA graph
        return sigma_builder

    def _build_guess(self, hdiag):
        torch = _torch()
        p = self.davidson_liu_params
        nguess = min(p.guess_per_root * self.nroot, self.basis_size)
        nguess_dets = min(p.ndets_per_guess * nguess, self.basis_size)
        if self.ci_params.energy_shift is not None:
            key = (hdiag - self.ci_params.energy_shift).abs()
        else:
            key = hdiag
        idx_dev = torch.sort(key, stable=True).indices[:nguess_dets].contiguous()
        if nguess_dets <= 64:
            # all on the device (no host wait): guess matrix, Jacobi, scatter into CSF rows
            from ._lib import check, lib, stream_handle

            m = nguess_dets
            Hg = torch.empty((m, m), dtype=torch.float64, device="cuda")
            check(lib().f2g_csf_matrix_dev(self.sigma_builder.h, self.spin_adapter.h, idx_dev.data_ptr(), m,
                                           Hg.data_ptr(), stream_handle()))
            ev = torch.empty(m, dtype=torch.float64, device="cuda")
            V = torch.empty((m, m), dtype=torch.float64, device="cuda")
            check(lib().f2g_dav_eigh(m, Hg.data_ptr(), ev.data_ptr(), V.data_ptr(), stream_handle()))
            rows = torch.zeros((nguess, self.basis_size), dtype=torch.float64, device="cuda")
            rows[:, idx_dev] = V[:, :nguess].T
            self.eigensolver.add_guess_rows(rows)
            return
        idx = idx_dev.cpu().numpy()
        Hg = self.sigma_builder.csf_matrix(self.spin_adapter, idx)
        _, vecs = np.linalg.eigh(Hg)
        guess = torch.zeros((self.basis_size, nguess), dtype=torch.float64, device="cuda")
        gi = torch.as_tensor(idx, device="cuda")
        guess[gi, :] = torch.as_tensor(vecs[:, :nguess], device="cuda")
        self.eigensolver.add_guesses(guess)

    def run(self):
        """Solve (ci.py:185-208); returns self with evals, evecs, converged."""
        out = drive(self.run_steps())
        _torch().cuda.synchronize()
        return out

    def run_steps(self):
        """Step generator of run() (see forte2_gb300.davidson.drive and forte2_gb300.batch)."""
        torch = _torch()
        t_all = time.perf_counter()
        ready = getattr(self, "_ready_event", None)
        if ready is not None:  # the previous solve of this object ran on another stream
            torch.cuda.current_stream().wait_event(ready)
            self._ready_event = None
        if not self.executed:
            self._startup()
        t0 = time.perf_counter()
        if getattr(self, "sigma_builder", None) is None:
            self.sigma_builder = CISigmaBuilder(self.ci_strings, self.E, self.H, self.V, self.log_level)
        else:
            # same strings: new integrals into the same builder, ordered on this stream (the first
            # host read below, in the guess, synchronises the stream before the builder is read)
            self.sigma_builder.update_integrals(self.E, self.H, self.V)
            self.sigma_builder.set_precision("fp64")
        self.sigma_builder.set_memory(self.ci_params.ci_builder_memory)
        self.sigma_builder.set_max_blocks(self.sigma_max_blocks)
        alg = self.ci_params.ci_algorithm.lower()
        if alg == "exact":
            return self._exact()
        self.sigma_builder.set_algorithm(alg)
        for name, value in (self.sigma_variants or {}).items():
            self.sigma_builder.set_variant(name, value)
        if self.autotune:
            from .autotune import autotune_sigma

            for prec in ("fp64", "fp32") if self.ci_params.precision == "mixed" else ("fp64",):
                autotune_sigma(self.sigma_builder, self.norb, self.na, self.nb, prec, fixed=self.sigma_variants)
        if self.sigma_variants:
            sb = self.sigma_builder
            if not hasattr(sb, "_tuned"):
                sb._tuned = {}
            for prec in ("fp64", "fp32"):
                sb._tuned.setdefault(prec, {}).update(self.sigma_variants)
            for name, value in self.sigma_variants.items():
                sb.set_variant(name, value)
        hdiag = self.sigma_builder.hdiag_csf_device(self.spin_adapter)
        self.timings["setup"] = time.perf_counter() - t0
        if self.ndet == 1:
            self.evals = np.array([float(hdiag[0])])
            self.evecs = torch.ones((1, 1), dtype=torch.float64, device="cuda")
            self.executed = True
            self.E_roots = self.evals
            return self
        if self.eigensolver is None:
            dl = self.davidson_liu_params
            if self.ci_params.precision == "mixed":
                from dataclasses import replace

                bpr = max(dl.basis_per_root, min(self.mixed_basis_per_root, 64 // self.nroot))
                cpr = max(dl.collapse_per_root, min(self.mixed_collapse_per_root, bpr - 1))
                dl = replace(dl, basis_per_root=bpr, collapse_per_root=cpr)
            self.eigensolver = DavidsonLiuSolver(size=self.basis_size, nroot=self.nroot,
                                                 davidson_liu_params=dl,
                                                 energy_shift=self.ci_params.energy_shift,
                                                 log_level=self.log_level, seed=self.seed,
                                                 use_graph=self.use_graph)
        self.eigensolver.collective = self.one_launch
        self.eigensolver.add_h_diag(hdiag)
        if self.rebuild_guess:
            self._build_guess(hdiag)
            self.rebuild_guess = False
        self.eigensolver.add_sigma_builder(self._make_sigma_closure())
        t0 = time.perf_counter()
        self.phases = []
        if self.ci_params.precision == "mixed":
            self.evals, evecs, self.converged = yield from self._solve_mixed_steps()
        else:
            self.evals, evecs = yield from self.eigensolver.solve_steps()
            self.converged = self.eigensolver.converged
            self.phases.append(("fp64", self.eigensolver.iter + 1, self.eigensolver.sigma_builds, list(self.evals)))
        self.timings["davidson"] = time.perf_counter() - t0
        self.evecs = evecs
        if not self.converged and self.die_if_not_converged:
            raise RuntimeError("Davidson-Liu solver did not converge.")
        self.E_roots = self.evals
        self.executed = True
        self.timings["total"] = time.perf_counter() - t_all
        if self.do_test_rdms:
            self._test_rdms()
        return self

    def _exact(self):
        H = self.sigma_builder.form_H_csf(None, self.spin_adapter, self.ci_params.ci_builder_memory)
        w, v = np.linalg.eigh(H)
        if self.ci_params.energy_shift is not None:
            o = np.argsort(np.abs(w - self.ci_params.energy_shift))
            w, v = w[o], v[:, o]
        self.evals = w[: self.nroot]
        self.evecs = v[:, : self.nroot]
        self.E_roots = self.evals
        self.converged = True
        self.executed = True
        return self

    def _solve_mixed_steps(self):
        """FP32 Davidson, then FP64 defect correction of the Ritz vectors.

        Phase 1 runs the Davidson iterations with FP32 sigma builds. Then, for the current Ritz
        vectors X (rows), each outer step builds S64 = H X in FP64 and S32 = H X in FP32 (nroot
        builds each), performs an FP64 Rayleigh-Ritz in span(X) and checks the FP64 residual. If
        not converged it continues the Davidson iterations, with FP32 sigma builds, on the
        corrected operator H' = H32 + D X^T + X D^T - X (X^T D) X^T with D = S64 - S32, which
        acts exactly as FP64 H on span(X) (its sigma for X is S64 itself) and as FP32 H elsewhere.
        The error of X then shrinks by about |H64 - H32| / gap per outer step, so a solve needs a
        few FP64 builds per root instead of FP64 Davidson iterations. When an outer step no
        longer halves the FP64 residual (the FP32 sigma noise floor, about 1e-6 for |H| ~ 20) or
        the outer steps run out, FP64 Davidson iterations warm-started from X finish the solve
        under the caller's tolerances. Returns (evals, evecs (size, nroot), converged) with the
        energies from the final FP64 Rayleigh-Ritz step.
        """
        torch = _torch()
        es, sb = self.eigensolver, self.sigma_builder
        e_tol, r_tol = es.e_tol, es.r_tol
        k = self.nroot
        plain = es._build_sigma
        sb.set_precision("fp32")
        es.e_tol, es.r_tol = max(e_tol, self.mixed_e_tol), max(r_tol, self.mixed_r_tol)
        es.stall_window, es.stall_floor = 25, 1e-3
        ev, _ = yield from es.solve_steps()
        self.phases.append(("fp32", es.iter + 1, es.sigma_builds, [float(x) for x in ev]))
        # persistent buffers: a captured graph of the corrected phase keeps their addresses
        if getattr(self, "_mixed_bufs", None) is None or self._mixed_bufs[0].shape != (k, es.size):
            shape = (k, es.size)
            self._mixed_bufs = tuple(torch.zeros(shape, dtype=torch.float64, device="cuda") for _ in range(4)) + (
                torch.zeros((k, k), dtype=torch.float64, device="cuda"),)
        X, S64, S32, D, Mb = self._mixed_bufs
        X.copy_(es.b[:k])
        lam_prev = None
        rn_prev = None
        converged = False
        w = np.asarray(ev, dtype=np.float64)
        for outer in range(self.mixed_max_outer):
            sb.set_precision("fp64")
            plain(X, S64)
            sb.set_precision("fp32")
            plain(X, S32)
            # FP64 Rayleigh-Ritz in span(X)
            (G,) = yield [es._dots_dev(X, S64)]
            w, U = np.linalg.eigh(0.5 * (G + G.T))
            if self.ci_params.energy_shift is not None:
                o = np.argsort(np.abs(w - self.ci_params.energy_shift))
                w, U = w[o], U[:, o]
            for M in (X, S64, S32):
                tmp = torch.empty_like(M)
                es._lincomb(M, U, tmp, 0.0)
                M.copy_(tmp)
            R = S64.clone()
            es._lincomb(X, -np.diag(w), R, 1.0)
            (RR,) = yield [es._dots_dev(R, R)]
            rn = np.sqrt(np.maximum(np.diag(RR), 0.0))
            de = np.inf if lam_prev is None else float(np.max(np.abs(w - lam_prev)))
            self.phases.append(("fp64-check", outer, 2 * k, [float(x) for x in w], float(rn.max()), de))
            if rn.max() < r_tol and de < e_tol:
                converged = True
                break
            if (rn_prev is not None and rn.max() > 0.5 * rn_prev) or outer == self.mixed_max_outer - 1:
                # the corrected FP32 iterations no longer reduce the FP64 residual (their sigma
                # noise floor): finish with FP64 Davidson iterations from X, whose FP64 sigma S64
                # is already known, under the caller's tolerances
                w, converged = yield from self._fp64_polish_steps(X, S64, w, plain, e_tol, r_tol)
                break
            rn_prev = float(rn.max())
            lam_prev = w.copy()
            torch.sub(S64, S32, out=D)
            Mxd = es._dots_dev(X, D)
            Mb.copy_(0.5 * (Mxd + Mxd.T))

            def corrected(B, S, X=X, D=D, Mxd=Mb):
                # enqueue only: H' B = H32 B + D (X B) + X (D B) - X Mxd (X B)
                plain(B, S)
                A = es._dots_dev(X, B)  # (k, m): <x_i, b_l>
                Bd = es._dots_dev(D, B)  # (k, m): <d_i, b_l>
                es._lincomb(D, A, S, 1.0)
                # Bd - Mxd A as a broadcast product and sum (tiny; keeps cuBLAS off per-job streams)
                es._lincomb(X, Bd - (Mxd[:, :, None] * A[None, :, :]).sum(1), S, 1.0)

            corrected.device_rows = True
            corrected.graph = (sb, self.spin_adapter, (X, D, Mb, k))
            es.add_sigma_builder(corrected)
            # warm start from X with its exact corrected sigma (S64): no FP32 rebuild of X
            es.b[:k].copy_(X)
            es.sigma[:k].copy_(S64)
            es.basis_size = es.sigma_size = k
            es.lam_old[:k] = w
            es.e_tol, es.r_tol = e_tol, 0.3 * r_tol
            es.stall_window, es.stall_floor = 40, 1e-5
            b0 = es.sigma_builds
            ev, _ = yield from es.solve_steps()
            self.phases.append(("fp32-corrected", es.iter + 1, es.sigma_builds - b0, [float(x) for x in ev]))
            X.copy_(es.b[:k])
        es.add_sigma_builder(plain)
        es.e_tol, es.r_tol = e_tol, r_tol
        es.stall_window, es.stall_floor = 0, 0.0
        sb.set_precision("fp64")
        es.b[:k].copy_(X)
        es.basis_size, es.sigma_size = k, 0
        es.converged = converged
        return w[:k], es.b[:k].T, converged

    def _fp64_polish_steps(self, X, S64, w, plain, e_tol, r_tol):
        """FP64 Davidson iterations warm-started from the rows X with their FP64 sigma S64; X is
        overwritten with the converged Ritz vectors. Returns (energies, converged)."""
        es, sb = self.eigensolver, self.sigma_builder
        k = self.nroot
        sb.set_precision("fp64")
        es.add_sigma_builder(plain)
        es.b[:k].copy_(X)
        es.sigma[:k].copy_(S64)
        es.basis_size = es.sigma_size = k
        es.lam_old[:k] = w[:k]
        es.e_tol, es.r_tol = e_tol, r_tol
        es.stall_window, es.stall_floor = 0, 0.0
        b0 = es.sigma_builds
        ev, _ = yield from es.solve_steps()
        self.phases.append(("fp64-polish", es.iter + 1, es.sigma_builds - b0, [float(x) for x in ev]))
        X.copy_(es.b[:k])
        return np.asarray(ev, dtype=np.float64), es.converged

    def avg_build_time(self):
        return self.sigma_builder.avg_build_time()

    # ---- reduced density matrices of the solved roots (ci.py:476-768) ----------------------------

    def _csf_to_det_device(self, csf_vec):
        torch = _torch()
        v = csf_vec
        if isinstance(v, np.ndarray):
            v = torch.from_numpy(np.ascontiguousarray(v))
        v = v.to(device="cuda", dtype=torch.float64).contiguous()
        det = torch.empty(self.ndet, dtype=torch.float64, device="cuda")
        self.spin_adapter.csf_C_to_det_C(v, det)
        return det

    def _det_vector(self, root):
        """Determinant-basis vector of a root, on the device."""
        return self._csf_to_det_device(self.evecs[:, root])

    def csf_C_to_det_C(self, csf_vec):
        """A CSF-basis vector in the determinant basis, as a numpy array (ci.py:454-470)."""
        return self._csf_to_det_device(csf_vec).cpu().numpy()

    def _root_vector_det(self, root: int):
        """CI vector of a root in the determinant basis (ci.py:472-474)."""
        return self.csf_C_to_det_C(self.evecs[:, root])

    def compute_natural_occupation_numbers(self):
        """Natural occupation numbers (norb, nroot), each column descending (ci.py:770-785)."""
        if not self.executed:
            raise RuntimeError("CI solver has not been executed yet.")
        no = np.zeros((self.norb, self.nroot))
        for i in range(self.nroot):
            no[:, i] = np.linalg.eigvalsh(self.make_1rdm(i))[::-1]
        return no

    def get_top_determinants(self, n=5):
        """Per root, the n determinants with the largest |coefficient| as ((alpha mask, beta mask),
        coefficient) pairs (ci.py:804-832)."""
        if not self.executed:
            raise RuntimeError("CI solver has not been executed yet.")
        dets = self.ci_strings.make_determinants()
        return [top_determinants(self._root_vector_det(i), dets, n) for i in range(self.nroot)]

    def _rdm_vectors(self, left_root, right_root):
        L = self._det_vector(left_root)
        R = L if right_root is None else self._det_vector(right_root)
        return L, R

    def _rdm(self, kinds, left_root, right_root):
        L, R = self._rdm_vectors(left_root, right_root)
        out = [getattr(self.sigma_builder, k)(L, R).cpu().numpy() for k in kinds]
        return out[0] if len(out) == 1 else tuple(out)

    def make_sd_1rdm(self, left_root: int, right_root: int | None = None):
        """Spin-dependent 1-RDMs (a, b) between two roots (ci.py:576-599)."""
        return self._rdm(("a_1rdm", "b_1rdm"), left_root, right_root)

    def make_sd_2rdm(self, left_root: int, right_root: int | None = None):
        """Spin-dependent 2-RDMs (aa packed, ab, bb packed) between two roots (ci.py:601-625)."""
        return self._rdm(("aa_2rdm", "ab_2rdm", "bb_2rdm"), left_root, right_root)

    def make_sf_1rdm(self, left_root: int, right_root: int | None = None):
        return self._rdm(("sf_1rdm",), left_root, right_root)

    def make_sf_2rdm(self, left_root: int, right_root: int | None = None):
        return self._rdm(("sf_2rdm",), left_root, right_root)

    def make_sf_2cumulant(self, left_root: int, right_root: int | None = None):
        return self._rdm(("sf_2cumulant",), left_root, right_root)

    def make_sd_3rdm(self, left_root: int, right_root: int | None = None):
        """Spin-dependent 3-RDMs (aaa, aab, abb, bbb) between two roots (ci.py:627-653)."""
        return self._rdm(("aaa_3rdm", "aab_3rdm", "abb_3rdm", "bbb_3rdm"), left_root, right_root)

    def make_sf_3rdm(self, left_root: int, right_root: int | None = None):
        return self._rdm(("sf_3rdm",), left_root, right_root)

    def make_sf_3cumulant(self, left_root: int, right_root: int | None = None):
        return self._rdm(("sf_3cumulant",), left_root, right_root)

    make_1rdm = make_sf_1rdm
    make_2rdm = make_sf_2rdm
    make_2cumulant = make_sf_2cumulant
    make_3rdm = make_sf_3rdm
    make_3cumulant = make_sf_3cumulant

    def rdm_energies(self, root):
        """The root's energy from its RDMs in the three forms the reference checks (ci.py:323-403):
        packed same-spin, expanded same-spin, spin-free."""
        n = self.norb
        g1 = self.make_sf_1rdm(root)
        aa, ab, bb = self.make_sd_2rdm(root)
        g2 = self.make_sf_2rdm(root)
        H, V = np.asarray(self.H), np.asarray(self.V)
        A = V - np.einsum("ijkl->ijlk", V)
        i, j = np.tril_indices(n, k=-1)
        M = A[i[:, None], j[:, None], i[None, :], j[None, :]]
        e1 = float(np.einsum("ij,ij", g1, H))
        packed = self.E + e1 + np.einsum("ij,ij", aa, M) + np.einsum("ijkl,ijkl", ab, V) + np.einsum("ij,ij", bb, M)
        expanded = (self.E + e1 + 0.25 * np.einsum("ijkl,ijkl", packed_tensor4_to_tensor4(aa, n), A)
                    + np.einsum("ijkl,ijkl", ab, V) + 0.25 * np.einsum("ijkl,ijkl", packed_tensor4_to_tensor4(bb, n), A))
        spin_free = self.E + e1 + 0.5 * np.einsum("ijkl,ijkl", g2, V)
        return float(packed), float(expanded), float(spin_free)

    def _test_rdms(self):
        for root in range(self.nroot):
            for form, e in zip(("RDMs", "expanded RDMs", "spin-free RDMs"), self.rdm_energies(root)):
                if not np.isclose(self.evals[root], e, rtol=1e-6, atol=1e-8):
                    raise AssertionError(f"CI energy {self.evals[root]} Eh does not match {form} energy {e} Eh")


def top_determinants(det_vec, dets, n):
    """The n entries of a determinant vector with the largest |coefficient|, descending, as
    (determinant, coefficient) pairs (the selection of ci.py:823-830)."""
    order = np.argsort(np.abs(det_vec))[::-1]
    return [(dets[int(j)], float(det_vec[j])) for j in order[: min(n, len(order))]]


def packed_tensor4_to_tensor4(packed, n):
    """Expand a packed same-spin 2-RDM [pq][rs] (p > q, r > s) to the antisymmetric (n, n, n, n)
    tensor (the reference's cpp_helpers.packed_tensor4_to_tensor4, used at ci.py:337-341)."""
    out = np.zeros((n, n, n, n))
    if n < 2:
        return out
    i, j = np.tril_indices(n, k=-1)
    P = np.asarray(packed).reshape(len(i), len(i))
    ii, jj = i[:, None], j[:, None]
    kk, ll = i[None, :], j[None, :]
    out[ii, jj, kk, ll] = P
    out[jj, ii, kk, ll] = -P
    out[ii, jj, ll, kk] = -P
    out[jj, ii, ll, kk] = P
    return out
