"""CASCI driver with the reference's per-state solver semantics (forte2/ci/ci.py:30-836,
_CISingleStateSolver), device-resident end to end.

``CASCISolver.run()`` does what ``_CISingleStateSolver.run()`` does (ci.py:185-303): build the
strings and the CSF spin adapter, build the sigma builder with the current integrals, form the
CSF diagonal, build guess vectors from the lowest diagonal CSFs (ci.py:411-452), and run the
Davidson-Liu solver with the closure csf -> det -> H -> det -> csf (ci.py:221-235). Here every
vector stays on the GPU and each Davidson block is transformed and sigma-built in one call.

``precision="mixed"`` runs the Davidson iterations with FP32 sigma builds and then continues
from the converged FP32 vectors with FP64 sigma builds until the requested tolerances are met
(the final FP64 refinement); orthogonalisation, residual norms and the subspace eigensolve are
FP64 throughout.
"""

from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from .ci_helpers import CISigmaBuilder, CISpinAdapter, CIStrings
from .davidson import DavidsonLiuSolver
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
    seed: int = 12345

    def __post_init__(self):
        self.executed = False
        self.rebuild_guess = True
        self.eigensolver = None
        self.timings = {}

    @property
    def twice_ms(self):
        return self.na - self.nb

    def _startup(self):
        t0 = time.perf_counter()
        self.ci_strings = CIStrings(self.na, self.nb, 0, [[0] * self.norb], [], [])
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

    def _make_sigma_closure(self):
        torch = _torch()
        sa, sb = self.spin_adapter, self.sigma_builder
        ndet = self.ndet
        bufs = {}

        def sigma_builder(B, S):
            m = B.shape[0]
            if bufs.get("m", 0) < m:
                bufs["det"] = torch.empty((m, ndet), dtype=torch.float64, device="cuda")
                bufs["sdet"] = torch.empty((m, ndet), dtype=torch.float64, device="cuda")
                bufs["m"] = m
            det, sdet = bufs["det"][:m], bufs["sdet"][:m]
            sa.csf_C_to_det_C(B, det)
            sb.Hamiltonian(det, sdet)
            sa.det_C_to_csf_C(sdet, S)

        sigma_builder.device_rows = True
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
        idx = torch.sort(key, stable=True).indices[:nguess_dets].cpu().numpy()
        Hg = self.sigma_builder.csf_matrix(self.spin_adapter, idx)
        _, vecs = np.linalg.eigh(Hg)
        guess = torch.zeros((self.basis_size, nguess), dtype=torch.float64, device="cuda")
        gi = torch.as_tensor(idx, device="cuda")
        guess[gi, :] = torch.as_tensor(vecs[:, :nguess], device="cuda")
        self.eigensolver.add_guesses(guess)

    def run(self):
        torch = _torch()
        t_all = time.perf_counter()
        if not self.executed:
            self._startup()
        t0 = time.perf_counter()
        self.sigma_builder = CISigmaBuilder(self.ci_strings, self.E, self.H, self.V, self.log_level)
        self.sigma_builder.set_memory(self.ci_params.ci_builder_memory)
        alg = self.ci_params.ci_algorithm.lower()
        if alg == "exact":
            return self._exact()
        self.sigma_builder.set_algorithm(alg)
        hdiag = self.sigma_builder.hdiag_csf_device(self.spin_adapter)
        self.timings["setup"] = time.perf_counter() - t0
        if self.ndet == 1:
            self.evals = np.array([float(hdiag[0])])
            self.evecs = torch.ones((1, 1), dtype=torch.float64, device="cuda")
            self.executed = True
            self.E_roots = self.evals
            return self
        if self.eigensolver is None:
            self.eigensolver = DavidsonLiuSolver(size=self.basis_size, nroot=self.nroot,
                                                 davidson_liu_params=self.davidson_liu_params,
                                                 energy_shift=self.ci_params.energy_shift,
                                                 log_level=self.log_level, seed=self.seed)
        self.eigensolver.add_h_diag(hdiag)
        if self.rebuild_guess:
            self._build_guess(hdiag)
            self.rebuild_guess = False
        self.eigensolver.add_sigma_builder(self._make_sigma_closure())
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        self.phases = []
        if self.ci_params.precision == "mixed":
            es = self.eigensolver
            e_tol, r_tol = es.e_tol, es.r_tol
            self.sigma_builder.set_precision("fp32")
            es.e_tol, es.r_tol = max(e_tol, self.mixed_e_tol), max(r_tol, self.mixed_r_tol)
            ev32, _ = es.solve()
            self.phases.append(("fp32", es.iter + 1, es.sigma_builds, list(ev32)))
            self.sigma_builder.set_precision("fp64")
            es.e_tol, es.r_tol = e_tol, r_tol
            b0 = es.sigma_builds
            self.evals, evecs = es.solve()
            self.phases.append(("fp64", es.iter + 1, es.sigma_builds - b0, list(self.evals)))
        else:
            self.evals, evecs = self.eigensolver.solve()
            self.phases.append(("fp64", self.eigensolver.iter + 1, self.eigensolver.sigma_builds, list(self.evals)))
        torch.cuda.synchronize()
        self.timings["davidson"] = time.perf_counter() - t0
        self.evecs = evecs
        self.converged = self.eigensolver.converged
        if not self.converged and self.die_if_not_converged:
            raise RuntimeError("Davidson-Liu solver did not converge.")
        self.E_roots = self.evals
        self.executed = True
        self.timings["total"] = time.perf_counter() - t_all
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

    def avg_build_time(self):
        return self.sigma_builder.avg_build_time()
