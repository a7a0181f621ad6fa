"""Parameter dataclasses with the reference's defaults and validation
(forte2/base_classes/params.py:106-178)."""

from __future__ import annotations

from dataclasses import dataclass

_ALGORITHMS = ("hz", "harrison-zarrabian", "kh", "knowles-handy", "exact")


@dataclass
class DavidsonLiuParams:
    guess_per_root: int = 2
    ndets_per_guess: int = 10
    collapse_per_root: int = 2
    basis_per_root: int = 4
    maxiter: int = 100
    e_tol: float = 1e-12
    r_tol: float = 1e-6

    def __post_init__(self):
        if self.collapse_per_root < 1:
            raise ValueError(
                f"Davidson-Liu solver: collapse_per_root ({self.collapse_per_root}) must be greater than or equal to 1.")
        if self.basis_per_root < self.collapse_per_root + 1:
            raise ValueError(
                f"Davidson-Liu solver: basis_per_root ({self.basis_per_root}) must be greater than or equal to "
                f"collapse_per_root + 1 ({self.collapse_per_root + 1}).")


@dataclass
class CIParams:
    ci_algorithm: str = "hz"
    ci_builder_memory: int = 1024
    energy_shift: float = None
    # GB300 extension: "fp64" (the reference's arithmetic) or "mixed" (FP32 sigma during the
    # Davidson iterations, FP64 refinement at the end).
    precision: str = "fp64"

    def __post_init__(self):
        if self.ci_algorithm.lower() not in _ALGORITHMS:
            raise ValueError(f"ci_algorithm must be one of {_ALGORITHMS}, got '{self.ci_algorithm}'")
        if self.precision not in ("fp64", "mixed"):
            raise ValueError(f"precision must be 'fp64' or 'mixed', got '{self.precision}'")
