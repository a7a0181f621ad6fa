"""Test infrastructure (oracle only): load the reference's own ``helpers/davidsonliu.py`` from a
reference checkout, with its three forte2 imports (logger, table, params;
davidsonliu.py:1-9) replaced by small stubs, so that golden CASCI energies come from the
reference's Davidson driving the reference's compiled sigma builder.

Used only by ``tests/golden/make_golden.py`` in a container that has the reference checkout.
"""

from __future__ import annotations

import importlib.util
import sys
import types
from dataclasses import dataclass


@dataclass
class DavidsonLiuParams:
    """Defaults of the reference's DavidsonLiuParams (base_classes/params.py:106-146)."""

    guess_per_root: int = 2
    ndets_per_guess: int = 10
    collapse_per_root: int = 2
    basis_per_root: int = 4
    maxiter: int = 100
    e_tol: float = 1e-12
    r_tol: float = 1e-6


class _Table:
    def __init__(self, *a, **k):
        pass

    def header(self):
        return ""

    def row(self, *a):
        return ""

    def footer(self):
        return ""


def load(reference_root: str):
    logger = types.ModuleType("forte2.helpers.logger")
    logger.log = lambda *a, **k: None
    logger.log_warning = lambda *a, **k: None
    logger.get_verbosity_level = lambda: 0
    table = types.ModuleType("forte2.helpers.table")
    table.AsciiTable = _Table
    params = types.ModuleType("forte2.base_classes.params")
    params.DavidsonLiuParams = DavidsonLiuParams
    pkg = types.ModuleType("forte2")
    helpers = types.ModuleType("forte2.helpers")
    helpers.logger = logger
    base = types.ModuleType("forte2.base_classes")
    saved = {k: sys.modules.get(k) for k in
             ("forte2", "forte2.helpers", "forte2.helpers.logger", "forte2.helpers.table",
              "forte2.base_classes", "forte2.base_classes.params")}
    sys.modules.update({"forte2": pkg, "forte2.helpers": helpers, "forte2.helpers.logger": logger,
                        "forte2.helpers.table": table, "forte2.base_classes": base,
                        "forte2.base_classes.params": params})
    try:
        spec = importlib.util.spec_from_file_location(
            "ref_davidsonliu", f"{reference_root}/forte2/helpers/davidsonliu.py")
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
    finally:
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v
    return mod.DavidsonLiuSolver, DavidsonLiuParams
