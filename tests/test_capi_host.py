"""CPU checks of the boundary: the CUDA library builds for sm_103a, loads, and exports every symbol
include/forte2_gb300.h declares; host-side validation mirrors the reference (no GPU calls)."""

import ctypes
import os
import re
import shutil

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    hdr = open(os.path.join(ROOT, "include", "forte2_gb300.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    return sorted(set(re.findall(r"\b(f2g_[a-z0-9_]+)\s*\(", hdr)))


@pytest.fixture(scope="module")
def libpath():
    from forte2_gb300.build import LIB_PATH, build

    if not os.path.exists(LIB_PATH):
        if not shutil.which("nvcc") and not os.path.exists("/usr/local/cuda/bin/nvcc"):
            pytest.skip("nvcc not available")
        build()
    return LIB_PATH


def test_library_exports_every_declared_symbol(libpath):
    lib = ctypes.CDLL(libpath)
    syms = declared_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_version_and_error_calls_need_no_gpu(libpath):
    from forte2_gb300._lib import lib

    assert b"sm_103a" in lib().f2g_version()
    # invalid arguments are rejected on the host before any CUDA call
    out = ctypes.c_void_p()
    assert lib().f2g_strings_create(-1, 0, 3, ctypes.byref(out)) == 2
    assert b"non-negative" in lib().f2g_last_error()


def test_cistrings_input_validation():
    """tests/ci/test_ci_strings.py:6-19 of the reference: negative counts -> ValueError, a flat
    orbital-symmetry list -> TypeError. Both are raised before any device work."""
    from forte2_gb300.ci_helpers import CIStrings

    with pytest.raises(ValueError):
        CIStrings(-1, 0, 0, [[]], [], [])
    with pytest.raises(ValueError):
        CIStrings(-1, -1, 0, [[]], [], [])
    with pytest.raises(ValueError):
        CIStrings(1, -1, 0, [[]], [], [])
    with pytest.raises(TypeError):
        CIStrings(1, 1, 0, [0], [], [])
    with pytest.raises(ValueError):
        CIStrings(1, 1, 0, [[0, 0]], [0, 0], [])


def test_params_validation():
    from forte2_gb300.params import CIParams, DavidsonLiuParams

    with pytest.raises(ValueError):
        DavidsonLiuParams(collapse_per_root=0)
    with pytest.raises(ValueError):
        DavidsonLiuParams(collapse_per_root=3, basis_per_root=3)
    with pytest.raises(ValueError):
        CIParams(ci_algorithm="sparse-not-here")
    assert CIParams().ci_algorithm == "hz" and CIParams().ci_builder_memory == 1024
    p = DavidsonLiuParams()
    assert (p.guess_per_root, p.ndets_per_guess, p.collapse_per_root, p.basis_per_root, p.maxiter,
            p.e_tol, p.r_tol) == (2, 10, 2, 4, 100, 1e-12, 1e-6)


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    import forte2_gb300._lib as L

    monkeypatch.setattr(L, "_lib", None)
    monkeypatch.setattr(L, "LIB_PATH", str(tmp_path / "nope.so"))
    with pytest.raises(L.CudaLibraryMissing):
        L.lib()


def test_new_entry_points_validate_handles_without_gpu(libpath):
    """The graph, CSF-sigma, variant and Gram-Schmidt entry points reject NULL handles and bad
    sizes with status 2 before any device work."""
    import numpy as np

    from forte2_gb300._lib import lib

    L = lib()
    out = ctypes.c_void_p()
    thr = np.array([1e-8, 1e-8, 1e-12])
    assert L.f2g_dgraph_create(None, None, 10, 1, 4, 2, 10, 1, 8, thr.ctypes.data, None, None, None, None, 10, 10,
                               10, None, ctypes.byref(out)) == 2
    assert b"NULL" in L.f2g_last_error()
    assert L.f2g_dgraph_reset(None, 1, 1, None, None, 0, None, 0, 1e-10, 1e-6, 10, 0, 0.0, None) == 2
    assert L.f2g_dgraph_launch(None, None) == 2
    assert L.f2g_sigma_apply_csf(None, None, None, None, 1, None) == 2
    assert L.f2g_sigma_set_variant(None, 0, 1) == 2
    assert L.f2g_sigma_set_max_blocks(None, 4) == 2
    assert L.f2g_sigma_set_tensor_cores(None, 1, None) == 2
    assert L.f2g_dav_gs_append(None, 10, 4, 0, None, 10, 1, 10, 1e-8, 1e-12, 1, 1, None, None) == 2
    # one-launch batches of graph solves: NULL handles and empty batches are refused on the host
    arr = (ctypes.c_void_p * 2)(None, None)
    assert L.f2g_dgraph_batch_create(None, 2, ctypes.byref(out)) == 2
    assert L.f2g_dgraph_batch_create(ctypes.addressof(arr), 0, ctypes.byref(out)) == 2
    assert b"at least one" in L.f2g_last_error()
    assert L.f2g_dgraph_batch_create(ctypes.addressof(arr), 2, ctypes.byref(out)) == 2
    assert b"NULL graph" in L.f2g_last_error()
    assert L.f2g_dgraph_batch_launch(None, None) == 2
    assert L.f2g_dgraph_batch_nodes(None, None) == 2
    serial = ctypes.c_uint64()
    assert L.f2g_dgraph_serial(None, ctypes.addressof(serial)) == 2
    # two-component builder and its RDMs
    assert L.f2g_rel_sigma_rdm(None, 0, None, None, None, None) == 2
    assert L.f2g_rel_sigma_apply(None, None, None, 1, None) == 2


def test_davidson_and_sigma_entry_points_validate_sizes_without_gpu(libpath):
    """Negative sizes and NULL buffers of the Davidson vector operations and of the sigma, CSF and
    RDM entry points give status 2 (ValueError) before any device work."""
    from forte2_gb300._lib import lib

    L = lib()
    assert L.f2g_dav_dots(None, -1, 8, None, 2, 8, 8, None, None, None) == 2
    assert L.f2g_dav_dots(None, 2, 8, None, 2, 8, 8, None, None, None) == 2  # NULL operands
    # the allocation-free variant validates the same way, before it touches the device
    assert L.f2g_dav_dots_noalloc(None, -1, 8, None, 2, 8, 8, None, None) == 2
    assert L.f2g_dav_dots_noalloc(None, 2, 8, None, 2, 8, 8, None, None) == 2
    assert b"A is NULL" in L.f2g_last_error()
    assert L.f2g_dav_lincomb(None, 2, 8, None, -3, None, 8, 0.0, 8, None) == 2
    assert L.f2g_dav_lincomb(None, 2, 8, None, 2, None, 8, 0.0, 8, None) == 2
    assert L.f2g_dav_residual(None, None, 2, 8, None, None, -1, None, 8, 1e-8, None, 8, None, None, None) == 2
    assert L.f2g_dav_residual(None, None, 2, 8, None, None, 1, None, 8, 1e-8, None, 8, None, None, None) == 2
    assert L.f2g_dav_eigh(-1, None, None, None, None) == 2
    assert L.f2g_dav_eigh(3, None, None, None, None) == 2
    for f in ("f2g_sigma_apply", "f2g_sigma_term", "f2g_sigma_det_energies", "f2g_sigma_avg_build_time"):
        assert getattr(L, f) is not None
    assert L.f2g_sigma_apply(None, None, None, 1, None) == 2
    assert L.f2g_sigma_apply_host(None, None, None, 1) == 2
    assert L.f2g_sigma_avg_build_time(None, None) == 2
    assert L.f2g_csf_to_det(None, None, None, 1, None) == 2
    assert L.f2g_det_to_csf(None, None, None, 1, None) == 2
    assert L.f2g_sigma_rdm(None, 0, None, None, None, None) == 2
