"""ctypes binding of the in-tree CUDA library (include/forte2_gb300.h).

The library must exist: there is no CPU fallback. If it has not been built, importing any
compute class raises with instructions (``python -c "import __graft_entry__ as g; g.build()"``).
"""

from __future__ import annotations

import ctypes as C
import os

from .build import LIB_PATH

_lib = None


class CudaLibraryMissing(ImportError):
    pass


def _declare(L):
    vp, i64, i32, d = C.c_void_p, C.c_int64, C.c_int, C.c_double
    pp = C.POINTER(C.c_void_p)
    P = C.c_void_p  # raw pointers (device or host) are passed as integers
    sig = {
        "f2g_last_error": (C.c_char_p, []),
        "f2g_version": (C.c_char_p, []),
        "f2g_strings_create": (i32, [i32, i32, i32, pp]),
        "f2g_strings_create_general": (i32, [i32, i32, i32, i32, P, P, i32, P, i32, P, pp]),
        "f2g_strings_blocks_info": (i32, [vp, P]),
        "f2g_rel_sigma_create": (i32, [vp, d, P, P, pp]),
        "f2g_rel_sigma_destroy": (i32, [vp]),
        "f2g_rel_sigma_set_algorithm": (i32, [vp, C.c_char_p]),
        "f2g_rel_sigma_get_algorithm": (i32, [vp, C.c_char_p, i32]),
        "f2g_rel_sigma_set_memory": (i32, [vp, i32]),
        "f2g_rel_sigma_apply": (i32, [vp, P, P, i32, vp]),
        "f2g_rel_sigma_hdiag": (i32, [vp, P, vp]),
        "f2g_rel_sigma_element": (i32, [vp, i64, i64, P]),
        "f2g_rel_rdm_size": (i64, [i32, i32]),
        "f2g_rel_sigma_rdm": (i32, [vp, i32, P, P, P, vp]),
        "f2g_blocks_enumerate": (i32, [i32, i32, i32, i32, P, P, i32, P, i32, P, P, P, P, P, P, P]),
        "f2g_strings_class_strings": (i32, [vp, i32, P, P]),
        "f2g_strings_block_table": (i32, [vp, P]),
        "f2g_strings_occupations": (i32, [vp, P, P, P]),
        "f2g_strings_destroy": (i32, [vp]),
        "f2g_strings_info": (i32, [vp, P]),
        "f2g_strings_masks": (i32, [vp, i32, P]),
        "f2g_strings_list1h": (i32, [vp, i32, P, C.POINTER(C.c_int64)]),
        "f2g_strings_list2h": (i32, [vp, i32, P, C.POINTER(C.c_int64)]),
        "f2g_sigma_create": (i32, [vp, d, P, P, i32, pp]),
        "f2g_sigma_destroy": (i32, [vp]),
        "f2g_sigma_set_hamiltonian": (i32, [vp, d, P, P]),
        "f2g_sigma_set_algorithm": (i32, [vp, C.c_char_p]),
        "f2g_sigma_get_algorithm": (i32, [vp, C.c_char_p, i32]),
        "f2g_sigma_set_memory": (i32, [vp, i32]),
        "f2g_sigma_set_precision": (i32, [vp, i32]),
        "f2g_sigma_set_max_blocks": (i32, [vp, i32]),
        "f2g_sigma_set_tensor_cores": (i32, [vp, i32, P]),
        "f2g_sigma_set_variant": (i32, [vp, i32, i32]),
        "f2g_sigma_reset_build_times": (i32, [vp]),
        "f2g_sigma_tc_error": (i32, [vp, P]),
        "f2g_sigma_apply": (i32, [vp, P, P, i32, vp]),
        "f2g_sigma_apply_host": (i32, [vp, P, P, i32]),
        "f2g_sigma_term": (i32, [vp, i32, P, P, vp]),
        "f2g_sigma_avg_build_time": (i32, [vp, P]),
        "f2g_sigma_det_energies": (i32, [vp, P, vp]),
        "f2g_rdm_size": (i64, [i32, i32]),
        "f2g_sigma_rdm": (i32, [vp, i32, P, P, P, vp]),
        "f2g_rdm_pair_list": (i32, [i32, i32, i32, P, P, P]),
        "f2g_spin_adapter_create": (i32, [vp, i32, i32, pp]),
        "f2g_spin_adapter_destroy": (i32, [vp]),
        "f2g_spin_adapter_info": (i32, [vp, P]),
        "f2g_csf_to_det": (i32, [vp, P, P, i32, vp]),
        "f2g_sigma_apply_csf": (i32, [vp, vp, P, P, i32, vp]),
        "f2g_det_to_csf": (i32, [vp, P, P, i32, vp]),
        "f2g_hdiag_csf": (i32, [vp, vp, P, vp]),
        "f2g_csf_matrix": (i32, [vp, vp, P, i32, P]),
        "f2g_csf_matrix_dev": (i32, [vp, vp, P, i32, P, vp]),
        "f2g_spin_adapter_dump": (i32, [vp, P, P, P, P]),
        "f2g_dav_scratch_size": (i64, [i64]),
        "f2g_dav_dots": (i32, [P, i32, i64, P, i32, i64, i64, P, P, vp]),
        "f2g_dav_dots_noalloc": (i32, [P, i32, i64, P, i32, i64, i64, P, vp]),
        "f2g_dav_lincomb": (i32, [P, i32, i64, P, i32, P, i64, d, i64, vp]),
        "f2g_dav_residual": (i32, [P, P, i32, i64, P, P, i32, P, i64, d, P, i64, P, P, vp]),
        "f2g_dav_eigh": (i32, [i32, P, P, P, vp]),
        "f2g_dav_gs_append": (i32, [P, i64, i32, i32, P, i64, i32, i64, d, d, i32, C.c_uint64, P, vp]),
        "f2g_dgraph_create": (i32, [vp, vp, i64, i32, i32, i32, i32, C.c_uint64, i32, P, P, P, P, P, i64, i64, i64,
                                    P, pp]),
        "f2g_dgraph_destroy": (i32, [vp]),
        "f2g_dgraph_set_correction": (i32, [vp, P, P, i64, P, i32]),
        "f2g_dgraph_reset": (i32, [vp, i32, i32, P, P, i32, P, i32, d, d, i32, i32, d, vp]),
        "f2g_dgraph_launch": (i32, [vp, vp]),
        "f2g_dgraph_state": (i32, [vp, P, P]),
        "f2g_dgraph_ritz": (i32, [vp, P, i64, vp]),
        "f2g_dgraph_history": (i32, [vp, P, i32]),
        "f2g_dgraph_serial": (i32, [vp, P]),
        "f2g_dgraph_batch_create": (i32, [P, i32, pp]),
        "f2g_dgraph_batch_destroy": (i32, [vp]),
        "f2g_dgraph_batch_launch": (i32, [vp, vp]),
        "f2g_dgraph_batch_nodes": (i32, [vp, P]),
        "f2g_sigma_set_hamiltonian_async": (i32, [vp, d, P, P, vp]),
        "f2g_probe_dfma": (i32, [i32, i32, i64, P, vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    return L


def lib():
    """Load the CUDA library (built by forte2_gb300.build / __graft_entry__.build())."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise CudaLibraryMissing(
                f"{LIB_PATH} is missing: the GPU path has no CPU fallback. Build it with "
                "`python -c \"import __graft_entry__ as g; g.build()\"`.")
        _lib = _declare(C.CDLL(LIB_PATH))
    return _lib


def check(rc: int):
    if rc == 0:
        return
    msg = lib().f2g_last_error().decode()
    if rc == 2:
        raise ValueError(msg)
    if rc == 4:
        raise MemoryError(msg)
    raise RuntimeError(msg)


_raw_stream = None


def stream_handle(stream=None):
    """cudaStream_t of `stream`, default the current stream of the current device."""
    global _raw_stream
    if stream is not None:
        return C.c_void_p(stream.cuda_stream)
    if _raw_stream is None:
        import torch

        get_raw = getattr(torch._C, "_cuda_getCurrentRawStream", None)
        get_dev = getattr(torch._C, "_cuda_getDevice", None)
        if get_raw is not None and get_dev is not None:
            _raw_stream = lambda: get_raw(get_dev())  # noqa: E731
        else:
            _raw_stream = lambda: torch.cuda.current_stream().cuda_stream  # noqa: E731
    return C.c_void_p(_raw_stream())
