"""ctypes binding of ``libautojax_gb300.so`` (the C ABI in ``include/autojax_gb300.h``).

The library is loaded on first use.  There is no fallback: if it has not been
built, or no CUDA device is visible, every entry point raises.
"""

from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

from .build import LIB_PATH

AJ_OK = 0
AJ_ERR_ARG = -1
AJ_ERR_CUDA = -2
AJ_ERR_WORKSPACE = -3
AJ_ERR_TOO_LARGE = -4
AJ_NOALLOC_SOLVE_MAX_S = 1024
AJ_BATCH_BRANCHES = 16
AJ_INFO_INDEX_RANGE = 1
AJ_INFO_NOT_POSITIVE_DEFINITE = 2
AJ_INFO_SINGULAR = 3
AJ_FP64 = 0
AJ_MIXED = 1

P = C.c_void_p
I64 = C.c_int64
D = C.c_double
SZ = C.c_size_t
INT = C.c_int


class Problem(C.Structure):
    """struct aj_problem (include/autojax_gb300.h)."""

    _fields_ = [
        ("M", I64),
        ("K", I64),
        ("S", I64),
        ("B", I64),
        ("P", I64),
        ("N", I64),
        ("dirty_image", P),
        ("data", P),
        ("noise_map", P),
        ("w_tilde64", P),
        ("w_tilde_hi", P),
        ("w_tilde_lo", P),
        ("w_compact", P),
        ("native_index", P),
        ("pix_indexes", P),
        ("pix_weights", P),
        ("neighbors", P),
        ("neighbors_sizes", P),
        ("coefficient", D),
        ("coefficient_dev", P),
    ]


# name -> (restype, argtypes), in the order of the header
SIGNATURES = {
    "aj_version": (C.c_char_p, []),
    "aj_last_cuda_error": (INT, []),
    "aj_launch_count": (C.c_ulonglong, []),
    "aj_probe_fma": (INT, [INT, I64, INT, P, P]),
    "aj_mask_2d_circular": (INT, [I64, I64, D, D, D, D, D, P, P]),
    "aj_slim_from_mask": (INT, [P, I64, I64, P, I64, P, P, P, P]),
    "aj_w_tilde_curvature_workspace_size": (SZ, [I64, I64, INT]),
    "aj_w_tilde_curvature": (INT, [P, P, P, I64, I64, P, P, P, SZ, INT, P]),
    "aj_digit_syrk_probe": (INT, [P, I64, I64, P, P, P, INT, P, P]),
    "aj_w_compact_curvature_workspace_size": (SZ, [I64, I64, INT]),
    "aj_w_compact_curvature": (INT, [I64, P, P, I64, D, P, P, SZ, INT, P]),
    "aj_w_tilde_preload_workspace_size": (SZ, [I64, I64, I64, INT]),
    "aj_w_tilde_preload": (INT, [P, P, I64, I64, I64, P, I64, I64, P, P, SZ, INT, P]),
    "aj_w_tilde_data_workspace_size": (SZ, [I64, I64, INT]),
    "aj_w_tilde_data": (INT, [P, P, P, P, I64, I64, P, P, SZ, INT, P]),
    "aj_w_tilde_via_compact": (INT, [P, I64, P, I64, P, P, P, P]),
    "aj_w_tilde_via_preload": (INT, [P, I64, I64, P, I64, P, P, P, P]),
    "aj_mapping_matrix": (INT, [P, P, I64, I64, I64, P, P, P]),
    "aj_data_vector": (INT, [P, P, I64, I64, P, P]),
    "aj_curvature_dense_workspace_size": (SZ, [I64, I64]),
    "aj_curvature_dense": (INT, [P, P, I64, I64, P, P, SZ, P]),
    "aj_sparse_workspace_size": (SZ, [I64, I64, I64, I64]),
    "aj_sparse_mapping_matrix_transpose_matmul": (INT, [P, I64, I64, P, P, I64, I64, P, P, SZ, P, P]),
    "aj_curvature_w_tilde_sparse": (INT, [P, I64, P, P, I64, I64, P, P, SZ, P, P]),
    "aj_curvature_w_tilde_sparse_mixed_workspace_size": (SZ, [I64, I64, I64]),
    "aj_curvature_w_tilde_sparse_mixed": (INT, [P, P, I64, P, P, I64, I64, P, P, SZ, P, P]),
    "aj_w_compact_matmul_sparse": (INT, [P, I64, P, I64, P, P, I64, I64, P, P, SZ, P, P]),
    "aj_curvature_w_compact_sparse": (INT, [P, I64, P, I64, P, P, I64, I64, P, P, SZ, P, P]),
    "aj_curvature_preload_original_workspace_size": (SZ, [I64, I64, I64]),
    "aj_curvature_preload_original": (INT, [P, I64, I64, P, P, P, I64, P, I64, I64, P, P, SZ, P, P]),
    "aj_mapping_matrix_original": (INT, [P, P, P, I64, I64, I64, I64, P, P, P, P, P]),
    "aj_constant_regularization": (INT, [D, P, P, I64, I64, P, P, P]),
    "aj_spd_solve_workspace_size": (SZ, [I64]),
    "aj_spd_solve": (INT, [P, P, I64, P, P, SZ, P, P]),
    "aj_spd_solve_noalloc": (INT, [P, P, I64, P, P, P]),
    "aj_lu_solve_workspace_size": (SZ, [I64]),
    "aj_lu_solve": (INT, [P, P, I64, P, P, P, SZ, P, P]),
    "aj_spd_logdet": (INT, [P, I64, P, P, SZ, P, P]),
    "aj_spd_inverse_workspace_size": (SZ, [I64]),
    "aj_spd_inverse": (INT, [P, I64, P, P, P, SZ, P, P]),
    "aj_spd_inverse_mixed_workspace_size": (SZ, [I64]),
    "aj_spd_inverse_mixed": (INT, [P, I64, P, P, P, SZ, P, P]),
    "aj_noise_normalization": (INT, [P, I64, P, P]),
    "aj_split_f64": (INT, [P, I64, P, P, P]),
    "aj_log_evidence_workspace_size": (SZ, [C.POINTER(Problem), INT, INT]),
    "aj_log_evidence": (INT, [C.POINTER(Problem), INT, INT, P, P, P, P, SZ, P, P]),
    "aj_set_tile_policy": (INT, [INT, INT]),
    "aj_get_tile_policy": (INT, [P]),
    "aj_dirty_image_workspace_size": (SZ, [I64, I64]),
    "aj_dirty_image": (INT, [P, P, P, P, I64, I64, P, P, SZ, P]),
    "aj_sis_trace": (INT, [P, I64, D, P, P, P]),
    "aj_sis_trace_vjp": (INT, [P, I64, P, P, P]),
    "aj_delaunay_weights": (INT, [P, I64, P, I64, P, I64, P, P, P, P]),
    "aj_delaunay_weights_vjp": (INT, [P, I64, P, I64, P, P, P, P, P]),
    "aj_bilinear_weights": (INT, [P, I64, I64, D, P, P, P]),
    "aj_bilinear_weights_vjp": (INT, [P, I64, I64, D, P, P, P]),
    "aj_log_evidence_batched": (INT, [C.POINTER(Problem), I64, INT, INT, P, P, P, P, P, P, P]),
    "aj_release_stream": (INT, [P]),
    "aj_graph_begin": (INT, [P]),
    "aj_graph_end": (INT, [P, C.POINTER(P)]),
    "aj_graph_launch": (INT, [P, P]),
    "aj_graph_destroy": (INT, [P]),
}

_lock = threading.Lock()
_lib = None


class LibraryError(RuntimeError):
    pass


def load() -> C.CDLL:
    """Load the in-tree library (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = Path(LIB_PATH)
        if not path.exists():
            raise LibraryError(
                f"{path.name} is not built; run `python -c 'import __graft_entry__ as g; g.build()'` "
                "or `python -m autojax_gb300.build` (there is no CPU fallback)"
            )
        import torch  # noqa: F401  (brings up the same CUDA runtime first)

        lib = C.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def exported_symbols() -> list[str]:
    return list(SIGNATURES)


def check(rc: int, what: str) -> None:
    if rc == AJ_OK:
        return
    lib = load()
    if rc == AJ_ERR_ARG:
        raise ValueError(f"{what}: invalid argument")
    if rc == AJ_ERR_WORKSPACE:
        raise RuntimeError(f"{what}: workspace too small")
    if rc == AJ_ERR_TOO_LARGE:
        raise ValueError(f"{what}: size above the entry point's fixed capacity")
    if rc == AJ_ERR_CUDA:
        raise RuntimeError(f"{what}: CUDA launch failed (cudaError {lib.aj_last_cuda_error()})")
    raise RuntimeError(f"{what}: status {rc}")
