"""GB300 (sm_103a) implementation of the autojax interferometer inversion.

The public functions mirror ``autojax.numba`` of ickc/python-autojax (same
names, same positional parameters) and run hand-written CUDA kernels through
the C ABI of ``libautojax_gb300.so``; there is no CPU fallback.
"""

from .api import (  # noqa: F401
    _w_compact_matmul_sparse_mapping_matrix_from,
    constant_regularization_matrix_from,
    curvature_matrix_via_w_compact_sparse_mapping_matrix_direct_from,
    curvature_matrix_via_w_compact_sparse_mapping_matrix_from,
    curvature_matrix_via_w_tilde_curvature_preload_interferometer_from,
    curvature_matrix_via_w_tilde_from,
    curvature_matrix_via_w_wilde_sparse_mapping_matrix_from,
    data_vector_from,
    dirty_image_from,
    log_evidence_and_grad,
    log_likelihood_function_via_w_compact_from,
    log_likelihood_function_via_w_tilde_from,
    mapping_matrix_from,
    mask_2d_centres_from,
    mask_2d_circular_from,
    noise_normalization_complex_from,
    reconstruction_positive_negative_from,
    slim_from_mask,
    sparse_mapping_matrix_transpose_matmul,
    w_compact_curvature_interferometer_from,
    w_tilde_curvature_interferometer_from,
    w_tilde_curvature_preload_interferometer_from,
    w_tilde_data_interferometer_from,
    w_tilde_via_compact_from,
    w_tilde_via_preload_from,
)

__version__ = "0.1.0"

# the functions of src/autojax/numba.py this package replaces, by name
NUMBA_API = (
    "mask_2d_centres_from",
    "mask_2d_circular_from",
    "w_tilde_data_interferometer_from",
    "w_tilde_curvature_interferometer_from",
    "w_compact_curvature_interferometer_from",
    "w_tilde_via_compact_from",
    "w_tilde_via_preload_from",
    "mapping_matrix_from",
    "data_vector_from",
    "curvature_matrix_via_w_tilde_from",
    "curvature_matrix_via_w_compact_sparse_mapping_matrix_direct_from",
    "_w_compact_matmul_sparse_mapping_matrix_from",
    "sparse_mapping_matrix_transpose_matmul",
    "curvature_matrix_via_w_wilde_sparse_mapping_matrix_from",
    "curvature_matrix_via_w_compact_sparse_mapping_matrix_from",
    "curvature_matrix_via_w_tilde_curvature_preload_interferometer_from",
    "constant_regularization_matrix_from",
    "reconstruction_positive_negative_from",
    "noise_normalization_complex_from",
    "log_likelihood_function_via_w_tilde_from",
    "log_likelihood_function_via_w_compact_from",
)

from . import torch_ops  # noqa: E402,F401  (registers torch.ops.autojax_gb300.*)
