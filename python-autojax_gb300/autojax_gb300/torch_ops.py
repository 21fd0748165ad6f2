"""The inversion as torch custom operators (``torch.ops.autojax_gb300.*``).

Every drop-in function of ``autojax.numba`` is an operator of the same name and
positional parameters (``torch.ops.autojax_gb300.mapping_matrix_from(...)``),
plus the two below with the library's own extensions.

Each operator is a thin wrapper over one C-ABI call of ``libautojax_gb300.so``
on the current stream, with a fake (shape-only) implementation so the ops can
be traced, and an autograd formula where the library computes the adjoint:

- ``w_tilde_curvature(noise_map_real, uv_wavelengths, grid_radians_slim,
  precision)`` -> (M, M) float64, numba.py:156-207.
- ``log_evidence(dirty_image, data, noise_map, w_tilde, pix_indexes,
  pix_weights, neighbors, neighbors_sizes, coefficient, precision)`` ->
  ``(out, grad_weights)``: out = [logE, dlogE/dlambda] (numba.py:761-857 with
  lambda = coefficient^2, the coefficient a device scalar), grad_weights =
  dlogE/dpix_weights (M, B).  logE is differentiable in ``pix_weights`` and
  ``coefficient`` (dlogE/dc = 2 c dlogE/dlambda).

``data`` and ``noise_map`` are complex128 (K,) tensors; ``precision`` is
``AJ_FP64`` (0) or ``AJ_MIXED`` (1).
"""

from __future__ import annotations

import torch

from . import _lib
from ._device import Call, ptr

_PREC = {_lib.AJ_FP64: "fp64", _lib.AJ_MIXED: "mixed"}


@torch.library.custom_op("autojax_gb300::w_tilde_curvature", mutates_args=())
def w_tilde_curvature(noise_map_real: torch.Tensor, uv_wavelengths: torch.Tensor, grid_radians_slim: torch.Tensor,
                      precision: int) -> torch.Tensor:
    from .api import w_tilde_curvature_interferometer_from

    return w_tilde_curvature_interferometer_from(noise_map_real, uv_wavelengths, grid_radians_slim,
                                                 precision=_PREC[precision])


@w_tilde_curvature.register_fake
def _(noise_map_real, uv_wavelengths, grid_radians_slim, precision):
    M = grid_radians_slim.shape[0]
    return grid_radians_slim.new_empty((M, M), dtype=torch.float64)


@torch.library.custom_op("autojax_gb300::log_evidence", mutates_args=())
def log_evidence(dirty_image: torch.Tensor, data: torch.Tensor, noise_map: torch.Tensor, w_tilde: torch.Tensor,
                 pix_indexes: torch.Tensor, pix_weights: torch.Tensor, neighbors: torch.Tensor,
                 neighbors_sizes: torch.Tensor, coefficient: torch.Tensor,
                 precision: int) -> tuple[torch.Tensor, torch.Tensor]:
    from .api import _evidence, _problem

    c = Call("log_evidence")
    p = _problem(c, dirty_image, data, noise_map, pix_indexes, pix_weights, neighbors, neighbors_sizes, 1.0,
                 w_tilde=w_tilde)
    coef = c.arr(coefficient.reshape(1), torch.float64, 1, "coefficient")
    p.coefficient_dev = ptr(coef)
    out, gw, _ = _evidence(c, p, _PREC[precision], True)
    return out, gw


@log_evidence.register_fake
def _(dirty_image, data, noise_map, w_tilde, pix_indexes, pix_weights, neighbors, neighbors_sizes, coefficient,
      precision):
    return dirty_image.new_empty(2, dtype=torch.float64), torch.empty_like(pix_weights, dtype=torch.float64)


def _setup(ctx, inputs, output):
    out, gw = output
    ctx.save_for_backward(out, gw, inputs[8])


def _backward(ctx, g_out, g_gw):
    out, gw, coefficient = ctx.saved_tensors
    g = g_out[0]
    d_weights = g * gw
    d_coef = (g * out[1] * 2.0 * coefficient).reshape(coefficient.shape)
    return None, None, None, None, None, d_weights, None, None, d_coef, None


log_evidence.register_autograd(_backward, setup_context=_setup)


# ------------------------------------------------------------------------------------------------
# One operator per drop-in function of autojax.numba (same name, same positional parameters): each
# calls the function of .api, i.e. one C-ABI entry point on the current stream.  Scalars of the
# reference (shape tuples, pixel scales, sizes, coefficients) are plain int / float arguments.

_F64 = torch.float64


def _api():
    from . import api

    return api


def _dev(*ts):
    for t in ts:
        if isinstance(t, torch.Tensor):
            return t.device
    return torch.device("cuda", torch.cuda.current_device()) if torch.cuda.is_available() else torch.device("meta")


@torch.library.custom_op("autojax_gb300::mask_2d_centres_from", mutates_args=())
def mask_2d_centres_from(shape_native: list[int], pixel_scales: list[float], centre: list[float]) -> torch.Tensor:
    """numba.py:13-44: the (y, x) centre in pixel units, as a float64 (2,) host tensor."""
    return torch.tensor(_api().mask_2d_centres_from(shape_native, pixel_scales, centre), dtype=_F64)


@mask_2d_centres_from.register_fake
def _(shape_native, pixel_scales, centre):
    return torch.empty(2, dtype=_F64)


@torch.library.custom_op("autojax_gb300::mask_2d_circular_from", mutates_args=())
def mask_2d_circular_from(shape_native: list[int], pixel_scales: list[float], radius: float,
                          centre: list[float]) -> torch.Tensor:
    """numba.py:50-86 on the current CUDA device."""
    from . import _lib as L

    ny, nx = int(shape_native[0]), int(shape_native[1])
    dev = _dev()
    out = torch.empty((ny, nx), dtype=torch.uint8, device=dev)
    L.check(L.load().aj_mask_2d_circular(ny, nx, float(pixel_scales[0]), float(pixel_scales[1]), float(radius),
                                         float(centre[0]), float(centre[1]), out.data_ptr(),
                                         torch.cuda.current_stream(dev).cuda_stream), "aj_mask_2d_circular")
    return out.bool()


@mask_2d_circular_from.register_fake
def _(shape_native, pixel_scales, radius, centre):
    return torch.empty((int(shape_native[0]), int(shape_native[1])), dtype=torch.bool, device=_dev())


@torch.library.custom_op("autojax_gb300::w_tilde_data_interferometer_from", mutates_args=())
def w_tilde_data_interferometer_from(visibilities_real: torch.Tensor, noise_map_real: torch.Tensor,
                                     uv_wavelengths: torch.Tensor, grid_radians_slim: torch.Tensor) -> torch.Tensor:
    return _api().w_tilde_data_interferometer_from(visibilities_real, noise_map_real, uv_wavelengths,
                                                   grid_radians_slim)


@w_tilde_data_interferometer_from.register_fake
def _(visibilities_real, noise_map_real, uv_wavelengths, grid_radians_slim):
    return grid_radians_slim.new_empty(grid_radians_slim.shape[0], dtype=_F64)


@torch.library.custom_op("autojax_gb300::w_tilde_curvature_interferometer_from", mutates_args=())
def w_tilde_curvature_interferometer_from(noise_map_real: torch.Tensor, uv_wavelengths: torch.Tensor,
                                          grid_radians_slim: torch.Tensor, precision: int = 0) -> torch.Tensor:
    return _api().w_tilde_curvature_interferometer_from(noise_map_real, uv_wavelengths, grid_radians_slim,
                                                        precision=_PREC[precision])


@w_tilde_curvature_interferometer_from.register_fake
def _(noise_map_real, uv_wavelengths, grid_radians_slim, precision=0):
    M = grid_radians_slim.shape[0]
    return grid_radians_slim.new_empty((M, M), dtype=_F64)


@torch.library.custom_op("autojax_gb300::w_compact_curvature_interferometer_from", mutates_args=())
def w_compact_curvature_interferometer_from(grid_size: int, noise_map_real: torch.Tensor,
                                            uv_wavelengths: torch.Tensor, pixel_scale: float) -> torch.Tensor:
    return _api().w_compact_curvature_interferometer_from(grid_size, noise_map_real, uv_wavelengths, pixel_scale)


@w_compact_curvature_interferometer_from.register_fake
def _(grid_size, noise_map_real, uv_wavelengths, pixel_scale):
    return noise_map_real.new_empty((grid_size, 2 * grid_size - 1), dtype=_F64)


@torch.library.custom_op("autojax_gb300::w_tilde_via_compact_from", mutates_args=())
def w_tilde_via_compact_from(w_compact: torch.Tensor, native_index_for_slim_index: torch.Tensor) -> torch.Tensor:
    return _api().w_tilde_via_compact_from(w_compact, native_index_for_slim_index)


@w_tilde_via_compact_from.register_fake
def _(w_compact, native_index_for_slim_index):
    M = native_index_for_slim_index.shape[0]
    return w_compact.new_empty((M, M), dtype=_F64)


@torch.library.custom_op("autojax_gb300::w_tilde_via_preload_from", mutates_args=())
def w_tilde_via_preload_from(w_tilde_preload: torch.Tensor, native_index_for_slim_index: torch.Tensor) -> torch.Tensor:
    return _api().w_tilde_via_preload_from(w_tilde_preload, native_index_for_slim_index)


@w_tilde_via_preload_from.register_fake
def _(w_tilde_preload, native_index_for_slim_index):
    M = native_index_for_slim_index.shape[0]
    return w_tilde_preload.new_empty((M, M), dtype=_F64)


@torch.library.custom_op("autojax_gb300::mapping_matrix_from", mutates_args=())
def mapping_matrix_from(pix_indexes_for_sub_slim_index: torch.Tensor, pix_weights_for_sub_slim_index: torch.Tensor,
                        pixels: int) -> torch.Tensor:
    return _api().mapping_matrix_from(pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index, pixels)


@mapping_matrix_from.register_fake
def _(pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index, pixels):
    return pix_weights_for_sub_slim_index.new_empty((pix_indexes_for_sub_slim_index.shape[0], pixels), dtype=_F64)


@torch.library.custom_op("autojax_gb300::data_vector_from", mutates_args=())
def data_vector_from(mapping_matrix: torch.Tensor, dirty_image: torch.Tensor) -> torch.Tensor:
    return _api().data_vector_from(mapping_matrix, dirty_image)


@data_vector_from.register_fake
def _(mapping_matrix, dirty_image):
    return mapping_matrix.new_empty(mapping_matrix.shape[1], dtype=_F64)


@torch.library.custom_op("autojax_gb300::curvature_matrix_via_w_tilde_from", mutates_args=())
def curvature_matrix_via_w_tilde_from(w_tilde: torch.Tensor, mapping_matrix: torch.Tensor) -> torch.Tensor:
    return _api().curvature_matrix_via_w_tilde_from(w_tilde, mapping_matrix)


@curvature_matrix_via_w_tilde_from.register_fake
def _(w_tilde, mapping_matrix):
    S = mapping_matrix.shape[1]
    return w_tilde.new_empty((S, S), dtype=_F64)


@torch.library.custom_op("autojax_gb300::sparse_mapping_matrix_transpose_matmul", mutates_args=())
def sparse_mapping_matrix_transpose_matmul(matrix: torch.Tensor, pix_indexes_for_sub_slim_index: torch.Tensor,
                                           pix_weights_for_sub_slim_index: torch.Tensor, pixels: int) -> torch.Tensor:
    return _api().sparse_mapping_matrix_transpose_matmul(matrix, pix_indexes_for_sub_slim_index,
                                                         pix_weights_for_sub_slim_index, pixels)


@sparse_mapping_matrix_transpose_matmul.register_fake
def _(matrix, pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index, pixels):
    return matrix.new_empty((pixels, matrix.shape[1]), dtype=_F64)


@torch.library.custom_op("autojax_gb300::curvature_matrix_via_w_wilde_sparse_mapping_matrix_from", mutates_args=())
def curvature_matrix_via_w_wilde_sparse_mapping_matrix_from(w_tilde: torch.Tensor,
                                                            pix_indexes_for_sub_slim_index: torch.Tensor,
                                                            pix_weights_for_sub_slim_index: torch.Tensor,
                                                            pixels: int) -> torch.Tensor:
    return _api().curvature_matrix_via_w_wilde_sparse_mapping_matrix_from(w_tilde, pix_indexes_for_sub_slim_index,
                                                                          pix_weights_for_sub_slim_index, pixels)


@curvature_matrix_via_w_wilde_sparse_mapping_matrix_from.register_fake
def _(w_tilde, pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index, pixels):
    return w_tilde.new_empty((pixels, pixels), dtype=_F64)


@torch.library.custom_op("autojax_gb300::_w_compact_matmul_sparse_mapping_matrix_from", mutates_args=())
def _w_compact_matmul_sparse_mapping_matrix_from(w_compact: torch.Tensor, native_index_for_slim_index: torch.Tensor,
                                                 pix_indexes_for_sub_slim_index: torch.Tensor,
                                                 pix_weights_for_sub_slim_index: torch.Tensor,
                                                 pixels: int) -> torch.Tensor:
    return _api()._w_compact_matmul_sparse_mapping_matrix_from(w_compact, native_index_for_slim_index,
                                                               pix_indexes_for_sub_slim_index,
                                                               pix_weights_for_sub_slim_index, pixels)


@_w_compact_matmul_sparse_mapping_matrix_from.register_fake
def _(w_compact, native_index_for_slim_index, pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index, pixels):
    return w_compact.new_empty((native_index_for_slim_index.shape[0], pixels), dtype=_F64)


def _compact_curvature_fake(w_compact, native_index_for_slim_index, pix_indexes_for_sub_slim_index,
                            pix_weights_for_sub_slim_index, pixels):
    return w_compact.new_empty((pixels, pixels), dtype=_F64)


@torch.library.custom_op("autojax_gb300::curvature_matrix_via_w_compact_sparse_mapping_matrix_from", mutates_args=())
def curvature_matrix_via_w_compact_sparse_mapping_matrix_from(w_compact: torch.Tensor,
                                                              native_index_for_slim_index: torch.Tensor,
                                                              pix_indexes_for_sub_slim_index: torch.Tensor,
                                                              pix_weights_for_sub_slim_index: torch.Tensor,
                                                              pixels: int) -> torch.Tensor:
    return _api().curvature_matrix_via_w_compact_sparse_mapping_matrix_from(
        w_compact, native_index_for_slim_index, pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index,
        pixels)


@torch.library.custom_op("autojax_gb300::curvature_matrix_via_w_compact_sparse_mapping_matrix_direct_from",
                         mutates_args=())
def curvature_matrix_via_w_compact_sparse_mapping_matrix_direct_from(w_compact: torch.Tensor,
                                                                     native_index_for_slim_index: torch.Tensor,
                                                                     pix_indexes_for_sub_slim_index: torch.Tensor,
                                                                     pix_weights_for_sub_slim_index: torch.Tensor,
                                                                     pixels: int) -> torch.Tensor:
    return _api().curvature_matrix_via_w_compact_sparse_mapping_matrix_direct_from(
        w_compact, native_index_for_slim_index, pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index,
        pixels)


@torch.library.custom_op("autojax_gb300::curvature_matrix_via_w_tilde_curvature_preload_interferometer_from",
                         mutates_args=())
def curvature_matrix_via_w_tilde_curvature_preload_interferometer_from(w_compact: torch.Tensor,
                                                                       native_index_for_slim_index: torch.Tensor,
                                                                       pix_indexes_for_sub_slim_index: torch.Tensor,
                                                                       pix_weights_for_sub_slim_index: torch.Tensor,
                                                                       pixels: int) -> torch.Tensor:
    return _api().curvature_matrix_via_w_tilde_curvature_preload_interferometer_from(
        w_compact, native_index_for_slim_index, pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index,
        pixels)


for _op in (curvature_matrix_via_w_compact_sparse_mapping_matrix_from,
            curvature_matrix_via_w_compact_sparse_mapping_matrix_direct_from,
            curvature_matrix_via_w_tilde_curvature_preload_interferometer_from):
    _op.register_fake(_compact_curvature_fake)


@torch.library.custom_op("autojax_gb300::constant_regularization_matrix_from", mutates_args=())
def constant_regularization_matrix_from(coefficient: float, neighbors: torch.Tensor,
                                        neighbors_sizes: torch.Tensor) -> torch.Tensor:
    return _api().constant_regularization_matrix_from(coefficient, neighbors, neighbors_sizes)


@constant_regularization_matrix_from.register_fake
def _(coefficient, neighbors, neighbors_sizes):
    S = neighbors.shape[0]
    return neighbors.new_empty((S, S), dtype=_F64)


@torch.library.custom_op("autojax_gb300::reconstruction_positive_negative_from", mutates_args=())
def reconstruction_positive_negative_from(data_vector: torch.Tensor, curvature_reg_matrix: torch.Tensor) -> torch.Tensor:
    return _api().reconstruction_positive_negative_from(data_vector, curvature_reg_matrix)


@reconstruction_positive_negative_from.register_fake
def _(data_vector, curvature_reg_matrix):
    return data_vector.new_empty(data_vector.shape[0], dtype=_F64)


@torch.library.custom_op("autojax_gb300::noise_normalization_complex_from", mutates_args=())
def noise_normalization_complex_from(noise_map: torch.Tensor) -> torch.Tensor:
    return _api().noise_normalization_complex_from(noise_map).clone()


@noise_normalization_complex_from.register_fake
def _(noise_map):
    return noise_map.new_empty((), dtype=_F64)


@torch.library.custom_op("autojax_gb300::log_likelihood_function_via_w_tilde_from", mutates_args=())
def log_likelihood_function_via_w_tilde_from(dirty_image: torch.Tensor, data: torch.Tensor, noise_map: torch.Tensor,
                                             w_tilde: torch.Tensor, pix_indexes_for_sub_slim_index: torch.Tensor,
                                             pix_weights_for_sub_slim_index: torch.Tensor, neighbors: torch.Tensor,
                                             neighbors_sizes: torch.Tensor, precision: int = 0) -> torch.Tensor:
    return _api().log_likelihood_function_via_w_tilde_from(
        dirty_image, data, noise_map, w_tilde, pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index,
        neighbors, neighbors_sizes, precision=_PREC[precision]).clone()


@log_likelihood_function_via_w_tilde_from.register_fake
def _(dirty_image, data, noise_map, w_tilde, pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index,
      neighbors, neighbors_sizes, precision=0):
    return dirty_image.new_empty((), dtype=_F64)


@torch.library.custom_op("autojax_gb300::log_likelihood_function_via_w_compact_from", mutates_args=())
def log_likelihood_function_via_w_compact_from(dirty_image: torch.Tensor, data: torch.Tensor,
                                               noise_map: torch.Tensor, w_compact: torch.Tensor,
                                               native_index_for_slim_index: torch.Tensor,
                                               pix_indexes_for_sub_slim_index: torch.Tensor,
                                               pix_weights_for_sub_slim_index: torch.Tensor, neighbors: torch.Tensor,
                                               neighbors_sizes: torch.Tensor, precision: int = 0) -> torch.Tensor:
    return _api().log_likelihood_function_via_w_compact_from(
        dirty_image, data, noise_map, w_compact, native_index_for_slim_index, pix_indexes_for_sub_slim_index,
        pix_weights_for_sub_slim_index, neighbors, neighbors_sizes, precision=_PREC[precision]).clone()


@log_likelihood_function_via_w_compact_from.register_fake
def _(dirty_image, data, noise_map, w_compact, native_index_for_slim_index, pix_indexes_for_sub_slim_index,
      pix_weights_for_sub_slim_index, neighbors, neighbors_sizes, precision=0):
    return dirty_image.new_empty((), dtype=_F64)


__all__ = ["w_tilde_curvature", "log_evidence", "mask_2d_centres_from", "mask_2d_circular_from",
           "w_tilde_data_interferometer_from", "w_tilde_curvature_interferometer_from",
           "w_compact_curvature_interferometer_from", "w_tilde_via_compact_from", "w_tilde_via_preload_from",
           "mapping_matrix_from", "data_vector_from", "curvature_matrix_via_w_tilde_from",
           "sparse_mapping_matrix_transpose_matmul", "curvature_matrix_via_w_wilde_sparse_mapping_matrix_from",
           "_w_compact_matmul_sparse_mapping_matrix_from", "curvature_matrix_via_w_compact_sparse_mapping_matrix_from",
           "curvature_matrix_via_w_compact_sparse_mapping_matrix_direct_from",
           "curvature_matrix_via_w_tilde_curvature_preload_interferometer_from",
           "constant_regularization_matrix_from", "reconstruction_positive_negative_from",
           "noise_normalization_complex_from", "log_likelihood_function_via_w_tilde_from",
           "log_likelihood_function_via_w_compact_from"]
