"""The inversion as torch custom operators (``torch.ops.autojax_gb300.*``).

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

__all__ = ["w_tilde_curvature", "log_evidence"]
