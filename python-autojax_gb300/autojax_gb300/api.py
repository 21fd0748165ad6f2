"""Drop-in GPU versions of ``autojax.numba`` (ickc/python-autojax ``src/autojax/numba.py``).

Every function keeps the reference's name and positional parameters.
NumPy arguments return NumPy results (float for scalars); torch tensors return
torch tensors on the device.  Keyword-only extensions:

* ``precision`` — ``"fp64"`` (IEEE float64 throughout, the parity path) or
  ``"mixed"``;
* ``coefficient`` on the likelihoods — the regularisation coefficient the
  reference hard-codes to 1.0 (numba.py:819, 923).

Errors: wrong NumPy dtypes or non-contiguous arrays raise TypeError (the
reference's typed signatures reject them); an index outside its range raises
IndexError; a curvature-plus-regularisation matrix that is not positive
definite raises ``numpy.linalg.LinAlgError``.
"""

from __future__ import annotations

import math

import numpy as np
import torch

from . import _lib
from ._device import Call, precision_code, ptr

f64, i64, u8 = torch.float64, torch.int64, torch.uint8


def _lib_call(fn_name: str, *args):
    lib = _lib.load()
    rc = getattr(lib, fn_name)(*args)
    _lib.check(rc, fn_name)


# ---------------------------------------------------------------- geometry


def mask_2d_centres_from(shape_native, pixel_scales, centre):
    """numba.py:13-44 — (y, x) centre of the mask in pixel units (scalar bookkeeping)."""
    return (
        0.5 * (shape_native[0] - 1) - (centre[0] / pixel_scales[0]),
        0.5 * (shape_native[1] - 1) + (centre[1] / pixel_scales[1]),
    )


def mask_2d_circular_from(shape_native, pixel_scales, radius, centre):
    """numba.py:50-86 — boolean mask, True outside the circle (bit-exact)."""
    c = Call("mask_2d_circular_from")
    ny, nx = int(shape_native[0]), int(shape_native[1])
    out = c.empty((ny, nx), u8)
    _lib_call("aj_mask_2d_circular", ny, nx, float(pixel_scales[0]), float(pixel_scales[1]), float(radius),
              float(centre[0]), float(centre[1]), ptr(out), c.stream())
    res = out.bool()
    return res.cpu().numpy() if c.numpy_out else res


def slim_from_mask(mask, grid_radians_2d=None):
    """tests.py:279-281, 304-306 — (native_index_for_slim_index, grid_radians_slim) of the unmasked pixels."""
    c = Call("slim_from_mask")
    if isinstance(mask, torch.Tensor):
        m = c.arr(mask.to(u8), u8, 2, "mask")
    else:
        import numpy as np

        m = c.arr(np.ascontiguousarray(np.asarray(mask, dtype=bool)).view(np.uint8), u8, 2, "mask")
    ny, nx = m.shape
    g = c.arr(grid_radians_2d, f64, 3, "grid_radians_2d") if grid_radians_2d is not None else None
    count = c.zeros(1, i64)
    nat = c.empty((ny * nx, 2), i64)
    gs = c.empty((ny * nx, 2), f64) if g is not None else None
    _lib_call("aj_slim_from_mask", ptr(m), ny, nx, ptr(g), ny * nx, ptr(nat), ptr(gs), ptr(count), c.stream())
    n = int(count.item())
    nat = nat[:n].contiguous()
    if g is None:
        return c.out(nat)
    return c.out(nat), c.out(gs[:n].contiguous())


# -------------------------------------------------------- w_tilde family


def w_tilde_data_interferometer_from(visibilities_real, noise_map_real, uv_wavelengths, grid_radians_slim, *,
                                     precision="fp64"):
    """numba.py:95-152."""
    c = Call("w_tilde_data_interferometer_from")
    v = c.arr(visibilities_real, f64, 1, "visibilities_real")
    n = c.arr(noise_map_real, f64, 1, "noise_map_real")
    uv = c.arr(uv_wavelengths, f64, 2, "uv_wavelengths")
    g = c.arr(grid_radians_slim, f64, 2, "grid_radians_slim")
    K, M = uv.shape[0], g.shape[0]
    pc = precision_code(precision)
    out = c.empty(M)
    ws = c.workspace(_lib.load().aj_w_tilde_data_workspace_size(M, K, pc))
    _lib_call("aj_w_tilde_data", ptr(v), ptr(n), ptr(uv), ptr(g), K, M, ptr(out), ptr(ws), ws.numel(), pc, c.stream())
    return c.out(out)


def dirty_image_from(visibilities, noise_map_real, uv_wavelengths, grid_radians_slim):
    """Dirty image (M,) of complex visibilities (no reference function: the reference reads it from
    its dataset): sum_k noise_k^-2 (Re V_k cos t - Im V_k sin t), t = 2 pi (x u_k + y v_k), with the
    w_tilde pairing of grid and uv columns (numba.py:204)."""
    c = Call("dirty_image_from")
    v = c.complex_as_real(visibilities, "visibilities")
    n = c.arr(noise_map_real, f64, 1, "noise_map_real")
    uv = c.arr(uv_wavelengths, f64, 2, "uv_wavelengths")
    g = c.arr(grid_radians_slim, f64, 2, "grid_radians_slim")
    K, M = uv.shape[0], g.shape[0]
    out = c.empty(M)
    ws = c.workspace(_lib.load().aj_dirty_image_workspace_size(M, K))
    _lib_call("aj_dirty_image", ptr(v), ptr(n), ptr(uv), ptr(g), K, M, ptr(out), ptr(ws), ws.numel(), c.stream())
    return c.out(out)


def w_tilde_curvature_interferometer_from(noise_map_real, uv_wavelengths, grid_radians_slim, *, precision="fp64",
                                          planes=False):
    """numba.py:156-207 — dense (M, M) w_tilde.

    ``planes=True`` also returns its (2, M, M) double-float planes (hi, lo), the
    form the mixed-precision likelihood reads.
    """
    c = Call("w_tilde_curvature_interferometer_from")
    n = c.arr(noise_map_real, f64, 1, "noise_map_real")
    uv = c.arr(uv_wavelengths, f64, 2, "uv_wavelengths")
    g = c.arr(grid_radians_slim, f64, 2, "grid_radians_slim")
    K, M = uv.shape[0], g.shape[0]
    pc = precision_code(precision)
    out = c.empty((M, M))
    pl = c.empty((2, M, M), torch.float32) if planes else None
    ws = c.workspace(_lib.load().aj_w_tilde_curvature_workspace_size(K, M, pc))
    _lib_call("aj_w_tilde_curvature", ptr(n), ptr(uv), ptr(g), K, M, ptr(out), ptr(pl), ptr(ws), ws.numel(), pc,
              c.stream())
    return (c.out(out), c.out(pl)) if planes else c.out(out)


def w_compact_curvature_interferometer_from(grid_size, noise_map_real, uv_wavelengths, pixel_scale, *,
                                            precision="fp64"):
    """numba.py:211-234 — the (N, 2N-1) offset table."""
    c = Call("w_compact_curvature_interferometer_from")
    n = c.arr(noise_map_real, f64, 1, "noise_map_real")
    uv = c.arr(uv_wavelengths, f64, 2, "uv_wavelengths")
    N, K = int(grid_size), uv.shape[0]
    pc = precision_code(precision)
    out = c.empty((N, 2 * N - 1))
    ws = c.workspace(_lib.load().aj_w_compact_curvature_workspace_size(N, K, pc))
    _lib_call("aj_w_compact_curvature", N, ptr(n), ptr(uv), K, float(pixel_scale), ptr(out), ptr(ws), ws.numel(), pc,
              c.stream())
    return c.out(out)


def w_tilde_curvature_preload_interferometer_from(noise_map_real, uv_wavelengths, shape_masked_pixels_2d,
                                                  grid_radians_2d, *, precision="fp64"):
    """original.py:230-403 — the 4-quadrant (2Y, 2X) preload table."""
    c = Call("w_tilde_curvature_preload_interferometer_from")
    n = c.arr(noise_map_real, f64, 1, "noise_map_real")
    uv = c.arr(uv_wavelengths, f64, 2, "uv_wavelengths")
    g = c.arr(grid_radians_2d, f64, 3, "grid_radians_2d")
    Y, X = int(shape_masked_pixels_2d[0]), int(shape_masked_pixels_2d[1])
    K = uv.shape[0]
    pc = precision_code(precision)
    out = c.empty((2 * Y, 2 * X))
    ws = c.workspace(_lib.load().aj_w_tilde_preload_workspace_size(Y, X, K, pc))
    _lib_call("aj_w_tilde_preload", ptr(n), ptr(uv), K, Y, X, ptr(g), g.shape[0], g.shape[1], ptr(out), ptr(ws),
              ws.numel(), pc, c.stream())
    return c.out(out)


def w_tilde_via_compact_from(w_compact, native_index_for_slim_index):
    """numba.py:238-255."""
    c = Call("w_tilde_via_compact_from")
    wc = c.arr(w_compact, f64, 2, "w_compact")
    nat = c.arr(native_index_for_slim_index, i64, 2, "native_index_for_slim_index")
    M = nat.shape[0]
    out = c.empty((M, M))
    info = c.info()
    _lib_call("aj_w_tilde_via_compact", ptr(wc), wc.shape[0], ptr(nat), M, ptr(out), None, ptr(info), c.stream())
    c.check_info(info)
    return c.out(out)


def w_tilde_via_preload_from(w_tilde_preload, native_index_for_slim_index):
    """numba.py:259-290."""
    c = Call("w_tilde_via_preload_from")
    pre = c.arr(w_tilde_preload, f64, 2, "w_tilde_preload")
    nat = c.arr(native_index_for_slim_index, i64, 2, "native_index_for_slim_index")
    M = nat.shape[0]
    out = c.empty((M, M))
    info = c.info()
    _lib_call("aj_w_tilde_via_preload", ptr(pre), pre.shape[0], pre.shape[1], ptr(nat), M, ptr(out), None, ptr(info),
              c.stream())
    c.check_info(info)
    return c.out(out)


# ----------------------------------------------------------- mapping matrix


def mapping_matrix_from(pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index, pixels):
    """numba.py:294-376 — dense (M, S) mapping matrix."""
    c = Call("mapping_matrix_from")
    idx = c.arr(pix_indexes_for_sub_slim_index, i64, 2, "pix_indexes_for_sub_slim_index")
    w = c.arr(pix_weights_for_sub_slim_index, f64, 2, "pix_weights_for_sub_slim_index")
    M, B = idx.shape
    S = int(pixels)
    out = c.empty((M, S))
    info = c.info()
    _lib_call("aj_mapping_matrix", ptr(idx), ptr(w), M, B, S, ptr(out), ptr(info), c.stream())
    c.check_info(info)
    return c.out(out)


def data_vector_from(mapping_matrix, dirty_image):
    """numba.py:380-406 — D = dirty_image @ T."""
    c = Call("data_vector_from")
    T = c.arr(mapping_matrix, f64, 2, "mapping_matrix")
    d = c.arr(dirty_image, f64, 1, "dirty_image")
    M, S = T.shape
    out = c.empty(S)
    _lib_call("aj_data_vector", ptr(T), ptr(d), M, S, ptr(out), c.stream())
    return c.out(out)


def curvature_matrix_via_w_tilde_from(w_tilde, mapping_matrix):
    """numba.py:410-435 — F = T^T W T with dense operands."""
    c = Call("curvature_matrix_via_w_tilde_from")
    W = c.arr(w_tilde, f64, 2, "w_tilde")
    T = c.arr(mapping_matrix, f64, 2, "mapping_matrix")
    M, S = T.shape
    out = c.empty((S, S))
    ws = c.workspace(_lib.load().aj_curvature_dense_workspace_size(M, S))
    _lib_call("aj_curvature_dense", ptr(W), ptr(T), M, S, ptr(out), ptr(ws), ws.numel(), c.stream())
    return c.out(out)


def _sparse_inputs(c: Call, pix_indexes, pix_weights):
    idx = c.arr(pix_indexes, i64, 2, "pix_indexes_for_sub_slim_index")
    w = c.arr(pix_weights, f64, 2, "pix_weights_for_sub_slim_index")
    return idx, w


def sparse_mapping_matrix_transpose_matmul(matrix, pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index,
                                           pixels):
    """numba.py:553-587 — T^T @ matrix with the sparse mapping."""
    c = Call("sparse_mapping_matrix_transpose_matmul")
    X = c.arr(matrix, f64, 2, "matrix")
    idx, w = _sparse_inputs(c, pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index)
    M, cols = X.shape
    B = idx.shape[1]
    S = int(pixels)
    out = c.zeros((S, cols))
    ws = c.workspace(_lib.load().aj_sparse_workspace_size(M, B, S, cols))
    info = c.info()
    _lib_call("aj_sparse_mapping_matrix_transpose_matmul", ptr(X), M, cols, ptr(idx), ptr(w), B, S, ptr(out), ptr(ws),
              ws.numel(), ptr(info), c.stream())
    c.check_info(info)
    return c.out(out)


def curvature_matrix_via_w_wilde_sparse_mapping_matrix_from(w_tilde, pix_indexes_for_sub_slim_index,
                                                            pix_weights_for_sub_slim_index, pixels, *,
                                                            precision="fp64", w_tilde_planes=None):
    """numba.py:591-614 (the reference's public name keeps its 'wilde' spelling).

    ``precision="mixed"`` runs the mixed likelihood's own double-float gathers
    on w_tilde's (hi, lo) planes (``w_tilde_planes`` (2, M, M) float32, split
    from ``w_tilde`` when not given) and returns F joined to float64.
    """
    c = Call("curvature_matrix_via_w_wilde_sparse_mapping_matrix_from")
    W = c.arr(w_tilde, f64, 2, "w_tilde")
    idx, w = _sparse_inputs(c, pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index)
    M, B, S = W.shape[0], idx.shape[1], int(pixels)
    out = c.empty((S, S))
    if precision_code(precision) == _lib.AJ_MIXED:
        if w_tilde_planes is None:
            pl = c.empty((2, M, M), torch.float32)
            _lib_call("aj_split_f64", ptr(W), M * M, ptr(pl[0]), ptr(pl[1]), c.stream())
        else:
            pl = c.arr(w_tilde_planes, torch.float32, 3, "w_tilde_planes")
        ws = c.workspace(_lib.load().aj_curvature_w_tilde_sparse_mixed_workspace_size(M, B, S))
        info = c.info()
        _lib_call("aj_curvature_w_tilde_sparse_mixed", ptr(pl[0]), ptr(pl[1]), M, ptr(idx), ptr(w), B, S, ptr(out),
                  ptr(ws), ws.numel(), ptr(info), c.stream())
        c.check_info(info)
        return c.out(out)
    ws = c.workspace(_lib.load().aj_sparse_workspace_size(M, B, S, M))
    info = c.info()
    _lib_call("aj_curvature_w_tilde_sparse", ptr(W), M, ptr(idx), ptr(w), B, S, ptr(out), ptr(ws), ws.numel(),
              ptr(info), c.stream())
    c.check_info(info)
    return c.out(out)


def _w_compact_matmul_sparse_mapping_matrix_from(w_compact, native_index_for_slim_index,
                                                 pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index,
                                                 pixels):
    """numba.py:500-549 — Omega = W T with W gathered from the compact table."""
    c = Call("_w_compact_matmul_sparse_mapping_matrix_from")
    wc = c.arr(w_compact, f64, 2, "w_compact")
    nat = c.arr(native_index_for_slim_index, i64, 2, "native_index_for_slim_index")
    idx, w = _sparse_inputs(c, pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index)
    M, B, S = nat.shape[0], idx.shape[1], int(pixels)
    out = c.empty((M, S))
    ws = c.workspace(_lib.load().aj_sparse_workspace_size(M, B, S, M))
    info = c.info()
    _lib_call("aj_w_compact_matmul_sparse", ptr(wc), wc.shape[0], ptr(nat), M, ptr(idx), ptr(w), B, S, ptr(out),
              ptr(ws), ws.numel(), ptr(info), c.stream())
    c.check_info(info)
    return c.out(out)


def curvature_matrix_via_w_compact_sparse_mapping_matrix_from(w_compact, native_index_for_slim_index,
                                                              pix_indexes_for_sub_slim_index,
                                                              pix_weights_for_sub_slim_index, pixels):
    """numba.py:618-647 — F = T^T (W T) from the compact table."""
    c = Call("curvature_matrix_via_w_compact_sparse_mapping_matrix_from")
    wc = c.arr(w_compact, f64, 2, "w_compact")
    nat = c.arr(native_index_for_slim_index, i64, 2, "native_index_for_slim_index")
    idx, w = _sparse_inputs(c, pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index)
    M, B, S = nat.shape[0], idx.shape[1], int(pixels)
    out = c.empty((S, S))
    ws = c.workspace(_lib.load().aj_sparse_workspace_size(M, B, S, M))
    info = c.info()
    _lib_call("aj_curvature_w_compact_sparse", ptr(wc), wc.shape[0], ptr(nat), M, ptr(idx), ptr(w), B, S, ptr(out),
              ptr(ws), ws.numel(), ptr(info), c.stream())
    c.check_info(info)
    return c.out(out)


# numba.py:651-653 keeps this alias for the preload-named benchmark
curvature_matrix_via_w_tilde_curvature_preload_interferometer_from = (
    curvature_matrix_via_w_compact_sparse_mapping_matrix_from
)


def curvature_matrix_via_w_compact_sparse_mapping_matrix_direct_from(w_compact, native_index_for_slim_index,
                                                                     pix_indexes_for_sub_slim_index,
                                                                     pix_weights_for_sub_slim_index, pixels):
    """numba.py:439-496 — same F as the two-step form (the GPU path never materialises W either way)."""
    return curvature_matrix_via_w_compact_sparse_mapping_matrix_from(
        w_compact, native_index_for_slim_index, pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index,
        pixels)


# ------------------------------------------------- regularisation and solve


def constant_regularization_matrix_from(coefficient, neighbors, neighbors_sizes):
    """numba.py:657-695."""
    c = Call("constant_regularization_matrix_from")
    nb = c.arr(neighbors, i64, 2, "neighbors")
    nsz = c.arr(neighbors_sizes, i64, 1, "neighbors_sizes")
    S, P = nb.shape
    out = c.empty((S, S))
    info = c.info()
    _lib_call("aj_constant_regularization", float(coefficient), ptr(nb), ptr(nsz), S, P, ptr(out), ptr(info),
              c.stream())
    c.check_info(info)
    return c.out(out)


def _lu_solve(c: Call, D, A, S, want_solution=True):
    """x = A^-1 D and log|det A| by the float64 LU with partial pivoting (numba.py:731, 849-850)."""
    out = c.empty(S) if want_solution else None
    logabsdet = c.empty(1)
    ws = c.workspace(_lib.load().aj_lu_solve_workspace_size(S))
    info = c.info()
    _lib_call("aj_lu_solve", ptr(D), ptr(A), S, ptr(out), ptr(logabsdet), ptr(ws), ws.numel(), ptr(info), c.stream())
    c.check_info(info)
    return out, logabsdet


def reconstruction_positive_negative_from(data_vector, curvature_reg_matrix):
    """numba.py:699-731 — s = A^-1 D.

    A float64 Cholesky solve; an A that is not positive definite (which the
    inversion's A = F + H never is, but a caller's matrix may be) is solved by
    the LU with partial pivoting the reference's np.linalg.solve uses, and a
    singular one raises LinAlgError as there.
    """
    c = Call("reconstruction_positive_negative_from")
    D = c.arr(data_vector, f64, 1, "data_vector")
    A = c.arr(curvature_reg_matrix, f64, 2, "curvature_reg_matrix")
    S = D.shape[0]
    out = c.empty(S)
    ws = c.workspace(_lib.load().aj_spd_solve_workspace_size(S))
    info = c.info()
    _lib_call("aj_spd_solve", ptr(D), ptr(A), S, ptr(out), ptr(ws), ws.numel(), ptr(info), c.stream())
    if int(info[0].item()) == _lib.AJ_INFO_NOT_POSITIVE_DEFINITE:
        out, _ = _lu_solve(c, D, A, S)
        return c.out(out)
    c.check_info(info)
    return c.out(out)


def noise_normalization_complex_from(noise_map):
    """numba.py:735-752."""
    c = Call("noise_normalization_complex_from")
    nm = c.complex_as_real(noise_map, "noise_map")
    K = nm.shape[0]
    out = c.empty(1)
    _lib_call("aj_noise_normalization", ptr(nm), K, ptr(out), c.stream())
    return c.scalar(out)


# ---------------------------------------------------------------- likelihood


def _problem(c: Call, dirty_image, data, noise_map, pix_indexes, pix_weights, neighbors, neighbors_sizes,
             coefficient, *, w_tilde=None, w_compact=None, native_index=None):
    p = _lib.Problem()
    d = c.arr(dirty_image, f64, 1, "dirty_image")
    da = c.complex_as_real(data, "data")
    nm = c.complex_as_real(noise_map, "noise_map")
    idx, w = _sparse_inputs(c, pix_indexes, pix_weights)
    nb = c.arr(neighbors, i64, 2, "neighbors")
    nsz = c.arr(neighbors_sizes, i64, 1, "neighbors_sizes")
    p.M, p.B = idx.shape
    p.K = da.shape[0]
    p.S, p.P = nb.shape[0], nb.shape[1]
    p.dirty_image, p.data, p.noise_map = ptr(d), ptr(da), ptr(nm)
    p.pix_indexes, p.pix_weights = ptr(idx), ptr(w)
    p.neighbors, p.neighbors_sizes = ptr(nb), ptr(nsz)
    p.coefficient = float(coefficient)
    if w_tilde is not None:
        W = c.arr(w_tilde, f64, 2, "w_tilde")
        p.w_tilde64 = ptr(W)
    else:
        wc = c.arr(w_compact, f64, 2, "w_compact")
        nat = c.arr(native_index, i64, 2, "native_index_for_slim_index")
        p.w_compact, p.native_index, p.N = ptr(wc), ptr(nat), wc.shape[0]
    return p


def _evidence(c: Call, p, precision, with_grad):
    lib = _lib.load()
    pc = precision_code(precision)
    ws = c.workspace(lib.aj_log_evidence_workspace_size(p, pc, int(with_grad)))
    out = c.zeros(2)
    gw = c.zeros((p.M, p.B)) if with_grad else None
    rec = c.empty(p.S)
    info = c.info()
    _lib_call("aj_log_evidence", p, pc, int(with_grad), ptr(out), ptr(gw), ptr(rec), ptr(ws), ws.numel(), ptr(info),
              c.stream())
    c.check_info(info)
    return out, gw, rec


def _evidence_by_lu(c: Call, F, dirty_image, data, noise_map, pix_indexes, pix_weights, neighbors, neighbors_sizes,
                    coefficient):
    """numba.py:839-857 assembled from the library's entry points with both log|det| and the solve
    by LU: the fallback for an A = F + H that is not positive definite (float64 throughout)."""
    S = int(c.arr(neighbors_sizes, i64, 1, "neighbors_sizes").shape[0])
    Fd = c.arr(F, f64, 2, "curvature_matrix")
    H = c.arr(constant_regularization_matrix_from(coefficient, c.arr(neighbors, i64, 2, "neighbors"),
                                                  c.arr(neighbors_sizes, i64, 1, "neighbors_sizes")), f64, 2, "H")
    A = (Fd + H).contiguous()
    T = mapping_matrix_from(c.arr(pix_indexes, i64, 2, "pix_indexes_for_sub_slim_index"),
                            c.arr(pix_weights, f64, 2, "pix_weights_for_sub_slim_index"), S)
    D = data_vector_from(T, c.arr(dirty_image, f64, 1, "dirty_image"))
    s, log_a = _lu_solve(c, D, A, S)
    _, log_h = _lu_solve(c, None, H, S, want_solution=False)
    da = c.complex_as_real(data, "data").reshape(-1)
    nm = c.complex_as_real(noise_map, "noise_map").reshape(-1)
    chi = da / nm
    norm = noise_normalization_complex_from(c.arr(noise_map, torch.complex128, 1, "noise_map"))
    return -0.5 * (chi @ chi - s @ D + log_a[0] - log_h[0] + norm)


def log_likelihood_function_via_w_tilde_from(dirty_image, data, noise_map, w_tilde, pix_indexes_for_sub_slim_index,
                                             pix_weights_for_sub_slim_index, neighbors, neighbors_sizes, *,
                                             coefficient=1.0, precision="fp64"):
    """numba.py:761-857 — the log-evidence with a dense w_tilde.

    An A = F + H that is not positive definite falls back to the reference's
    LU semantics (solve and log|det| by LU, float64), see _evidence_by_lu.
    """
    c = Call("log_likelihood_function_via_w_tilde_from")
    p = _problem(c, dirty_image, data, noise_map, pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index,
                 neighbors, neighbors_sizes, coefficient, w_tilde=w_tilde)
    try:
        out, _, _ = _evidence(c, p, precision, False)
    except np.linalg.LinAlgError:
        T = mapping_matrix_from(c.arr(pix_indexes_for_sub_slim_index, i64, 2, "pix_indexes_for_sub_slim_index"),
                                c.arr(pix_weights_for_sub_slim_index, f64, 2, "pix_weights_for_sub_slim_index"),
                                int(p.S))
        F = curvature_matrix_via_w_tilde_from(c.arr(w_tilde, f64, 2, "w_tilde"), T)
        return c.scalar(_evidence_by_lu(c, F, dirty_image, data, noise_map, pix_indexes_for_sub_slim_index,
                                        pix_weights_for_sub_slim_index, neighbors, neighbors_sizes, coefficient))
    return c.scalar(out[0])


def log_likelihood_function_via_w_compact_from(dirty_image, data, noise_map, w_compact, native_index_for_slim_index,
                                               pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index,
                                               neighbors, neighbors_sizes, *, coefficient=1.0, precision="fp64"):
    """numba.py:866-967 — the log-evidence from the compact table (LU fallback as above)."""
    c = Call("log_likelihood_function_via_w_compact_from")
    p = _problem(c, dirty_image, data, noise_map, pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index,
                 neighbors, neighbors_sizes, coefficient, w_compact=w_compact, native_index=native_index_for_slim_index)
    try:
        out, _, _ = _evidence(c, p, precision, False)
    except np.linalg.LinAlgError:
        F = curvature_matrix_via_w_compact_sparse_mapping_matrix_from(
            c.arr(w_compact, f64, 2, "w_compact"), c.arr(native_index_for_slim_index, i64, 2, "native_index"),
            c.arr(pix_indexes_for_sub_slim_index, i64, 2, "pix_indexes_for_sub_slim_index"),
            c.arr(pix_weights_for_sub_slim_index, f64, 2, "pix_weights_for_sub_slim_index"), int(p.S))
        return c.scalar(_evidence_by_lu(c, F, dirty_image, data, noise_map, pix_indexes_for_sub_slim_index,
                                        pix_weights_for_sub_slim_index, neighbors, neighbors_sizes, coefficient))
    return c.scalar(out[0])


def log_evidence_and_grad(dirty_image, data, noise_map, w_tilde, pix_indexes_for_sub_slim_index,
                          pix_weights_for_sub_slim_index, neighbors, neighbors_sizes, *, coefficient=1.0,
                          precision="fp64", w_compact=None, native_index_for_slim_index=None,
                          return_reconstruction=False):
    """logE with its adjoint (no reference counterpart).

    Returns ``(logE, dlogE/dlambda, dlogE/dpix_weights)`` with lambda =
    coefficient**2; pass ``w_tilde=None`` with ``w_compact`` and
    ``native_index_for_slim_index`` for the compact form.  With
    ``return_reconstruction=True`` the evaluation's own s = (F + H)^-1 D
    (numba.py:699-731) comes fourth.
    """
    c = Call("log_evidence_and_grad")
    if w_tilde is not None:
        p = _problem(c, dirty_image, data, noise_map, pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index,
                     neighbors, neighbors_sizes, coefficient, w_tilde=w_tilde)
    else:
        p = _problem(c, dirty_image, data, noise_map, pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index,
                     neighbors, neighbors_sizes, coefficient, w_compact=w_compact,
                     native_index=native_index_for_slim_index)
    out, gw, rec = _evidence(c, p, precision, True)
    if c.numpy_out:
        o = out.cpu().numpy()
        res = (float(o[0]), float(o[1]), gw.cpu().numpy())
        return res + (rec.cpu().numpy(),) if return_reconstruction else res
    return (out[0], out[1], gw, rec) if return_reconstruction else (out[0], out[1], gw)


LOG_TWO_PI = math.log(2.0 * math.pi)
