"""NumPy restatement of the reference's FP64 inversion chain (test oracle).

Test infrastructure: see the package docstring.  Each function has the name and
positional parameters of the reference function it restates and cites the
lines of ``src/autojax/numba.py`` (or ``src/autojax/original.py``) whose
arithmetic it follows.  Loops of the reference are vectorised; the summation
order therefore differs from the reference's at the last-ulp level only.

Semantics kept from the reference:

* sparse mapping rows stop at the first ``-1`` (``numba.py:372-373``);
* ``mapping_matrix_from`` *assigns* (a repeated source index keeps the last
  weight, ``numba.py:375``) while the sparse products *accumulate*
  (``numba.py:586``, ``548``, ``495``);
* neighbour rows stop at the first ``-1`` and repeated neighbours accumulate
  (``numba.py:689-694``);
* the likelihoods hard-code ``coefficient = 1.0`` (``numba.py:819``, ``923``).
"""

from __future__ import annotations

import numpy as np

TWO_PI = 2.0 * np.pi
LOG_TWO_PI = np.log(TWO_PI)

# visibilities per vectorised block; bounds the (M, M, chunk) temporaries
_K_BLOCK = 64


# ---------------------------------------------------------------------------
# geometry (numba.py:10-86)
# ---------------------------------------------------------------------------


def mask_2d_centres_from(shape_native, pixel_scales, centre):
    """numba.py:13-44 — (y, x) centre of the mask in pixel units."""
    return (
        0.5 * (shape_native[0] - 1) - (centre[0] / pixel_scales[0]),
        0.5 * (shape_native[1] - 1) + (centre[1] / pixel_scales[1]),
    )


def mask_2d_circular_from(shape_native, pixel_scales, radius, centre):
    """numba.py:50-86 — True marks a masked pixel (outside the circle)."""
    cy, cx = mask_2d_centres_from(shape_native, pixel_scales, centre)
    ys, xs = np.indices(shape_native)
    return (radius * radius) < (
        np.square((ys - cy) * pixel_scales[0]) + np.square((xs - cx) * pixel_scales[1])
    )


# ---------------------------------------------------------------------------
# w_tilde and its compact / preload forms (numba.py:89-290, original.py:229-449)
# ---------------------------------------------------------------------------


def w_tilde_data_interferometer_from(visibilities_real, noise_map_real, uv_wavelengths, grid_radians_slim):
    """numba.py:95-152 — res_i = sum_k (n_k^2/v_k)^2 cos(2pi(g_i1 u_k0 + g_i0 u_k1))."""
    g_2pi = TWO_PI * np.asarray(grid_radians_slim, dtype=np.float64)
    M = g_2pi.shape[0]
    K = uv_wavelengths.shape[0]
    w = np.square(np.square(noise_map_real) / visibilities_real)
    res = np.zeros(M)
    for k0 in range(0, K, 4096):
        k1 = min(K, k0 + 4096)
        ph = np.outer(g_2pi[:, 1], uv_wavelengths[k0:k1, 0]) + np.outer(g_2pi[:, 0], uv_wavelengths[k0:k1, 1])
        res += np.cos(ph) @ w[k0:k1]
    return res


def w_tilde_curvature_interferometer_from(noise_map_real, uv_wavelengths, grid_radians_slim):
    """numba.py:156-207 — dense W~_ij = sum_k n_k^-2 cos(dg1_ij u_k0 + dg0_ij u_k1), dg = 2pi(g_i - g_j)."""
    g_2pi = TWO_PI * np.asarray(grid_radians_slim, dtype=np.float64)
    M = g_2pi.shape[0]
    K = uv_wavelengths.shape[0]
    d0 = g_2pi[:, None, 0] - g_2pi[None, :, 0]
    d1 = g_2pi[:, None, 1] - g_2pi[None, :, 1]
    inv = np.reciprocal(np.square(noise_map_real))
    w = np.zeros((M, M))
    blk = max(1, min(_K_BLOCK, (1 << 24) // max(1, M * M)))
    for k0 in range(0, K, blk):
        k1 = min(K, k0 + blk)
        u0 = uv_wavelengths[k0:k1, 0]
        u1 = uv_wavelengths[k0:k1, 1]
        ph = d1[None] * u0[:, None, None] + d0[None] * u1[:, None, None]
        w += np.tensordot(inv[k0:k1], np.cos(ph), axes=(0, 0))
    return w


def w_tilde_entries(noise_map_real, uv_wavelengths, grid_radians_slim, rows, cols):
    """Entries (rows[e], cols[e]) of numba.py:156-207's W~, by the same sum over every visibility.

    For checking W~ at sizes where the full M x M oracle sum would take hours: the phase of
    entry (i, j) is dg1_ij u_k0 + dg0_ij u_k1 with dg = 2pi (g_i - g_j) (numba.py:204).
    """
    g_2pi = TWO_PI * np.asarray(grid_radians_slim, dtype=np.float64)
    rows = np.asarray(rows, dtype=np.int64)
    cols = np.asarray(cols, dtype=np.int64)
    d0 = g_2pi[rows, 0] - g_2pi[cols, 0]
    d1 = g_2pi[rows, 1] - g_2pi[cols, 1]
    inv = np.reciprocal(np.square(noise_map_real))
    K = uv_wavelengths.shape[0]
    out = np.zeros(rows.shape[0])
    blk = max(1, (1 << 22) // max(1, rows.shape[0]))
    for k0 in range(0, K, blk):
        k1 = min(K, k0 + blk)
        ph = np.outer(d1, uv_wavelengths[k0:k1, 0]) + np.outer(d0, uv_wavelengths[k0:k1, 1])
        out += np.cos(ph) @ inv[k0:k1]
    return out


def w_compact_curvature_interferometer_from(grid_size, noise_map_real, uv_wavelengths, pixel_scale):
    """numba.py:211-234 — offset table w_c[n0, n1+N-1] = sum_k n_k^-2 cos(D(n1 u_k0 - n0 u_k1)).

    D = pi^2 * pixel_scale / 324000 = 2 pi * (pixel_scale in radians) (numba.py:223).
    """
    N = int(grid_size)
    K = uv_wavelengths.shape[0]
    twopi_d = (np.pi * np.pi * pixel_scale) / 324000.0
    d0 = (twopi_d * np.arange(N, dtype=np.float64)).reshape(-1, 1)
    d1 = twopi_d * (np.arange(2 * N - 1, dtype=np.float64) - (N - 1))
    inv = np.square(np.reciprocal(noise_map_real))
    out = np.zeros((N, 2 * N - 1))
    blk = max(1, min(1024, (1 << 24) // max(1, N * (2 * N - 1))))
    for k0 in range(0, K, blk):
        k1 = min(K, k0 + blk)
        u0 = uv_wavelengths[k0:k1, 0]
        u1 = uv_wavelengths[k0:k1, 1]
        ph = d1[None, None, :] * u0[:, None, None] - d0[None, :, :] * u1[:, None, None]
        out += np.tensordot(inv[k0:k1], np.cos(ph), axes=(0, 0))
    return out


def w_tilde_curvature_preload_interferometer_from(
    noise_map_real, uv_wavelengths, shape_masked_pixels_2d, grid_radians_2d
):
    """original.py:230-403 — the 4-quadrant (2Y, 2X) preload table.

    Each quadrant holds sum_k n_k^-2 cos(2pi(x_off u_k0 + y_off u_k1)) where the
    offsets are measured from one corner of the (Y, X) top-left block of the
    grid: (0,0) for [i, j] (original.py:352-362), (0,-1) for [i, -j], j>0
    (364-375), (-1,0) for [-i, j], i>0 (377-388), (-1,-1) for [-i, -j], i,j>0
    (390-401).  Row/column Y (resp. X) is never written and stays zero.
    """
    Y, X = int(shape_masked_pixels_2d[0]), int(shape_masked_pixels_2d[1])
    g = np.asarray(grid_radians_2d, dtype=np.float64)[0:Y, 0:X]
    gy, gx = g.shape[0], g.shape[1]
    inv = np.asarray(noise_map_real, dtype=np.float64) ** -2.0
    I, J = np.meshgrid(np.arange(Y), np.arange(X), indexing="ij")
    out = np.zeros((2 * Y, 2 * X))

    def quadrant(valid, corner, src_i, src_j, dst_i, dst_j):
        ii, jj = I[valid], J[valid]
        si, sj = src_i(ii, jj), src_j(ii, jj)
        yo = g[corner[0], corner[1], 0] - g[si, sj, 0]
        xo = g[corner[0], corner[1], 1] - g[si, sj, 1]
        vals = _cos_sum(xo, yo, inv, uv_wavelengths)
        out[dst_i(ii), dst_j(jj)] += vals

    everything = np.ones((Y, X), dtype=bool)
    quadrant(everything, (0, 0), lambda i, j: i, lambda i, j: j, lambda i: i, lambda j: j)
    quadrant(J > 0, (0, -1), lambda i, j: i, lambda i, j: gx - j - 1, lambda i: i, lambda j: 2 * X - j)
    quadrant(I > 0, (-1, 0), lambda i, j: gy - i - 1, lambda i, j: j, lambda i: 2 * Y - i, lambda j: j)
    quadrant(
        (I > 0) & (J > 0),
        (-1, -1),
        lambda i, j: gy - i - 1,
        lambda i, j: gx - j - 1,
        lambda i: 2 * Y - i,
        lambda j: 2 * X - j,
    )
    return out


def _cos_sum(xo, yo, inv, uv):
    """sum_k inv_k cos(2pi (xo u_k0 + yo u_k1)) for every offset pair (xo, yo)."""
    res = np.zeros(xo.shape[0])
    for k0 in range(0, uv.shape[0], 2048):
        k1 = min(uv.shape[0], k0 + 2048)
        ph = 2.0 * np.pi * (np.outer(xo, uv[k0:k1, 0]) + np.outer(yo, uv[k0:k1, 1]))
        res += np.cos(ph) @ inv[k0:k1]
    return res


def w_compact_separable(grid_size, noise_map_real, uv_wavelengths, pixel_scale, block=16384):
    """numba.py:211-234's offset table by a separable complex product (host input preparation).

    cos(D(n1 u - n0 v)) = Re[e^{i D n1 u} e^{-i D n0 v}], so the table is
    Re(E_v^H diag(w) E_u) with E_u[k, n1 + N - 1] = e^{i D n1 u_k} and
    E_v[k, n0] = e^{i D n0 v_k}: one complex GEMM per visibility block instead
    of N (2N - 1) cosines per visibility.  The same sum as
    ``w_compact_curvature_interferometer_from`` in another order, fast enough
    to build the table for 1e6 visibilities on host cores.
    """
    N = int(grid_size)
    K = uv_wavelengths.shape[0]
    twopi_d = (np.pi * np.pi * pixel_scale) / 324000.0
    n1 = np.arange(2 * N - 1, dtype=np.float64) - (N - 1)
    n0 = np.arange(N, dtype=np.float64)
    inv = np.square(np.reciprocal(noise_map_real))
    acc = np.zeros((N, 2 * N - 1), dtype=np.complex128)
    for k0 in range(0, K, block):
        k1 = min(K, k0 + block)
        Eu = np.exp(1j * (twopi_d * uv_wavelengths[k0:k1, 0])[:, None] * n1[None, :])
        Ev = np.exp(1j * (twopi_d * uv_wavelengths[k0:k1, 1])[:, None] * n0[None, :])
        acc += (np.conj(Ev) * inv[k0:k1, None]).T @ Eu
    return np.ascontiguousarray(acc.real)


def w_tilde_via_compact_from(w_compact, native_index_for_slim_index):
    """numba.py:238-255 — W~_ij = w_c[|di0|, (di1 if di0 >= 0 else -di1) + N - 1]."""
    idx = np.asarray(native_index_for_slim_index)
    offset = w_compact.shape[0] - 1
    m = idx[:, None, 0] - idx[None, :, 0]
    d = idx[:, None, 1] - idx[None, :, 1]
    n = np.where(m >= 0, d, -d) + offset
    return np.ascontiguousarray(w_compact[np.abs(m), n])


def w_tilde_via_preload_from(w_tilde_preload, native_index_for_slim_index):
    """numba.py:259-290 — W~_ij = preload[y_j - y_i, x_j - x_i] (negative indices wrap)."""
    idx = np.asarray(native_index_for_slim_index)
    dy = idx[None, :, 0] - idx[:, None, 0]
    dx = idx[None, :, 1] - idx[:, None, 1]
    return np.ascontiguousarray(w_tilde_preload[dy, dx])


# ---------------------------------------------------------------------------
# mapping matrix and sparse products (numba.py:293-653)
# ---------------------------------------------------------------------------


def _valid_entries(pix_indexes):
    """Mask of entries that precede the first -1 of their row (numba.py:372-373)."""
    return np.cumprod(np.asarray(pix_indexes) != -1, axis=1).astype(bool)


def _summed_mapping(pix_indexes, pix_weights, pixels):
    """Dense T with repeated indices of a row summed (the sparse-product semantics)."""
    M = pix_indexes.shape[0]
    valid = _valid_entries(pix_indexes)
    rows = np.broadcast_to(np.arange(M)[:, None], pix_indexes.shape)[valid]
    T = np.zeros((M, int(pixels)))
    np.add.at(T, (rows, pix_indexes[valid]), pix_weights[valid])
    return T


def mapping_matrix_from(pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index, pixels):
    """numba.py:294-376 — dense (M, S) mapping; a repeated index keeps its last weight."""
    idx = np.asarray(pix_indexes_for_sub_slim_index)
    wts = np.asarray(pix_weights_for_sub_slim_index, dtype=np.float64)
    M, B = idx.shape
    valid = _valid_entries(idx)
    T = np.zeros((M, int(pixels)))
    rows = np.arange(M)
    for b in range(B):
        sel = valid[:, b]
        T[rows[sel], idx[sel, b]] = wts[sel, b]
    return T


def data_vector_from(mapping_matrix, dirty_image):
    """numba.py:380-406 — D = dirty_image @ T."""
    return dirty_image @ mapping_matrix


def curvature_matrix_via_w_tilde_from(w_tilde, mapping_matrix):
    """numba.py:410-435 — F = T^T W~ T."""
    return mapping_matrix.T @ w_tilde @ mapping_matrix


def sparse_mapping_matrix_transpose_matmul(matrix, pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index, pixels):
    """numba.py:553-587 — T^T @ matrix with T in its sparse (index, weight) form."""
    T = _summed_mapping(np.asarray(pix_indexes_for_sub_slim_index), np.asarray(pix_weights_for_sub_slim_index), pixels)
    return T.T @ matrix


def curvature_matrix_via_w_wilde_sparse_mapping_matrix_from(
    w_tilde, pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index, pixels
):
    """numba.py:591-614 — F = T^T (T^T W~)^T via two sparse products."""
    TW = sparse_mapping_matrix_transpose_matmul(w_tilde, pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index, pixels)
    return sparse_mapping_matrix_transpose_matmul(
        np.ascontiguousarray(TW.T), pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index, pixels
    )


def _w_compact_matmul_sparse_mapping_matrix_from(
    w_compact, native_index_for_slim_index, pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index, pixels
):
    """numba.py:500-549 — Omega = W~ T with W~ gathered from the compact table."""
    W = w_tilde_via_compact_from(w_compact, native_index_for_slim_index)
    T = _summed_mapping(np.asarray(pix_indexes_for_sub_slim_index), np.asarray(pix_weights_for_sub_slim_index), pixels)
    return W @ T


def curvature_matrix_via_w_compact_sparse_mapping_matrix_from(
    w_compact, native_index_for_slim_index, pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index, pixels
):
    """numba.py:618-647 — F = T^T (W~ T) from the compact table."""
    omega = _w_compact_matmul_sparse_mapping_matrix_from(
        w_compact, native_index_for_slim_index, pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index, pixels
    )
    return sparse_mapping_matrix_transpose_matmul(omega, pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index, pixels)


# numba.py:651-653 keeps this alias for the preload-named benchmark.
curvature_matrix_via_w_tilde_curvature_preload_interferometer_from = curvature_matrix_via_w_compact_sparse_mapping_matrix_from


def curvature_matrix_via_w_compact_sparse_mapping_matrix_direct_from(
    w_compact, native_index_for_slim_index, pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index, pixels
):
    """numba.py:439-496 — the same F by the direct four-loop form (same arithmetic, other order)."""
    W = w_tilde_via_compact_from(w_compact, native_index_for_slim_index)
    T = _summed_mapping(np.asarray(pix_indexes_for_sub_slim_index), np.asarray(pix_weights_for_sub_slim_index), pixels)
    return T.T @ W @ T


# ---------------------------------------------------------------------------
# regularisation, solve, likelihood (numba.py:656-967)
# ---------------------------------------------------------------------------


def constant_regularization_matrix_from(coefficient, neighbors, neighbors_sizes):
    """numba.py:657-695 — H = diag(1e-8 + c^2 n_i) - c^2 sum over neighbour entries."""
    nb = np.asarray(neighbors)
    S = nb.shape[0]
    c2 = coefficient * coefficient
    H = np.diag(1e-8 + c2 * np.asarray(neighbors_sizes, dtype=np.float64))
    valid = _valid_entries(nb)
    rows = np.broadcast_to(np.arange(S)[:, None], nb.shape)[valid]
    np.subtract.at(H, (rows, nb[valid]), c2)
    return H


def reconstruction_positive_negative_from(data_vector, curvature_reg_matrix):
    """numba.py:699-731 — s = (F + H)^-1 D by LU (LAPACK gesv)."""
    return np.linalg.solve(curvature_reg_matrix, data_vector)


def noise_normalization_complex_from(noise_map):
    """numba.py:735-752 — 2 (K log 2pi + sum log|Re| + sum log|Im|)."""
    nm = np.ascontiguousarray(noise_map)
    return 2.0 * (nm.size * LOG_TWO_PI + np.log(np.abs(nm.view(np.float64))).sum())


def _evidence(noise_map, data, curvature_matrix, regularization_matrix, data_vector):
    """numba.py:839-857 (and 943-967) — assemble logE from its parts."""
    noise_normalization = noise_normalization_complex_from(noise_map)
    curvature_reg_matrix = curvature_matrix + regularization_matrix
    reconstruction = reconstruction_positive_negative_from(data_vector, curvature_reg_matrix)
    chi = np.ascontiguousarray(data).view(np.float64) / np.ascontiguousarray(noise_map).view(np.float64)
    reg_plus_chi2 = chi @ chi - reconstruction @ data_vector
    log_a = np.linalg.slogdet(curvature_reg_matrix)[1]
    log_h = np.linalg.slogdet(regularization_matrix)[1]
    return -0.5 * (reg_plus_chi2 + log_a - log_h + noise_normalization)


def log_likelihood_function_via_w_tilde_from(
    dirty_image, data, noise_map, w_tilde, pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index, neighbors, neighbors_sizes, coefficient=1.0
):
    """numba.py:761-857 — logE with F = T^T W~ T (dense T from mapping_matrix_from).

    ``coefficient`` is hard-coded to 1.0 in the reference (numba.py:819); the
    keyword exists so the tests can pin the lambda-dependence the GPU path exposes.
    """
    S = np.asarray(neighbors_sizes).size
    T = mapping_matrix_from(pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index, S)
    F = curvature_matrix_via_w_tilde_from(w_tilde, T)
    H = constant_regularization_matrix_from(coefficient, neighbors, neighbors_sizes)
    D = data_vector_from(T, dirty_image)
    return _evidence(noise_map, data, F, H, D)


def log_likelihood_function_via_w_compact_from(
    dirty_image,
    data,
    noise_map,
    w_compact,
    native_index_for_slim_index,
    pix_indexes_for_sub_slim_index,
    pix_weights_for_sub_slim_index,
    neighbors,
    neighbors_sizes,
    coefficient=1.0,
):
    """numba.py:866-967 — logE with F from the compact table (sparse, summed T) and D from the dense T."""
    S = np.asarray(neighbors_sizes).size
    F = curvature_matrix_via_w_compact_sparse_mapping_matrix_from(
        w_compact, native_index_for_slim_index, pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index, S
    )
    H = constant_regularization_matrix_from(coefficient, neighbors, neighbors_sizes)
    T = mapping_matrix_from(pix_indexes_for_sub_slim_index, pix_weights_for_sub_slim_index, S)
    D = data_vector_from(T, dirty_image)
    return _evidence(noise_map, data, F, H, D)


# ---------------------------------------------------------------------------
# the `original.py` signatures that differ from numba.py
# ---------------------------------------------------------------------------


def original_mapping_matrix_from(
    pix_indexes_for_sub_slim_index,
    pix_size_for_sub_slim_index,
    pix_weights_for_sub_slim_index,
    pixels,
    total_mask_pixels,
    slim_index_for_sub_slim_index,
    sub_fraction,
):
    """original.py:453-545 — accumulate sub_fraction * weight over pix_size entries per sub-pixel."""
    idx = np.asarray(pix_indexes_for_sub_slim_index)
    sizes = np.asarray(pix_size_for_sub_slim_index)
    slim = np.asarray(slim_index_for_sub_slim_index)
    T = np.zeros((int(total_mask_pixels), int(pixels)))
    valid = np.arange(idx.shape[1])[None, :] < sizes[:, None]
    sub = np.broadcast_to(np.arange(idx.shape[0])[:, None], idx.shape)[valid]
    rows = slim[sub]
    np.add.at(T, (rows, idx[valid]), np.asarray(sub_fraction)[rows] * np.asarray(pix_weights_for_sub_slim_index)[valid])
    return T


def original_curvature_matrix_via_w_tilde_curvature_preload_interferometer_from(
    curvature_preload, pix_indexes_for_sub_slim_index, pix_size_for_sub_slim_index, pix_weights_for_sub_slim_index, native_index_for_slim_index, pix_pixels
):
    """original.py:600-700 — F from the preload table: upper pairs (ip1 > ip0) plus their mirror plus the diagonal."""
    idx = np.asarray(native_index_for_slim_index)
    M = idx.shape[0]
    dy = idx[None, :, 0] - idx[:, None, 0]
    dx = idx[None, :, 1] - idx[:, None, 1]
    W = curvature_preload[dy, dx]
    upper = np.triu(W, 1)
    sizes = np.asarray(pix_size_for_sub_slim_index)
    pidx = np.asarray(pix_indexes_for_sub_slim_index)
    valid = np.arange(pidx.shape[1])[None, :] < sizes[:, None]
    rows = np.broadcast_to(np.arange(M)[:, None], pidx.shape)[valid]
    T = np.zeros((M, int(pix_pixels)))
    np.add.at(T, (rows, pidx[valid]), np.asarray(pix_weights_for_sub_slim_index)[valid])
    Fu = T.T @ upper @ T
    F = Fu + Fu.T
    F += curvature_preload[0, 0] * (T.T @ T)
    return F
