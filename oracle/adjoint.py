"""Closed-form adjoint of the log-evidence (test oracle, no reference counterpart).

Test infrastructure: see the package docstring.  The reference computes
(numba.py:839-857)

    logE = -1/2 [ chi.chi - s.D + log|A| - log|H| + norm ],
    A = F + H,  F = T^T W T,  D = T^T d,  s = A^-1 D,
    H = 1e-8 I + lam * L,  L = diag(n) - Adj  (lam = coefficient^2, numba.py:686-694).

Differentiating (W symmetric, Omega = W T):

    dlogE/dlam   = -1/2 [ s^T L s + tr(A^-1 L) - tr(H^-1 L) ]
    dlogE/dT[m,j] = d_m s_j - (Omega s)_m s_j - (Omega A^-1)[m, j]

The weight gradient is dlogE/dT read on the sparsity pattern: entries after
the first -1 of a row, and entries overwritten by a later repeat of the same
index (mapping_matrix_from assigns, numba.py:375), get zero.
"""

from __future__ import annotations

import numpy as np

from . import numpy_port as ref


def laplacian_from(neighbors, neighbors_sizes):
    """L = diag(n) - Adj with the neighbour-row semantics of numba.py:688-694."""
    H1 = ref.constant_regularization_matrix_from(1.0, neighbors, neighbors_sizes)
    return H1 - 1e-8 * np.eye(H1.shape[0])


def effective_weight_mask(pix_indexes):
    """True where a weight reaches the dense mapping matrix (valid and not overwritten later)."""
    idx = np.asarray(pix_indexes)
    valid = np.cumprod(idx != -1, axis=1).astype(bool)
    keep = valid.copy()
    B = idx.shape[1]
    for b in range(B):
        for b2 in range(b + 1, B):
            keep[:, b] &= ~(valid[:, b2] & (idx[:, b2] == idx[:, b]))
    return keep


def log_evidence_and_grad(
    dirty_image, data, noise_map, w_tilde, pix_indexes, pix_weights, neighbors, neighbors_sizes, coefficient=1.0
):
    """Return (logE, dlogE/dlam, dlogE/dweights[M, B]) for the w_tilde likelihood.

    logE equals numba.py:761-857 evaluated with regularisation ``coefficient``.
    """
    idx = np.asarray(pix_indexes)
    S = np.asarray(neighbors_sizes).size
    lam = coefficient * coefficient
    T = ref.mapping_matrix_from(idx, pix_weights, S)
    omega = w_tilde @ T
    F = T.T @ omega
    L = laplacian_from(neighbors, neighbors_sizes)
    H = 1e-8 * np.eye(S) + lam * L
    A = F + H
    D = T.T @ dirty_image
    s = np.linalg.solve(A, D)
    chi = np.ascontiguousarray(data).view(np.float64) / np.ascontiguousarray(noise_map).view(np.float64)
    norm = ref.noise_normalization_complex_from(noise_map)
    logE = -0.5 * (chi @ chi - s @ D + np.linalg.slogdet(A)[1] - np.linalg.slogdet(H)[1] + norm)

    Ainv = np.linalg.inv(A)
    Hinv = np.linalg.inv(H)
    dlam = -0.5 * (s @ L @ s + np.sum(Ainv * L.T) - np.sum(Hinv * L.T))

    G = np.outer(dirty_image, s) - np.outer(omega @ s, s) - omega @ Ainv
    keep = effective_weight_mask(idx)
    rows = np.broadcast_to(np.arange(idx.shape[0])[:, None], idx.shape)
    gw = np.where(keep, G[rows, np.where(keep, idx, 0)], 0.0)
    return logE, dlam, gw
