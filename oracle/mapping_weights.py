"""NumPy restatement of the mapping-weight builder and its adjoint (test oracle).

Test infrastructure, like the rest of ``oracle/``: only tests and the bench's
CPU leg use it.  The reference takes the mapping (``pix_indexes``,
``pix_weights``) as an input of its likelihood (numba.py:294-376,
761-857); the weights themselves come from PyAutoLens, which the reference
does not vendor (``external/get_dataset.py:5,30-60``).  So this module is
written from the mathematics, not pinned to reference outputs ("parity
unpinned"); the tests pin it with central finite differences and against
``scipy.spatial.Delaunay``.

* SIS deflection: beta = theta - theta_E theta / |theta| (arcsec), lens at the origin.
* Delaunay barycentric weights: with cross(u, v) = u_x v_y - u_y v_x, a triangle
  (a, b, c) and a point x, D = cross(b - a, c - a), N_a = cross(b - x, c - x),
  N_b = cross(c - x, a - x), N_c = cross(a - x, b - x); w_j = N_j / D.  A point
  lies in the first triangle (lowest index) whose N_j all share D's sign (or
  are zero); outside the hull it maps to its nearest vertex with weight 1 and
  the row is -1 padded.
* Bilinear weights on an n x n rectangular mesh over [-hw, hw]^2, rows growing
  downwards in y: the four corners of the cell, weights (1-ty)(1-tx), (1-ty)tx,
  ty(1-tx), ty tx.
"""

from __future__ import annotations

import numpy as np


def _cross(u, v):
    return u[..., 0] * v[..., 1] - u[..., 1] * v[..., 0]


def sis_trace(theta, einstein_radius):
    theta = np.asarray(theta, dtype=np.float64)
    r = np.hypot(theta[:, 0], theta[:, 1])
    return theta - einstein_radius * theta / r[:, None]


def sis_trace_vjp(theta, einstein_radius, grad_beta):
    """dL/d theta_E for dL/d beta = grad_beta (beta = sis_trace(theta, theta_E))."""
    theta = np.asarray(theta, dtype=np.float64)
    r = np.hypot(theta[:, 0], theta[:, 1])
    return float(-np.sum(grad_beta * theta / r[:, None]))


def locate(beta, points, simplices, chunk=2048):
    """Index of the first triangle containing each point, or -1 (vectorised over triangle chunks)."""
    beta = np.asarray(beta, dtype=np.float64)
    P = np.asarray(points, dtype=np.float64)
    tri = np.asarray(simplices, dtype=np.int64)
    a, b, c = P[tri[:, 0]], P[tri[:, 1]], P[tri[:, 2]]
    D = _cross(b - a, c - a)
    out = -np.ones(beta.shape[0], dtype=np.int64)
    for m0 in range(0, beta.shape[0], chunk):
        x = beta[m0 : m0 + chunk, None, :]
        na = _cross(b[None] - x, c[None] - x)
        nb = _cross(c[None] - x, a[None] - x)
        nc = _cross(a[None] - x, b[None] - x)
        s = np.sign(D)[None]
        inside = (na * s >= 0) & (nb * s >= 0) & (nc * s >= 0) & (D[None] != 0)
        hit = inside.any(axis=1)
        first = np.argmax(inside, axis=1)
        out[m0 : m0 + chunk] = np.where(hit, first, -1)
    return out


def delaunay_weights(beta, points, simplices):
    """(pix_indexes (M, 3) int64, pix_weights (M, 3) float64) of the traced points."""
    beta = np.asarray(beta, dtype=np.float64)
    P = np.asarray(points, dtype=np.float64)
    tri = np.asarray(simplices, dtype=np.int64)
    t = locate(beta, P, tri)
    M = beta.shape[0]
    idx = -np.ones((M, 3), dtype=np.int64)
    w = np.zeros((M, 3))
    ins = t >= 0
    v = tri[t[ins]]
    a, b, c = P[v[:, 0]], P[v[:, 1]], P[v[:, 2]]
    x = beta[ins]
    D = _cross(b - a, c - a)
    w[ins] = np.stack([_cross(b - x, c - x), _cross(c - x, a - x), _cross(a - x, b - x)], axis=1) / D[:, None]
    idx[ins] = v
    out = ~ins
    if out.any():
        d2 = np.square(beta[out, None, :] - P[None]).sum(axis=2)
        idx[out, 0] = np.argmin(d2, axis=1)
        w[out, 0] = 1.0
    return idx, w


def delaunay_weights_vjp(beta, points, pix_indexes, pix_weights_grad):
    """Pull dL/dw (M, 3) back to dL/d points (S, 2) and dL/d beta (M, 2).

    Rows with a -1 in position 1 (outside the hull: one vertex, weight 1) have
    no gradient.  With l = sum_j g_j N_j / D = Q / D:
    dl/dv = (dQ/dv - l dD/dv) / D.
    """
    beta = np.asarray(beta, dtype=np.float64)
    P = np.asarray(points, dtype=np.float64)
    idx = np.asarray(pix_indexes)
    G = np.asarray(pix_weights_grad, dtype=np.float64)
    gP = np.zeros_like(P)
    gB = np.zeros_like(beta)
    ins = idx[:, 1] >= 0
    v = idx[ins]
    a, b, c = P[v[:, 0]], P[v[:, 1]], P[v[:, 2]]
    x = beta[ins]
    g = G[ins]

    def du(u, vv):  # d cross(u, vv) / du
        return np.stack([vv[:, 1], -vv[:, 0]], axis=1)

    def dv(u, vv):  # d cross(u, vv) / dvv
        return np.stack([-u[:, 1], u[:, 0]], axis=1)

    D = _cross(b - a, c - a)
    Q = g[:, 0] * _cross(b - x, c - x) + g[:, 1] * _cross(c - x, a - x) + g[:, 2] * _cross(a - x, b - x)
    ell = Q / D
    dQa = g[:, 1:2] * dv(c - x, a - x) + g[:, 2:3] * du(a - x, b - x)
    dQb = g[:, 0:1] * du(b - x, c - x) + g[:, 2:3] * dv(a - x, b - x)
    dQc = g[:, 0:1] * dv(b - x, c - x) + g[:, 1:2] * du(c - x, a - x)
    dDb = du(b - a, c - a)
    dDc = dv(b - a, c - a)
    dDa = -(dDb + dDc)
    r = 1.0 / D[:, None]
    ga = (dQa - ell[:, None] * dDa) * r
    gb = (dQb - ell[:, None] * dDb) * r
    gc = (dQc - ell[:, None] * dDc) * r
    np.add.at(gP, v[:, 0], ga)
    np.add.at(gP, v[:, 1], gb)
    np.add.at(gP, v[:, 2], gc)
    gB[ins] = -(dQa + dQb + dQc) * r
    return gP, gB


def bilinear_weights(beta, n, half_width):
    """(pix_indexes (M, 4), pix_weights (M, 4)) on the n x n mesh over [-hw, hw]^2."""
    beta = np.asarray(beta, dtype=np.float64)
    h = 2.0 * half_width / (n - 1)
    fy = np.clip((half_width - beta[:, 0]) / h, 0.0, n - 1 - 1e-9)
    fx = np.clip((beta[:, 1] + half_width) / h, 0.0, n - 1 - 1e-9)
    r0 = np.floor(fy).astype(np.int64)
    c0 = np.floor(fx).astype(np.int64)
    ty = fy - r0
    tx = fx - c0
    idx = np.stack([r0 * n + c0, r0 * n + c0 + 1, (r0 + 1) * n + c0, (r0 + 1) * n + c0 + 1], axis=1)
    w = np.stack([(1 - ty) * (1 - tx), (1 - ty) * tx, ty * (1 - tx), ty * tx], axis=1)
    return idx, w


def bilinear_weights_vjp(beta, n, half_width, pix_weights_grad):
    """dL/d beta (M, 2); zero along a clipped coordinate."""
    beta = np.asarray(beta, dtype=np.float64)
    G = np.asarray(pix_weights_grad, dtype=np.float64)
    h = 2.0 * half_width / (n - 1)
    fy_raw = (half_width - beta[:, 0]) / h
    fx_raw = (beta[:, 1] + half_width) / h
    fy = np.clip(fy_raw, 0.0, n - 1 - 1e-9)
    fx = np.clip(fx_raw, 0.0, n - 1 - 1e-9)
    ty = fy - np.floor(fy)
    tx = fx - np.floor(fx)
    dty = G[:, 0] * -(1 - tx) + G[:, 1] * -tx + G[:, 2] * (1 - tx) + G[:, 3] * tx
    dtx = G[:, 0] * -(1 - ty) + G[:, 1] * (1 - ty) + G[:, 2] * -ty + G[:, 3] * ty
    free_y = (fy_raw > 0.0) & (fy_raw < n - 1 - 1e-9)
    free_x = (fx_raw > 0.0) & (fx_raw < n - 1 - 1e-9)
    gB = np.zeros_like(beta)
    gB[:, 0] = np.where(free_y, dty * (-1.0 / h), 0.0)
    gB[:, 1] = np.where(free_x, dtx * (1.0 / h), 0.0)
    return gB
