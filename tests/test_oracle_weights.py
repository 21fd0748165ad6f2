"""The mapping-weight oracle (SIS trace, Delaunay barycentric and bilinear weights, their adjoints).

Not in the reference (it takes the mapping as an input), so the oracle is
pinned here: point location and weights against scipy.spatial.Delaunay, and
every adjoint against central finite differences, down to dlogE/dtheta_E and
dlogE/dpoints through the oracle's float64 likelihood.
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import adjoint
from oracle import mapping_weights as mw
from oracle import numpy_port as ref


@pytest.fixture(scope="module")
def mesh():
    from scipy.spatial import Delaunay

    rng = np.random.default_rng(1)
    pts = rng.uniform(-1, 1, (300, 2))
    beta = rng.uniform(-1.1, 1.1, (2000, 2))
    return pts, Delaunay(pts), beta, rng


def test_delaunay_weights_match_scipy(mesh):
    pts, tri, beta, _ = mesh
    idx, w = mw.delaunay_weights(beta, pts, tri.simplices)
    simplex = tri.find_simplex(beta)
    inside = simplex >= 0
    assert (mw.locate(beta, pts, tri.simplices) >= 0).tolist() == inside.tolist()
    np.testing.assert_array_equal(idx[inside], tri.simplices[simplex[inside]])
    Tm = tri.transform[simplex[inside]]
    b2 = np.einsum("nij,nj->ni", Tm[:, :2, :], beta[inside] - Tm[:, 2, :])
    np.testing.assert_allclose(w[inside], np.concatenate([b2, 1 - b2.sum(1, keepdims=True)], 1), rtol=0, atol=1e-13)
    np.testing.assert_allclose(w.sum(axis=1), 1.0, rtol=0, atol=1e-14)
    out = ~inside
    d2 = ((beta[out, None, :] - pts[None]) ** 2).sum(-1)
    np.testing.assert_array_equal(idx[out, 0], d2.argmin(1))
    assert (idx[out, 1:] == -1).all() and (w[out, 0] == 1).all()


def test_delaunay_vjp_matches_finite_differences(mesh):
    pts, tri, beta, rng = mesh
    idx, w = mw.delaunay_weights(beta, pts, tri.simplices)
    G = rng.standard_normal(w.shape)
    gP, gB = mw.delaunay_weights_vjp(beta, pts, idx, G)

    def L(P, B):
        i, ww = mw.delaunay_weights(B, P, tri.simplices)
        assert (i == idx).all()
        return (G * ww).sum()

    h = 1e-6
    for _ in range(8):
        s, d = rng.integers(pts.shape[0]), rng.integers(2)
        P1, P2 = pts.copy(), pts.copy()
        P1[s, d] += h
        P2[s, d] -= h
        fd = (L(P1, beta) - L(P2, beta)) / (2 * h)
        assert abs(fd - gP[s, d]) <= 1e-7 * max(1.0, abs(fd))
        m, d = rng.integers(beta.shape[0]), rng.integers(2)
        B1, B2 = beta.copy(), beta.copy()
        B1[m, d] += h
        B2[m, d] -= h
        fd = (L(pts, B1) - L(pts, B2)) / (2 * h)
        assert abs(fd - gB[m, d]) <= 1e-7 * max(1.0, abs(fd))


def test_bilinear_weights_and_vjp(mesh):
    from autojax_gb300 import synthetic

    _, _, beta, rng = mesh
    n, hw = 16, 1.2
    idx, w = mw.bilinear_weights(beta, n, hw)
    i2, w2, _ = synthetic.bilinear_mesh(beta, n, hw)
    np.testing.assert_array_equal(idx, i2)
    np.testing.assert_array_equal(w, w2)
    G = rng.standard_normal(w.shape)
    gB = mw.bilinear_weights_vjp(beta, n, hw, G)
    h = 1e-6
    for _ in range(10):
        m, d = rng.integers(beta.shape[0]), rng.integers(2)
        B1, B2 = beta.copy(), beta.copy()
        B1[m, d] += h
        B2[m, d] -= h
        fd = ((G * mw.bilinear_weights(B1, n, hw)[1]).sum() - (G * mw.bilinear_weights(B2, n, hw)[1]).sum()) / (2 * h)
        assert abs(fd - gB[m, d]) <= 1e-7 * max(1.0, abs(fd))


def lensed_problem(seed=3, S=90, K=300):
    """A small Delaunay-mapped dataset: image grid, visibilities, w_tilde, and source points taken
    from the grid traced at theta_E = 0.8" (jittered), with their triangulation and neighbours."""
    from autojax_gb300 import synthetic
    from autojax_gb300.lensing import triangulate

    d = synthetic.make_dataset("cfg1", K=K, seed=seed)
    theta = d["grid_radians_slim"] / synthetic.ARCSEC
    rng = np.random.default_rng(seed)
    beta0 = mw.sis_trace(theta, 0.8)
    pts = beta0[rng.choice(beta0.shape[0], S, replace=False)] + 1e-3 * rng.standard_normal((S, 2))
    simplices, nb, nsz = triangulate(pts)
    W = ref.w_tilde_curvature_interferometer_from(d["noise_map_real"], d["uv_wavelengths"], d["grid_radians_slim"])
    return d, theta, pts, simplices, nb, nsz, W


def oracle_chain(d, theta, pts, simplices, nb, nsz, W, theta_e, coef):
    """logE and its gradients in (theta_E, points) through the oracle's weights and adjoint."""
    beta = mw.sis_trace(theta, theta_e)
    idx, w = mw.delaunay_weights(beta, pts, simplices)
    logE, dlam, gw = adjoint.log_evidence_and_grad(d["dirty_image"], d["data"], d["noise_map"], W, idx, w, nb, nsz,
                                                   coefficient=coef)
    gP, gB = mw.delaunay_weights_vjp(beta, pts, idx, gw)
    return logE, mw.sis_trace_vjp(theta, theta_e, gB), gP, dlam, idx


def test_lens_parameter_gradients_match_finite_differences():
    d, theta, pts, simplices, nb, nsz, W = lensed_problem()
    te, coef = 0.8, 0.7
    logE, g_te, gP, _, idx = oracle_chain(d, theta, pts, simplices, nb, nsz, W, te, coef)
    # small enough that no pixel changes triangle (a pixel at the hull edge jumps from its
    # nearest vertex to barycentric weights at 1e-5 here); FD rounding ~1e-9 |logE| / h
    h = 1e-6
    lp = oracle_chain(d, theta, pts, simplices, nb, nsz, W, te + h, coef)
    lm = oracle_chain(d, theta, pts, simplices, nb, nsz, W, te - h, coef)
    assert (lp[4] == idx).all() and (lm[4] == idx).all()  # no pixel crosses an edge within the step
    fd = (lp[0] - lm[0]) / (2 * h)
    assert abs(fd - g_te) <= 1e-5 * abs(fd) + 2e-3, (fd, g_te)
    rng = np.random.default_rng(4)
    for _ in range(4):
        s, k = rng.integers(pts.shape[0]), rng.integers(2)
        P1, P2 = pts.copy(), pts.copy()
        P1[s, k] += h
        P2[s, k] -= h
        a = oracle_chain(d, theta, P1, simplices, nb, nsz, W, te, coef)
        b = oracle_chain(d, theta, P2, simplices, nb, nsz, W, te, coef)
        if not ((a[4] == idx).all() and (b[4] == idx).all()):
            continue
        fd = (a[0] - b[0]) / (2 * h)
        assert abs(fd - gP[s, k]) <= 1e-5 * abs(fd) + 2e-3, (s, k, fd, gP[s, k])
