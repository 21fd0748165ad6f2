"""The GPU mapping-weight builder and lens-parameter gradients against the oracle.

Point location and weights use the oracle's float64 operations in the same
order (no contraction), so indices and weights are compared exactly; the
adjoints accumulate with atomics and are compared at 1e-12 of their scale.
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import mapping_weights as mw

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lensing():
    from autojax_gb300 import lensing

    return lensing


@pytest.mark.parametrize("S,M", [(3, 50), (300, 2000), (3000, 5000)])
def test_delaunay_weights_match_oracle(lensing, S, M):
    from scipy.spatial import Delaunay

    rng = np.random.default_rng(S)
    pts = rng.uniform(-1, 1, (S, 2))
    tri = Delaunay(pts).simplices.astype(np.int64)  # S = 3000 gives > 4096 triangles: several staged tiles
    beta = rng.uniform(-1.1, 1.1, (M, 2))
    idx, w = lensing.delaunay_weights(beta, pts, tri)
    r_idx, r_w = mw.delaunay_weights(beta, pts, tri)
    np.testing.assert_array_equal(idx, r_idx)
    assert np.abs(w - r_w).max() <= 2.3e-16
    G = rng.standard_normal(w.shape)
    gP, gB = lensing.delaunay_weights_vjp(beta, pts, idx, G)
    r_gP, r_gB = mw.delaunay_weights_vjp(beta, pts, r_idx, G)
    np.testing.assert_allclose(gP, r_gP, rtol=0, atol=1e-12 * max(1.0, np.abs(r_gP).max()))
    np.testing.assert_allclose(gB, r_gB, rtol=0, atol=1e-12 * max(1.0, np.abs(r_gB).max()))


def test_points_on_vertices_and_edges(lensing):
    """Grid points on a regular triangulation's vertices and shared edges: the first containing
    triangle wins on both sides."""
    from scipy.spatial import Delaunay

    g = np.linspace(-1, 1, 9)
    pts = np.stack(np.meshgrid(g, g, indexing="ij"), -1).reshape(-1, 2)
    tri = Delaunay(pts).simplices.astype(np.int64)
    h = np.linspace(-1, 1, 33)
    beta = np.stack(np.meshgrid(h, h, indexing="ij"), -1).reshape(-1, 2)
    idx, w = lensing.delaunay_weights(beta, pts, tri)
    r_idx, r_w = mw.delaunay_weights(beta, pts, tri)
    np.testing.assert_array_equal(idx, r_idx)
    np.testing.assert_array_equal(w, r_w)


def test_sis_trace_and_bilinear_match_oracle(lensing):
    rng = np.random.default_rng(2)
    theta = rng.uniform(-2, 2, (3000, 2))
    beta = lensing.sis_trace(theta, 0.8)
    np.testing.assert_allclose(beta, mw.sis_trace(theta, 0.8), rtol=4e-16, atol=4e-16)
    gB = rng.standard_normal(beta.shape)
    assert abs(lensing.sis_trace_vjp(theta, gB) - mw.sis_trace_vjp(theta, 0.8, gB)) <= 1e-12 * np.abs(gB).sum()
    idx, w = lensing.bilinear_weights(beta, 16, 1.3)
    r_idx, r_w = mw.bilinear_weights(beta, 16, 1.3)
    np.testing.assert_array_equal(idx, r_idx)
    np.testing.assert_array_equal(w, r_w)
    G = rng.standard_normal(w.shape)
    np.testing.assert_allclose(lensing.bilinear_weights_vjp(beta, 16, 1.3, G), mw.bilinear_weights_vjp(beta, 16, 1.3, G),
                               rtol=1e-14, atol=1e-14)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_lensed_evidence_gradients_match_oracle(lensing, precision):
    import torch

    from test_oracle_weights import lensed_problem, oracle_chain

    from autojax_gb300.inversion import Dataset

    d, theta, pts, simplices, nb, nsz, W = lensed_problem()
    ds = Dataset(d["dirty_image"], d["data"], d["noise_map"], W, precision=precision)
    le = lensing.LensedEvidence(ds, theta, pts)
    assert le.S == pts.shape[0]
    np.testing.assert_array_equal(le.simplices.cpu().numpy(), simplices)
    for te, coef in ((0.8, 0.7), (0.75, 2.0)):
        logE, g_te, gP, dlam = le.evaluate(te, pts, coef)
        r = oracle_chain(d, theta, pts, simplices, nb, nsz, W, te, coef)
        tol = 1e-10 if precision == "fp64" else 1e-8
        assert abs(logE - r[0]) <= tol * abs(r[0]), (logE, r[0])
        gtol = 1e-7 if precision == "fp64" else 1e-5
        assert abs(g_te - r[1]) <= gtol * max(1.0, abs(r[1])), (g_te, r[1])
        np.testing.assert_allclose(gP, r[2], rtol=0, atol=gtol * np.abs(r[2]).max())
    # the same through a captured graph and through autograd
    le.capture()
    te = torch.tensor(0.78, dtype=torch.float64, device="cuda", requires_grad=True)
    P = torch.tensor(pts, device="cuda", requires_grad=True)
    c = torch.tensor(1.1, dtype=torch.float64, device="cuda", requires_grad=True)
    out = lensing.LensedLogEvidenceFunction.apply(te, P, c, le)
    out.backward()
    r = oracle_chain(d, theta, pts, simplices, nb, nsz, W, 0.78, 1.1)
    tol = 1e-10 if precision == "fp64" else 1e-8
    assert abs(float(out) - r[0]) <= tol * abs(r[0])
    gtol = 1e-7 if precision == "fp64" else 1e-5
    assert abs(float(te.grad) - r[1]) <= gtol * max(1.0, abs(r[1]))
    np.testing.assert_allclose(P.grad.cpu().numpy(), r[2], rtol=0, atol=gtol * np.abs(r[2]).max())
    assert abs(float(c.grad) - 2 * 1.1 * r[3]) <= 1e-5 * abs(2 * 1.1 * r[3]) + 1e-6 * pts.shape[0] / 1.21
