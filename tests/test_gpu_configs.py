"""Parity at the benchmark sizes, against the oracle on the same inputs.

Two configurations: K = 1e5 visibilities with M = 5,024 image pixels and S = 1,000
Delaunay source pixels (80 x 80 at 0.05", r = 2"), and K = 1e6 with M = 9,504 and
S = 1,500 (100 x 100 at 0.04", r = 2.4").  Every size exercises the multi-chunk
gathers (M > 1,024) and the multi-panel factorisations (S > 1,024 at K = 1e6).

* w_tilde (numba.py:156-207): the GPU's float64 W~ (compact table + expansion at
  full K) on sampled entries against the oracle's sum over every visibility; the
  direct builds (float64 and mixed) on a visibility sample against each other and
  against the oracle.
* F (numba.py:410-435), D (numba.py:380-406), s (numba.py:699-731) and logE
  (numba.py:761-857) with its adjoint: both sides take the GPU's float64 W~ (the
  oracle's own M x M sum over 1e6 visibilities would take hours on the host).

Tolerances: float64 path rel 1e-10 (entries that cancel judged against 1e-11 of
the result's scale); logE where A is so ill-conditioned (cond ~1e13 at lambda =
1e-3) that equally valid float64 evaluations already disagree by more than
that (F summed in another order, LU or Cholesky), within twice their spread; s
against cond(A) as in the golden solve test; the mixed path as each test states.
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import adjoint
from oracle import numpy_port as ref

pytestmark = pytest.mark.gpu

RTOL = 1e-10
ATOL_FRAC = 1e-11
LAMBDAS = (1e-3, 1e3)


@pytest.fixture(scope="module", params=["cfg2", "cfg3"])
def cfg(request):
    import torch

    import autojax_gb300 as aj
    from autojax_gb300 import synthetic

    d = synthetic.make_dataset(request.param)
    dev = torch.device("cuda", 0)
    n = torch.from_numpy(d["noise_map_real"]).to(dev)
    uv = torch.from_numpy(d["uv_wavelengths"]).to(dev)
    wc = aj.w_compact_curvature_interferometer_from(d["grid_size"], n, uv, d["pixel_scale"])
    Wd = aj.w_tilde_via_compact_from(wc, torch.from_numpy(d["native_index_for_slim_index"]).to(dev))
    W = Wd.cpu().numpy()
    T = ref.mapping_matrix_from(d["pix_indexes_for_sub_slim_index"], d["pix_weights_for_sub_slim_index"], d["S"])
    yield {"d": d, "W": W, "Wd": Wd, "T": T}
    del Wd
    torch.cuda.empty_cache()


def _args(d, W):
    return (d["dirty_image"], d["data"], d["noise_map"], W, d["pix_indexes_for_sub_slim_index"],
            d["pix_weights_for_sub_slim_index"], d["neighbors"], d["neighbors_sizes"])


def _entries(M, seed=0):
    rng = np.random.default_rng(seed)
    rows = np.repeat(np.array([0, M // 3, M // 2, M - 1]), 48)
    cols = rng.integers(0, M, rows.size)
    cols[::48] = rows[::48]  # the diagonal too
    return rows, cols


def test_w_tilde_full_k_entries_match_oracle(cfg):
    d, W = cfg["d"], cfg["W"]
    rows, cols = _entries(d["M"])
    exp = ref.w_tilde_entries(d["noise_map_real"], d["uv_wavelengths"], d["grid_radians_slim"], rows, cols)
    scale = float(np.abs(np.diag(W)).max())
    np.testing.assert_allclose(W[rows, cols], exp, rtol=RTOL, atol=ATOL_FRAC * scale)
    assert np.array_equal(W, W.T)


def test_direct_w_tilde_builds_match_oracle(cfg):
    """The direct builds at the configuration's M on a 4,096-visibility sample."""
    import autojax_gb300 as aj

    d = cfg["d"]
    Ks = 4096
    n, uv, g = d["noise_map_real"][:Ks].copy(), d["uv_wavelengths"][:Ks].copy(), d["grid_radians_slim"]
    W64 = aj.w_tilde_curvature_interferometer_from(n, uv, g)
    Wmx, P = aj.w_tilde_curvature_interferometer_from(n, uv, g, precision="mixed", planes=True)
    rows, cols = _entries(d["M"], seed=1)
    exp = ref.w_tilde_entries(n, uv, g, rows, cols)
    scale = float(np.abs(np.diag(W64)).max())
    np.testing.assert_allclose(W64[rows, cols], exp, rtol=RTOL, atol=ATOL_FRAC * scale)
    # mixed: ~1e-12 of the scale (float64 panel, exact digit products or double-float sums)
    np.testing.assert_allclose(Wmx, W64, rtol=0, atol=1e-12 * scale)
    np.testing.assert_allclose(Wmx[rows, cols], exp, rtol=0, atol=1e-12 * scale)
    np.testing.assert_allclose(P[0].astype(np.float64) + P[1].astype(np.float64), Wmx, rtol=0, atol=1e-15 * scale)


def test_fp64_products_match_oracle(cfg):
    import torch

    import autojax_gb300 as aj

    d, W, T = cfg["d"], cfg["W"], cfg["T"]
    dev = cfg["Wd"].device
    idx = torch.from_numpy(d["pix_indexes_for_sub_slim_index"]).to(dev)
    w = torch.from_numpy(d["pix_weights_for_sub_slim_index"]).to(dev)
    F = aj.curvature_matrix_via_w_wilde_sparse_mapping_matrix_from(cfg["Wd"], idx, w, d["S"]).cpu().numpy()
    F_ref = ref.curvature_matrix_via_w_tilde_from(W, T)
    np.testing.assert_allclose(F, F_ref, rtol=RTOL, atol=ATOL_FRAC * np.abs(F_ref).max())
    D = aj.data_vector_from(T, d["dirty_image"])
    D_ref = ref.data_vector_from(T, d["dirty_image"])
    np.testing.assert_allclose(D, D_ref, rtol=RTOL, atol=ATOL_FRAC * np.abs(D_ref).max())
    Tg = aj.mapping_matrix_from(d["pix_indexes_for_sub_slim_index"], d["pix_weights_for_sub_slim_index"], d["S"])
    np.testing.assert_array_equal(Tg, T)


@pytest.mark.parametrize("lam", LAMBDAS)
def test_fp64_solve_matches_oracle(cfg, lam):
    import autojax_gb300 as aj

    d, W, T = cfg["d"], cfg["W"], cfg["T"]
    H = ref.constant_regularization_matrix_from(np.sqrt(lam), d["neighbors"], d["neighbors_sizes"])
    A = ref.curvature_matrix_via_w_tilde_from(W, T) + H
    D = ref.data_vector_from(T, d["dirty_image"])
    s = aj.reconstruction_positive_negative_from(D, A)
    exp = ref.reconstruction_positive_negative_from(D, A)
    ev = np.linalg.eigvalsh(A)
    cond = ev[-1] / ev[0]
    err = np.linalg.norm(s - exp) / np.linalg.norm(exp)
    assert err <= max(1e-13, 1e-15 * cond), (err, cond)
    res = np.linalg.norm(A @ s - D) / (np.linalg.norm(A) * np.linalg.norm(s))
    assert res < 1e-13, res


def _fp64_spread(d, W, T, H, D):
    """How far apart equally valid float64 evaluations of the same logE land at A's conditioning:
    F = T^T W T as dense products, as the reference's sparse products (another summation order)
    and symmetrised, each with LAPACK's LU (the reference's slogdet/solve); and the dense F with
    a Cholesky.  Returns (max - min, the dense-LU value)."""
    import scipy.linalg as sl

    F_dense = ref.curvature_matrix_via_w_tilde_from(W, T)
    F_sparse = ref.curvature_matrix_via_w_wilde_sparse_mapping_matrix_from(
        W, d["pix_indexes_for_sub_slim_index"], d["pix_weights_for_sub_slim_index"], T.shape[1])
    vals = [ref._evidence(d["noise_map"], d["data"], F, H, D)
            for F in (F_dense, F_sparse, 0.5 * (F_dense + F_dense.T))]
    ca = sl.cho_factor(F_dense + H, lower=True)
    ch = sl.cho_factor(H, lower=True)
    s = sl.cho_solve(ca, D)
    chi = np.ascontiguousarray(d["data"]).view(np.float64) / np.ascontiguousarray(d["noise_map"]).view(np.float64)
    vals.append(-0.5 * (chi @ chi - s @ D + 2 * np.log(np.diag(ca[0])).sum() - 2 * np.log(np.diag(ch[0])).sum()
                        + ref.noise_normalization_complex_from(d["noise_map"])))
    return max(vals) - min(vals), vals[0]


@pytest.mark.parametrize("lam", LAMBDAS)
def test_fp64_log_evidence_matches_oracle(cfg, lam):
    """logE at rel 1e-10, or, where A's conditioning puts equally valid float64 evaluations further
    apart than that (cond ~1e13 at lambda = 1e-3: F's summation order alone moves logE by ~3e-10),
    within twice their spread."""
    import autojax_gb300 as aj

    d = cfg["d"]
    c = float(np.sqrt(lam))
    logE, dlam, gw, s = aj.log_evidence_and_grad(*_args(d, cfg["Wd"]), coefficient=c, precision="fp64",
                                                  return_reconstruction=True)
    logE, dlam, gw, s = float(logE), float(dlam), gw.cpu().numpy(), s.cpu().numpy()
    a = _args(d, cfg["W"])
    r_logE, r_dlam, r_gw = adjoint.log_evidence_and_grad(*a, coefficient=c)
    H = ref.constant_regularization_matrix_from(c, d["neighbors"], d["neighbors_sizes"])
    F = ref.curvature_matrix_via_w_tilde_from(cfg["W"], cfg["T"])
    D = ref.data_vector_from(cfg["T"], d["dirty_image"])
    spread, _ = _fp64_spread(d, cfg["W"], cfg["T"], H, D)
    tol = max(RTOL * abs(r_logE), 2.0 * spread)
    assert abs(logE - r_logE) <= tol, (logE, r_logE, tol)
    plain = ref.log_likelihood_function_via_w_tilde_from(*a, coefficient=c)
    assert abs(logE - plain) <= tol, (logE, plain)
    # s, dlogE/dlambda and the weight gradient go through A^-1: judged against cond(A)
    A = F + H
    ev = np.linalg.eigvalsh(A)
    cond = ev[-1] / ev[0]
    s_ref = np.linalg.solve(A, D)
    assert np.linalg.norm(s - s_ref) / np.linalg.norm(s_ref) <= max(1e-13, 1e-15 * cond)
    trace_scale = d["S"] / lam
    assert abs(dlam - r_dlam) <= max(1e-10, 1e-15 * cond) * trace_scale + 1e-8 * abs(r_dlam), (dlam, r_dlam)
    np.testing.assert_allclose(gw, r_gw, rtol=0, atol=max(1e-9, 1e-15 * cond) * np.abs(r_gw).max())


@pytest.mark.parametrize("lam", LAMBDAS)
def test_mixed_matches_oracle(cfg, lam):
    """The mixed path against the float64 oracle on the same W~.

    Stated tolerances: logE rel 1e-7 (the target is 1e-6); F 1e-12 of its scale
    (double-float gathers, ~2^-47 a term); s against cond(A) at double-float
    rounding (2^-47 cond); the weight gradient as in the small-case mixed
    tests; dlogE/dlambda as there, or within ten times the movement of the
    oracle's own value under a double-float-sized perturbation of A, whichever
    is larger (the backward-error bound of a double-float evaluation).
    """
    import torch

    import autojax_gb300 as aj

    d, W, T = cfg["d"], cfg["W"], cfg["T"]
    c = float(np.sqrt(lam))
    logE, dlam, gw, s = aj.log_evidence_and_grad(*_args(d, cfg["Wd"]), coefficient=c, precision="mixed",
                                                  return_reconstruction=True)
    logE, dlam, gw, s = float(logE), float(dlam), gw.cpu().numpy(), s.cpu().numpy()
    r_logE, r_dlam, r_gw = adjoint.log_evidence_and_grad(*_args(d, W), coefficient=c)
    assert abs(logE - r_logE) <= 1e-7 * abs(r_logE), (logE, r_logE, abs(logE - r_logE) / abs(r_logE))
    dev = cfg["Wd"].device
    F = aj.curvature_matrix_via_w_wilde_sparse_mapping_matrix_from(
        cfg["Wd"], torch.from_numpy(d["pix_indexes_for_sub_slim_index"]).to(dev),
        torch.from_numpy(d["pix_weights_for_sub_slim_index"]).to(dev), d["S"], precision="mixed").cpu().numpy()
    F_ref = ref.curvature_matrix_via_w_tilde_from(W, T)
    np.testing.assert_allclose(F, F_ref, rtol=0, atol=1e-12 * np.abs(F_ref).max())
    H = ref.constant_regularization_matrix_from(c, d["neighbors"], d["neighbors_sizes"])
    A = F_ref + H
    ev = np.linalg.eigvalsh(A)
    cond = ev[-1] / ev[0]
    s_ref = np.linalg.solve(A, ref.data_vector_from(T, d["dirty_image"]))
    assert np.linalg.norm(s - s_ref) / np.linalg.norm(s_ref) <= max(1e-10, 2.0**-47 * cond)
    # dlogE/dlambda = -1/2 [s^T L s + tr(A^-1 L) - tr(H^-1 L)]: at cond(A) ~1e14 (lambda = 1e-3)
    # tr(A^-1 L) itself moves when A is perturbed at double-float rounding (2^-47 |A|), so the
    # bound is also ten times that movement of the oracle's own value
    L = adjoint.laplacian_from(d["neighbors"], d["neighbors_sizes"])
    rng = np.random.default_rng(0)
    E = rng.standard_normal(A.shape) * (2.0**-47 * np.abs(A))
    Ap = A + 0.5 * (E + E.T)
    sp = np.linalg.solve(Ap, ref.data_vector_from(T, d["dirty_image"]))
    moved = abs(-0.5 * (sp @ L @ sp + np.sum(np.linalg.inv(Ap) * L.T) - np.sum(np.linalg.inv(H) * L.T)) - r_dlam)
    trace_scale = d["S"] / lam
    tol_lam = max(1e-6 * trace_scale + 1e-5 * abs(r_dlam), 10.0 * moved)
    assert abs(dlam - r_dlam) <= tol_lam, (dlam, r_dlam, tol_lam)
    np.testing.assert_allclose(gw, r_gw, rtol=0, atol=max(1e-5, 2e-15 * cond) * np.abs(r_gw).max())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_compact_table_route_matches_at_size(cfg, precision):
    """The low-memory route (F from the N x (2N-1) offset table, W~ never stored; numba.py:439-653,
    866-967) against the dense-W~ route on the same table, at the configuration's M."""
    import torch

    import autojax_gb300 as aj

    d = cfg["d"]
    dev = cfg["Wd"].device
    n = torch.from_numpy(d["noise_map_real"]).to(dev)
    uv = torch.from_numpy(d["uv_wavelengths"]).to(dev)
    wc = aj.w_compact_curvature_interferometer_from(d["grid_size"], n, uv, d["pixel_scale"])
    nat = torch.from_numpy(d["native_index_for_slim_index"]).to(dev)
    a = _args(d, cfg["Wd"])
    c = 1.0
    dense = float(aj.log_likelihood_function_via_w_tilde_from(*a, coefficient=c, precision=precision))
    compact = float(aj.log_likelihood_function_via_w_compact_from(a[0], a[1], a[2], wc, nat, *a[4:], coefficient=c,
                                                                  precision=precision))
    tol = 1e-10 if precision == "fp64" else 1e-8
    assert abs(compact - dense) <= tol * abs(dense), (compact, dense)
    exp = ref.log_likelihood_function_via_w_tilde_from(*_args(d, cfg["W"]), coefficient=c)
    assert abs(compact - exp) <= (1e-10 if precision == "fp64" else 1e-7) * abs(exp), (compact, exp)


def _cond_at(cfg, coef):
    d, W, T = cfg["d"], cfg["W"], cfg["T"]
    H = ref.constant_regularization_matrix_from(coef, d["neighbors"], d["neighbors_sizes"])
    ev = np.linalg.eigvalsh(ref.curvature_matrix_via_w_tilde_from(W, T) + H)
    return ev[-1] / ev[0]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_compact_route_gradients_match_dense(cfg, precision):
    """The gradient from the compact table (W~ never stored: F and Omega = W~ T gathered from the
    N x (2N - 1) table) against the dense-W~ gradient, at the configuration's sizes."""
    import torch

    import autojax_gb300 as aj

    d = cfg["d"]
    dev = cfg["Wd"].device
    wc = aj.w_compact_curvature_interferometer_from(d["grid_size"], torch.from_numpy(d["noise_map_real"]).to(dev),
                                                    torch.from_numpy(d["uv_wavelengths"]).to(dev), d["pixel_scale"])
    nat = torch.from_numpy(d["native_index_for_slim_index"]).to(dev)
    a = _args(d, cfg["Wd"])
    dense = aj.log_evidence_and_grad(*a, coefficient=1.0, precision=precision)
    compact = aj.log_evidence_and_grad(*a[:3], None, *a[4:], coefficient=1.0, precision=precision, w_compact=wc,
                                       native_index_for_slim_index=nat)
    cond = _cond_at(cfg, 1.0)
    tol = 1e-10 if precision == "fp64" else 1e-8
    assert abs(float(compact[0]) - float(dense[0])) <= tol * abs(float(dense[0]))
    assert abs(float(compact[1]) - float(dense[1])) <= max(1e-8, 1e-15 * cond) * d["S"] + 1e-6 * abs(float(dense[1]))
    g_c, g_d = compact[2].cpu().numpy(), dense[2].cpu().numpy()
    np.testing.assert_allclose(g_c, g_d, rtol=0, atol=max(1e-8, 2e-15 * cond) * np.abs(g_d).max())


def test_lens_parameter_gradients_at_size(cfg):
    """Differentiation at the configuration's sizes: logE and its gradients in the SIS Einstein radius,
    the S x 2 source-pixel positions and lambda, through the GPU weight builder and adjoint, against
    the oracle chain (oracle weights, closed-form adjoint, weight VJPs; finite-difference-checked on
    the small case)."""
    from test_oracle_weights import oracle_chain

    from autojax_gb300 import lensing, synthetic
    from autojax_gb300.inversion import Dataset
    from oracle import mapping_weights as mw

    d = cfg["d"]
    theta = d["grid_radians_slim"] / synthetic.ARCSEC
    rng = np.random.default_rng(9)
    beta0 = mw.sis_trace(theta, 0.8)
    pts = beta0[rng.choice(beta0.shape[0], d["S"], replace=False)] + 1e-3 * rng.standard_normal((d["S"], 2))
    simplices, nb, nsz = lensing.triangulate(pts)
    r = oracle_chain(d, theta, pts, simplices, nb, nsz, cfg["W"], 0.8, 1.0)
    T = ref.mapping_matrix_from(r[4], mw.delaunay_weights(mw.sis_trace(theta, 0.8), pts, simplices)[1], d["S"])
    H = ref.constant_regularization_matrix_from(1.0, nb, nsz)
    ev = np.linalg.eigvalsh(ref.curvature_matrix_via_w_tilde_from(cfg["W"], T) + H)
    cond = ev[-1] / ev[0]
    for precision in ("fp64", "mixed"):
        ds = Dataset(d["dirty_image"], d["data"], d["noise_map"], cfg["Wd"], precision=precision)
        le = lensing.LensedEvidence(ds, theta, pts)
        logE, g_te, gP, dlam = le.evaluate(0.8, pts, 1.0)
        tol = 1e-10 if precision == "fp64" else 1e-8
        assert abs(logE - r[0]) <= tol * abs(r[0]), (precision, logE, r[0])
        gtol = max(1e-7 if precision == "fp64" else 1e-5, 2e-15 * cond)
        assert abs(g_te - r[1]) <= gtol * max(1.0, abs(r[1])), (precision, g_te, r[1])
        np.testing.assert_allclose(gP, r[2], rtol=0, atol=gtol * np.abs(r[2]).max())
        assert abs(dlam - r[3]) <= 1e-6 * d["S"] + gtol * abs(r[3]), (precision, dlam, r[3])
