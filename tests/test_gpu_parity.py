"""FP64 parity of the CUDA path with the reference's own outputs (golden fixtures) and with the oracle.

Every call goes through the public API, which calls the C ABI of
libautojax_gb300.so.  Tolerances: rel 1e-10 for float64 results, with an
absolute floor of 1e-11 of the result's scale for entries that cancel to ~0;
integer and boolean outputs bit-exact.  The linear solve is judged against
its conditioning (see test_solve_matches_reference).
"""

from __future__ import annotations

import numpy as np
import pytest

import golden_util as gu
from oracle import adjoint
from oracle import numpy_port as ref

pytestmark = pytest.mark.gpu

RTOL = 1e-10
ATOL_FRAC = 1e-11

FUNCS = [
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
    "constant_regularization_matrix_from",
    "noise_normalization_complex_from",
    "log_likelihood_function_via_w_tilde_from",
    "log_likelihood_function_via_w_compact_from",
]
CASES = [(c, f) for c in gu.CASES for f in FUNCS if f in gu.expected_keys(c, "numba")]


@pytest.fixture(scope="module")
def aj():
    import autojax_gb300

    return autojax_gb300


@pytest.mark.parametrize("case,name", CASES, ids=[f"{c}-{f}" for c, f in CASES])
def test_matches_reference_outputs(aj, case, name):
    d = gu.full_inputs(case)
    got = gu.call(getattr(aj, name), d)
    exp = gu.expected(case, "numba__" + name)
    gu.assert_matches(got, exp, rtol=RTOL, atol_frac=ATOL_FRAC, what=f"{case}:{name}")


@pytest.mark.parametrize("case", gu.CASES)
def test_preload_matches_original(aj, case):
    d = gu.full_inputs(case)
    got = aj.w_tilde_curvature_preload_interferometer_from(
        d["noise_map_real"], d["uv_wavelengths"], d["shape_masked_pixels_2d"], d["grid_radians_2d"]
    )
    exp = gu.expected(case, "original__w_tilde_curvature_preload_interferometer_from")
    gu.assert_matches(got, exp, rtol=RTOL, atol_frac=ATOL_FRAC, what=f"{case}:preload")


@pytest.mark.parametrize("case", gu.CASES)
def test_solve_matches_reference(aj, case):
    """s = A^-1 D: forward error bounded by cond(A) * 1e-15, residual at rounding level."""
    d = gu.full_inputs(case)
    A, D = d["curvature_reg_matrix"], d["data_vector"]
    s = aj.reconstruction_positive_negative_from(D, A)
    exp = gu.expected(case, "numba__reconstruction_positive_negative_from")
    cond = np.linalg.cond(A)
    err = np.linalg.norm(s - exp) / np.linalg.norm(exp)
    assert err <= max(1e-13, 1e-15 * cond), (err, cond)
    res = np.linalg.norm(A @ s - D) / (np.linalg.norm(A) * np.linalg.norm(s))
    assert res < 1e-13, res


@pytest.mark.parametrize("case", ["cfg1", "edge"])
@pytest.mark.parametrize("coef", [0.5, 2.0])
def test_loglike_coefficient_and_gradient_match_oracle(aj, case, coef):
    d = gu.full_inputs(case)
    args = (d["dirty_image"], d["data"], d["noise_map"], d["w_tilde"], d["pix_indexes_for_sub_slim_index"],
            d["pix_weights_for_sub_slim_index"], d["neighbors"], d["neighbors_sizes"])
    logE, dlam, gw = aj.log_evidence_and_grad(*args, coefficient=coef)
    r_logE, r_dlam, r_gw = adjoint.log_evidence_and_grad(*args, coefficient=coef)
    assert abs(logE - r_logE) <= RTOL * abs(r_logE), (logE, r_logE)
    assert abs(dlam - r_dlam) <= 1e-8 * max(1.0, abs(r_dlam)), (dlam, r_dlam)
    np.testing.assert_allclose(gw, r_gw, rtol=1e-8, atol=1e-9 * np.abs(r_gw).max())
    plain = aj.log_likelihood_function_via_w_tilde_from(*args, coefficient=coef)
    assert abs(plain - r_logE) <= RTOL * abs(r_logE)


@pytest.mark.parametrize("case", ["cfg1", "edge"])
def test_reference_coefficient_goldens(aj, case):
    d = gu.full_inputs(case)
    for key in gu.expected_keys(case, "numba"):
        if not key.startswith("log_likelihood_coefficient_"):
            continue
        coef = float(key.rsplit("_", 1)[1])
        got = aj.log_likelihood_function_via_w_tilde_from(
            d["dirty_image"], d["data"], d["noise_map"], d["w_tilde"], d["pix_indexes_for_sub_slim_index"],
            d["pix_weights_for_sub_slim_index"], d["neighbors"], d["neighbors_sizes"], coefficient=coef)
        exp = float(gu.expected(case, "numba__" + key))
        assert abs(got - exp) <= RTOL * abs(exp), (coef, got, exp)


def test_compact_gradient_matches_oracle_without_repeats(aj):
    d = gu.full_inputs("cfg1")
    args_c = (d["dirty_image"], d["data"], d["noise_map"], None, d["pix_indexes_for_sub_slim_index"],
              d["pix_weights_for_sub_slim_index"], d["neighbors"], d["neighbors_sizes"])
    logE, dlam, gw = aj.log_evidence_and_grad(*args_c, coefficient=1.3, w_compact=d["w_compact"],
                                              native_index_for_slim_index=d["native_index_for_slim_index"])
    r = adjoint.log_evidence_and_grad(d["dirty_image"], d["data"], d["noise_map"], d["w_tilde"],
                                      d["pix_indexes_for_sub_slim_index"], d["pix_weights_for_sub_slim_index"],
                                      d["neighbors"], d["neighbors_sizes"], coefficient=1.3)
    assert abs(logE - r[0]) <= 1e-9 * abs(r[0])
    assert abs(dlam - r[1]) <= 1e-7 * max(1.0, abs(r[1]))
    np.testing.assert_allclose(gw, r[2], rtol=1e-7, atol=1e-8 * np.abs(r[2]).max())


def test_torch_in_torch_out_stays_on_device(aj):
    import torch

    d = gu.full_inputs("cfg1")
    idx = torch.from_numpy(d["pix_indexes_for_sub_slim_index"]).cuda()
    w = torch.from_numpy(d["pix_weights_for_sub_slim_index"]).cuda()
    T = aj.mapping_matrix_from(idx, w, d["pixels"])
    assert isinstance(T, torch.Tensor) and T.is_cuda and T.dtype == torch.float64
    np.testing.assert_array_equal(T.cpu().numpy(), ref.mapping_matrix_from(d["pix_indexes_for_sub_slim_index"],
                                                                          d["pix_weights_for_sub_slim_index"],
                                                                          d["pixels"]))


def test_slim_from_mask_matches_argwhere(aj):
    d = gu.full_inputs("refgen")
    mask = ref.mask_2d_circular_from((30, 30), (0.2, 0.2), 3.0, (0.0, 0.0))
    nat, gs = aj.slim_from_mask(mask, d["grid_radians_2d"])
    np.testing.assert_array_equal(nat, np.argwhere(~mask))
    np.testing.assert_array_equal(gs, d["grid_radians_2d"][~mask])


# ------------------------------------------------------------- edge cases


def test_index_out_of_range_raises(aj):
    idx = np.array([[0, 1, 5]], dtype=np.int64)
    with pytest.raises(IndexError):
        aj.mapping_matrix_from(idx, np.ones((1, 3)), 4)
    nb = np.array([[1, -1], [7, -1]], dtype=np.int64)
    with pytest.raises(IndexError):
        aj.constant_regularization_matrix_from(1.0, nb, np.array([1, 1], dtype=np.int64))


def test_indefinite_solves_and_singular_raises(aj):
    """As np.linalg.solve (numba.py:731): an indefinite non-singular A is solved (by the LU
    fallback), a singular one raises LinAlgError."""
    A = np.array([[1.0, 2.0], [2.0, 1.0]])
    np.testing.assert_allclose(aj.reconstruction_positive_negative_from(np.ones(2), A),
                               np.linalg.solve(A, np.ones(2)), rtol=1e-14)
    with pytest.raises(np.linalg.LinAlgError):
        aj.reconstruction_positive_negative_from(np.ones(2), np.array([[1.0, 2.0], [2.0, 4.0]]))


def test_empty_visibilities_give_zero_w_tilde(aj):
    g = np.random.default_rng(0).standard_normal((7, 2)) * 1e-5
    W = aj.w_tilde_curvature_interferometer_from(np.zeros(0), np.zeros((0, 2)), g)
    np.testing.assert_array_equal(W, np.zeros((7, 7)))
    wc = aj.w_compact_curvature_interferometer_from(5, np.zeros(0), np.zeros((0, 2)), 0.1)
    np.testing.assert_array_equal(wc, np.zeros((5, 9)))


def test_all_rows_empty_mapping(aj):
    idx = -np.ones((6, 3), dtype=np.int64)
    T = aj.mapping_matrix_from(idx, np.ones((6, 3)), 5)
    np.testing.assert_array_equal(T, np.zeros((6, 5)))
    X = np.random.default_rng(1).standard_normal((6, 4))
    np.testing.assert_array_equal(aj.sparse_mapping_matrix_transpose_matmul(X, idx, np.ones((6, 3)), 5), np.zeros((5, 4)))


@pytest.mark.parametrize("M,K", [(1, 3), (33, 65), (129, 1)])
def test_w_tilde_odd_sizes_match_oracle(aj, M, K):
    rng = np.random.default_rng(M * 1000 + K)
    g = rng.standard_normal((M, 2)) * 1e-5
    uv = rng.uniform(-5e5, 5e5, (K, 2))
    n = rng.uniform(0.1, 1.0, K)
    got = aj.w_tilde_curvature_interferometer_from(n, uv, g)
    exp = ref.w_tilde_curvature_interferometer_from(n, uv, g)
    gu.assert_matches(got, exp, rtol=RTOL, atol_frac=ATOL_FRAC)


@pytest.mark.parametrize("N,K", [(1, 5), (7, 300), (70, 2000)])
def test_w_compact_sizes_match_oracle(aj, N, K):
    rng = np.random.default_rng(N + K)
    uv = rng.uniform(-5e5, 5e5, (K, 2))
    n = rng.uniform(0.1, 1.0, K)
    got = aj.w_compact_curvature_interferometer_from(N, n, uv, 0.05)
    exp = ref.w_compact_curvature_interferometer_from(N, n, uv, 0.05)
    gu.assert_matches(got, exp, rtol=RTOL, atol_frac=ATOL_FRAC)


@pytest.mark.parametrize("S", [1, 31, 32, 33, 100, 257])
def test_solve_sizes_against_numpy(aj, S):
    rng = np.random.default_rng(S)
    X = rng.standard_normal((S, S))
    A = X @ X.T + S * np.eye(S)
    b = rng.standard_normal(S)
    s = aj.reconstruction_positive_negative_from(b, A)
    np.testing.assert_allclose(s, np.linalg.solve(A, b), rtol=1e-11, atol=1e-13)


@pytest.mark.parametrize("K", [1, 1000, 4097])
def test_dirty_image_matches_host_dft(aj, K):
    """The GPU dirty image equals the host restatement's separable DFT of the same visibilities."""
    from autojax_gb300 import synthetic

    d = synthetic.make_dataset("cfg1", K=K, seed=8)
    got = aj.dirty_image_from(d["data"], d["noise_map_real"], d["uv_wavelengths"], d["grid_radians_slim"])
    exp = d["dirty_image"]
    np.testing.assert_allclose(got, exp, rtol=0, atol=1e-10 * np.abs(exp).max())
