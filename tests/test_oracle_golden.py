"""Pin the NumPy oracle to outputs of the reference implementation itself (CPU only)."""

from __future__ import annotations

import numpy as np
import pytest

import golden_util as gu
from oracle import adjoint
from oracle import numpy_port as ref

# original.py names whose signatures differ from numba.py map to the oracle's original_* restatements;
# the others (and the likelihoods, whose original.py arithmetic is the same expansion) use numba.py's form.
ORIGINAL_ONLY = {
    "mapping_matrix_from": ref.original_mapping_matrix_from,
    "curvature_matrix_via_w_tilde_curvature_preload_interferometer_from": (
        ref.original_curvature_matrix_via_w_tilde_curvature_preload_interferometer_from
    ),
}


def _oracle_for(prefix: str, name: str):
    if name.startswith("log_likelihood_coefficient_"):
        coef = float(name.rsplit("_", 1)[1])
        return lambda d: ref.log_likelihood_function_via_w_tilde_from(
            d["dirty_image"], d["data"], d["noise_map"], d["w_tilde"], d["pix_indexes_for_sub_slim_index"],
            d["pix_weights_for_sub_slim_index"], d["neighbors"], d["neighbors_sizes"], coefficient=coef,
        )
    if prefix in ("ref", "original") and name in ORIGINAL_ONLY:
        if prefix == "ref" and name == "curvature_matrix_via_w_tilde_curvature_preload_interferometer_from":
            f = ORIGINAL_ONLY[name]
        elif prefix == "original" or name == "mapping_matrix_from":
            f = ORIGINAL_ONLY[name]
        else:
            f = getattr(ref, name)
        return lambda d: gu.call(f, d)
    f = getattr(ref, name)
    return lambda d: gu.call(f, {k: v for k, v in d.items() if k != "coefficient"} if "log_likelihood" in name else d)


CASES = [(case, prefix, name) for case in gu.CASES for prefix in ("numba", "ref", "original") for name in gu.expected_keys(case, prefix)]


@pytest.mark.parametrize("case,prefix,name", CASES, ids=[f"{c}-{p}-{n}" for c, p, n in CASES])
def test_oracle_matches_reference(case, prefix, name):
    d = gu.full_inputs(case)
    got = _oracle_for(prefix, name)(d)
    exp = gu.expected(case, f"{prefix}__{name}")
    # the oracle vectorises the reference's loops; only summation order differs
    gu.assert_matches(got, exp, rtol=1e-9, atol_frac=1e-11, what=f"{case}:{prefix}__{name}")


@pytest.mark.parametrize("case", ["cfg1", "edge"])
def test_adjoint_value_matches_reference_loglike(case):
    d = gu.full_inputs(case)
    logE, _, _ = adjoint.log_evidence_and_grad(
        d["dirty_image"], d["data"], d["noise_map"], d["w_tilde"], d["pix_indexes_for_sub_slim_index"],
        d["pix_weights_for_sub_slim_index"], d["neighbors"], d["neighbors_sizes"],
    )
    exp = float(gu.expected(case, "numba__log_likelihood_function_via_w_tilde_from"))
    assert abs(logE - exp) <= 1e-10 * abs(exp)


@pytest.mark.parametrize("case,coef", [("cfg1", 0.7), ("edge", 1.3)])
def test_adjoint_gradients_match_finite_differences(case, coef):
    """Central differences of the pinned log-evidence.

    Weights use a 1e-6 step.  lambda uses a 1e-5 relative step: log|H| carries
    ~1e-7 of rounding noise from H's eigenvalue 1e-8 (the constant vector, L 1 = 0),
    which a 1e-6 step would amplify to ~1e-1 (1e-4 is already truncation-limited on the small edge case).
    """
    d = gu.full_inputs(case)
    args = (d["dirty_image"], d["data"], d["noise_map"], d["w_tilde"], d["pix_indexes_for_sub_slim_index"])
    w = d["pix_weights_for_sub_slim_index"].copy()
    nb, nsz = d["neighbors"], d["neighbors_sizes"]
    logE, dlam, gw = adjoint.log_evidence_and_grad(*args, w, nb, nsz, coefficient=coef)

    def f(weights, lam):
        return ref.log_likelihood_function_via_w_tilde_from(*args, weights, nb, nsz, coefficient=np.sqrt(lam))

    lam = coef * coef
    h = 1e-5 * lam
    fd_lam = (f(w, lam + h) - f(w, lam - h)) / (2 * h)
    assert abs(fd_lam - dlam) <= 1e-5 * max(1.0, abs(dlam)), (fd_lam, dlam)
    rng = np.random.default_rng(0)
    keep = adjoint.effective_weight_mask(d["pix_indexes_for_sub_slim_index"])
    picks = [tuple(x) for x in np.argwhere(keep)[rng.choice(int(keep.sum()), 6, replace=False)]]
    picks += [tuple(x) for x in np.argwhere(~keep)[:2]]
    for m, b in picks:
        hw = 1e-6
        wp = w.copy()
        wp[m, b] += hw
        wm = w.copy()
        wm[m, b] -= hw
        fd = (f(wp, lam) - f(wm, lam)) / (2 * hw)
        scale = max(1.0, float(np.max(np.abs(gw))))
        assert abs(fd - gw[m, b]) <= 2e-5 * scale, (m, b, fd, gw[m, b])


@pytest.mark.parametrize("case", ["refgen", "cfg1"])
def test_w_tilde_entries_and_separable_table_match_the_pinned_oracle(case):
    """The two host helpers the large-size checks use (sampled W~ entries, and the offset
    table by a separable complex product) against the golden-pinned oracle sums."""
    d = gu.full_inputs(case)
    W = d["w_tilde"]
    M = W.shape[0]
    rng = np.random.default_rng(4)
    rows, cols = rng.integers(0, M, 300), rng.integers(0, M, 300)
    e = ref.w_tilde_entries(d["noise_map_real"], d["uv_wavelengths"], d["grid_radians_slim"], rows, cols)
    np.testing.assert_allclose(e, W[rows, cols], rtol=1e-12, atol=1e-13 * np.abs(W).max())
    wc = ref.w_compact_separable(d["grid_size"], d["noise_map_real"], d["uv_wavelengths"], d["pixel_scale"])
    np.testing.assert_allclose(wc, d["w_compact"], rtol=1e-11, atol=1e-12 * np.abs(d["w_compact"]).max())
