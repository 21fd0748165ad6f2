"""Batched evaluations: many lens models (own S, mapping, neighbours, coefficient) against one dataset.

Each model's logE, dlogE/dlambda and weight gradient from one
aj_log_evidence_batched call (eagerly and replayed from a captured graph) is
checked against the float64 oracle at the single-evaluation tolerances:
rel 1e-10 for the float64 path, the mixed-path bounds of test_gpu_mixed.py
for the mixed one.
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import adjoint

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    import autojax_gb300 as aj
    from autojax_gb300 import synthetic

    d = synthetic.make_dataset("cfg1", K=600, seed=5)
    W = aj.w_tilde_curvature_interferometer_from(d["noise_map_real"], d["uv_wavelengths"], d["grid_radians_slim"])
    models = synthetic.lens_models(d, 7, S_range=(20, 180), lam_range=(1e-2, 1e2), seed=9)
    refs = [adjoint.log_evidence_and_grad(d["dirty_image"], d["data"], d["noise_map"], W,
                                          m["pix_indexes_for_sub_slim_index"], m["pix_weights_for_sub_slim_index"],
                                          m["neighbors"], m["neighbors_sizes"], coefficient=m["coefficient"])
            for m in models]
    return d, W, models, refs


def _batch(setup, precision):
    from autojax_gb300.inversion import Dataset, LogEvidenceBatch

    d, W, models, _ = setup
    ds = Dataset(d["dirty_image"], d["data"], d["noise_map"], W, precision=precision)
    P = max(m["neighbors"].shape[1] for m in models)
    batch = LogEvidenceBatch(ds, [m["S"] for m in models], B=3, P=P)
    for i, m in enumerate(models):
        batch.set_model(i, m["pix_indexes_for_sub_slim_index"], m["pix_weights_for_sub_slim_index"], m["neighbors"],
                        m["neighbors_sizes"], m["coefficient"])
    return batch


def _cond(setup, m):
    """cond(A) and ||H|| / 1e-8: H = 1e-8 I + lambda L keeps the eigenvalue 1e-8 (the
    constant vector), so float64 log|H| and tr(H^-1) carry ~eps ||H|| / 1e-8 of rounding
    in any float64 implementation, the oracle's LAPACK included."""
    from oracle import numpy_port as ref

    W = setup[1]
    T = ref.mapping_matrix_from(m["pix_indexes_for_sub_slim_index"], m["pix_weights_for_sub_slim_index"], m["S"])
    H = ref.constant_regularization_matrix_from(m["coefficient"], m["neighbors"], m["neighbors_sizes"])
    ev = np.linalg.eigvalsh(T.T @ W @ T + H)
    return ev[-1] / ev[0], np.linalg.eigvalsh(H)[-1] / 1e-8


def _check(batch, setup, precision):
    import torch

    _, _, models, refs = setup
    torch.cuda.synchronize()
    batch.check()
    out = batch.out.cpu().numpy()
    for i, (m, (r_logE, r_dlam, r_gw)) in enumerate(zip(models, refs)):
        gw = batch.evals[i].grad_weights.cpu().numpy()
        cond, cond_h = _cond(setup, m)
        if precision == "fp64":
            # float64 rounding grows with cond(A) (s^T D = D^T A^-1 D) and, in absolute terms, with
            # ||H|| / 1e-8 (log|H|; LU and Cholesky log|H| differ by ~1e-6 on these models)
            tol = max(1e-10, 4e-16 * cond) * abs(r_logE) + 2.2e-16 * cond_h
            assert abs(out[i, 0] - r_logE) <= tol, (i, out[i, 0], r_logE, cond, cond_h)
            tol_lam = max(1e-8, 4e-16 * cond) * max(1.0, abs(r_dlam)) + 2.2e-16 * cond_h / m["coefficient"] ** 2
            assert abs(out[i, 1] - r_dlam) <= tol_lam, (i, out[i, 1], r_dlam)
            np.testing.assert_allclose(gw, r_gw, rtol=1e-8, atol=max(1e-9, 4e-16 * cond) * np.abs(r_gw).max())
        else:
            c = m["coefficient"]
            assert abs(out[i, 0] - r_logE) <= 1e-8 * abs(r_logE), (i, out[i, 0], r_logE)
            assert abs(out[i, 1] - r_dlam) <= 1e-6 * m["S"] / c**2 + 1e-5 * abs(r_dlam), (i, out[i, 1], r_dlam)
            # the weight gradient goes through A^-1: its error scales with cond(A)
            np.testing.assert_allclose(gw, r_gw, rtol=0, atol=max(1e-5, 2e-15 * cond) * np.abs(r_gw).max())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_matches_oracle(setup, precision):
    batch = _batch(setup, precision)
    batch.launch()
    _check(batch, setup, precision)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_equals_single_evaluations(setup, precision):
    """The batch runs each model's kernels in the same order as a lone evaluation: results are identical."""
    import torch

    from autojax_gb300.inversion import LogEvidence

    d, W, models, _ = setup
    batch = _batch(setup, precision)
    batch.launch()
    torch.cuda.synchronize()
    for i, m in enumerate(models):
        e = LogEvidence(S=m["S"], B=3, P=batch.evals[i].P, precision=precision, dataset=batch.dataset)
        e.set_model(m["pix_indexes_for_sub_slim_index"], m["pix_weights_for_sub_slim_index"], m["neighbors"],
                    m["neighbors_sizes"], m["coefficient"])
        e.launch()
        torch.cuda.synchronize()
        assert torch.equal(e.out, batch.out[i]), (i, e.out.tolist(), batch.out[i].tolist())
        assert torch.equal(e.grad_weights, batch.evals[i].grad_weights), i


def test_batch_graph_replay_matches_oracle(setup):
    import torch

    batch = _batch(setup, "mixed")
    batch.capture()
    batch.out.zero_()
    for e in batch.evals:
        e.grad_weights.zero_()
    batch.step()
    _check(batch, setup, "mixed")
    assert batch.launches_per_batch and batch.launches_per_batch > 10 * batch.n
    # new coefficients go through the captured graph
    _, _, models, _ = setup
    for i, m in enumerate(models):
        batch.evals[i].set_coefficient(m["coefficient"] * 1.5)
    batch.step()
    torch.cuda.synchronize()
    d, W = setup[0], setup[1]
    for i in (0, len(models) - 1):
        m = models[i]
        r = adjoint.log_evidence_and_grad(d["dirty_image"], d["data"], d["noise_map"], W,
                                          m["pix_indexes_for_sub_slim_index"], m["pix_weights_for_sub_slim_index"],
                                          m["neighbors"], m["neighbors_sizes"], coefficient=m["coefficient"] * 1.5)
        assert abs(float(batch.out[i, 0]) - r[0]) <= 1e-8 * abs(r[0])


def test_batch_rejects_a_short_workspace(setup):
    import ctypes

    import torch

    from autojax_gb300 import _lib

    batch = _batch(setup, "fp64")
    batch._ws_bytes[2] = 16
    rc = batch.lib.aj_log_evidence_batched(batch._problems, batch.n, _lib.AJ_FP64, 1, batch.out.data_ptr(),
                                           ctypes.cast(batch._grads, ctypes.c_void_p),
                                           ctypes.cast(batch._recons, ctypes.c_void_p),
                                           ctypes.cast(batch._ws, ctypes.c_void_p),
                                           ctypes.cast(batch._ws_bytes, ctypes.c_void_p), batch.info.data_ptr(),
                                           torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.AJ_ERR_WORKSPACE


def test_crowded_batch_is_deterministic():
    """40 mixed-precision models on 16 branches (several per branch, panels competing for SMs):
    every replay equals the lone evaluations bit for bit.  A panel kernel that wrote its pivot
    block back into L while late-starting blocks of the same launch still had to read it failed
    exactly this way, on different models from run to run."""
    import torch

    from autojax_gb300 import synthetic
    from autojax_gb300.inversion import Dataset, LogEvidence, LogEvidenceBatch

    d, W = _crowded_setup()
    models = synthetic.lens_models(d, 40, S_range=(200, 440), lam_range=(1e-2, 1e2), seed=21)
    ds = Dataset(d["dirty_image"], d["data"], d["noise_map"], W, precision="mixed")
    P = max(m["neighbors"].shape[1] for m in models)
    batch = LogEvidenceBatch(ds, [m["S"] for m in models], B=3, P=P)
    for i, m in enumerate(models):
        batch.set_model(i, m["pix_indexes_for_sub_slim_index"], m["pix_weights_for_sub_slim_index"], m["neighbors"],
                        m["neighbors_sizes"], m["coefficient"])
    singles = []
    for i, m in enumerate(models):
        e = LogEvidence(S=m["S"], B=3, P=P, precision="mixed", dataset=ds)
        e.set_model(m["pix_indexes_for_sub_slim_index"], m["pix_weights_for_sub_slim_index"], m["neighbors"],
                    m["neighbors_sizes"], m["coefficient"])
        e.launch()
        torch.cuda.synchronize()
        e.check()
        singles.append((e.out.clone(), e.grad_weights.clone()))
        del e
    batch.capture()
    for _ in range(3):
        batch.step()
        torch.cuda.synchronize()
        batch.check()
        for i, (out, gw) in enumerate(singles):
            assert torch.equal(batch.out[i], out), (i, batch.out[i].tolist(), out.tolist())
            assert torch.equal(batch.evals[i].grad_weights, gw), i


def _crowded_setup():
    import autojax_gb300 as aj
    from autojax_gb300 import synthetic

    d = synthetic.make_dataset("cfg1", K=600, seed=6)
    W = aj.w_tilde_curvature_interferometer_from(d["noise_map_real"], d["uv_wavelengths"], d["grid_radians_slim"])
    return d, W


def test_release_stream_frees_and_recreates_side_streams(setup):
    """aj_release_stream drops the lanes and branches of a caller stream; the next call on the
    stream builds a fresh set and gives bit-identical results."""
    import torch

    from autojax_gb300 import _lib

    lib = _lib.load()
    batch = _batch(setup, "mixed")
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        batch.launch()
    s.synchronize()
    first = batch.out.cpu().numpy().copy()
    assert lib.aj_release_stream(s.cuda_stream) == _lib.AJ_OK
    assert lib.aj_release_stream(s.cuda_stream) == _lib.AJ_OK  # nothing left to free
    with torch.cuda.stream(s):
        batch.launch()
    s.synchronize()
    np.testing.assert_array_equal(batch.out.cpu().numpy(), first)
    assert lib.aj_release_stream(s.cuda_stream) == _lib.AJ_OK


def test_batch_at_the_batched_configuration_sizes_matches_oracle():
    """Three members of a batch at the batched configuration's sizes (K = 5e5, M = 7,860 image
    pixels, S = 500, 1,250 and 2,000), mixed precision with gradients, against the oracle on the
    same shared w_tilde (the float64 table expansion the batch reads)."""
    import torch

    import autojax_gb300 as aj
    from autojax_gb300 import synthetic
    from autojax_gb300.inversion import Dataset, LogEvidenceBatch

    d = synthetic.make_dataset("cfg5")
    dev = torch.device("cuda", 0)
    wc = aj.w_compact_curvature_interferometer_from(d["grid_size"], torch.from_numpy(d["noise_map_real"]).to(dev),
                                                    torch.from_numpy(d["uv_wavelengths"]).to(dev), d["pixel_scale"])
    Wd = aj.w_tilde_via_compact_from(wc, torch.from_numpy(d["native_index_for_slim_index"]).to(dev))
    W = Wd.cpu().numpy()
    models = [synthetic.lens_models(d, 1, S_range=(S, S), seed=70 + S)[0] for S in (500, 1250, 2000)]
    ds = Dataset(d["dirty_image"], d["data"], d["noise_map"], Wd, precision="mixed", device=dev)
    P = max(m["neighbors"].shape[1] for m in models)
    batch = LogEvidenceBatch(ds, [m["S"] for m in models], B=3, P=P)
    for i, m in enumerate(models):
        batch.set_model(i, m["pix_indexes_for_sub_slim_index"], m["pix_weights_for_sub_slim_index"], m["neighbors"],
                        m["neighbors_sizes"], m["coefficient"])
    batch.launch()
    torch.cuda.synchronize()
    batch.check()
    out = batch.out.cpu().numpy()
    for i, m in enumerate(models):
        r_logE, r_dlam, r_gw = adjoint.log_evidence_and_grad(
            d["dirty_image"], d["data"], d["noise_map"], W, m["pix_indexes_for_sub_slim_index"],
            m["pix_weights_for_sub_slim_index"], m["neighbors"], m["neighbors_sizes"], coefficient=m["coefficient"])
        c = m["coefficient"]
        assert abs(out[i, 0] - r_logE) <= 1e-7 * abs(r_logE), (m["S"], out[i, 0], r_logE)
        assert abs(out[i, 1] - r_dlam) <= 1e-6 * m["S"] / c**2 + 1e-5 * abs(r_dlam), (m["S"], out[i, 1], r_dlam)
        from oracle import numpy_port as ref

        T = ref.mapping_matrix_from(m["pix_indexes_for_sub_slim_index"], m["pix_weights_for_sub_slim_index"], m["S"])
        H = ref.constant_regularization_matrix_from(c, m["neighbors"], m["neighbors_sizes"])
        ev = np.linalg.eigvalsh(T.T @ W @ T + H)
        cond = ev[-1] / ev[0]
        gw = batch.evals[i].grad_weights.cpu().numpy()
        np.testing.assert_allclose(gw, r_gw, rtol=0, atol=max(1e-5, 2e-15 * cond) * np.abs(r_gw).max())
