"""The inversion as torch custom operators: registration and shapes on CPU, values and gradients on the GPU."""

from __future__ import annotations

import numpy as np
import pytest
import torch

import golden_util as gu
from oracle import adjoint


def test_ops_are_registered_with_fake_shapes():
    import autojax_gb300  # noqa: F401

    M, B, S, P, K = 7, 3, 5, 4, 11
    meta = dict(device="meta")
    out, gw = torch.ops.autojax_gb300.log_evidence(
        torch.empty(M, dtype=torch.float64, **meta), torch.empty(K, dtype=torch.complex128, **meta),
        torch.empty(K, dtype=torch.complex128, **meta), torch.empty(M, M, dtype=torch.float64, **meta),
        torch.empty(M, B, dtype=torch.int64, **meta), torch.empty(M, B, dtype=torch.float64, **meta),
        torch.empty(S, P, dtype=torch.int64, **meta), torch.empty(S, dtype=torch.int64, **meta),
        torch.empty((), dtype=torch.float64, **meta), 1)
    assert out.shape == (2,) and gw.shape == (M, B)
    W = torch.ops.autojax_gb300.w_tilde_curvature(torch.empty(K, dtype=torch.float64, **meta),
                                                  torch.empty(K, 2, dtype=torch.float64, **meta),
                                                  torch.empty(M, 2, dtype=torch.float64, **meta), 0)
    assert W.shape == (M, M) and W.dtype == torch.float64


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_log_evidence_op_values_and_autograd(precision):
    import autojax_gb300  # noqa: F401

    d = gu.full_inputs("cfg1")
    dev = "cuda"
    args = [torch.from_numpy(np.ascontiguousarray(d[k])).to(dev) for k in
            ("dirty_image", "data", "noise_map", "w_tilde", "pix_indexes_for_sub_slim_index")]
    w = torch.from_numpy(d["pix_weights_for_sub_slim_index"]).to(dev).requires_grad_(True)
    nb = torch.from_numpy(d["neighbors"]).to(dev)
    nsz = torch.from_numpy(d["neighbors_sizes"]).to(dev)
    c = torch.tensor(0.8, dtype=torch.float64, device=dev, requires_grad=True)
    out, gw = torch.ops.autojax_gb300.log_evidence(*args, w, nb, nsz, c, precision)
    gw_w, gc = torch.autograd.grad(out[0], (w, c))
    r = adjoint.log_evidence_and_grad(d["dirty_image"], d["data"], d["noise_map"], d["w_tilde"],
                                      d["pix_indexes_for_sub_slim_index"], d["pix_weights_for_sub_slim_index"],
                                      d["neighbors"], d["neighbors_sizes"], coefficient=0.8)
    tol = 1e-10 if precision == 0 else 1e-8
    assert abs(float(out[0]) - r[0]) <= tol * abs(r[0])
    np.testing.assert_allclose(gw_w.cpu().numpy(), r[2], rtol=0, atol=1e-5 * np.abs(r[2]).max())
    assert torch.equal(gw_w, gw)
    assert abs(float(gc) - 2 * 0.8 * r[1]) <= 1e-5 * abs(2 * 0.8 * r[1]) + 1e-6 * d["pixels"] / 0.64


@pytest.mark.gpu
def test_ops_pass_opcheck():
    import autojax_gb300  # noqa: F401

    d = gu.full_inputs("edge")
    dev = "cuda"
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in d.items() if isinstance(v, np.ndarray)}
    c = torch.tensor(1.1, dtype=torch.float64, device=dev)
    torch.library.opcheck(torch.ops.autojax_gb300.log_evidence.default,
                          (t["dirty_image"], t["data"], t["noise_map"], t["w_tilde"],
                           t["pix_indexes_for_sub_slim_index"], t["pix_weights_for_sub_slim_index"], t["neighbors"],
                           t["neighbors_sizes"], c, 0),
                          test_utils=("test_schema", "test_faketensor"))


def test_every_reference_function_is_an_op_with_its_parameter_names():
    """Each function of autojax.numba resolves under torch.ops.autojax_gb300 with the reference's
    positional parameter names first (tests/golden/reference_signatures.json)."""
    import json
    from pathlib import Path

    import autojax_gb300  # noqa: F401

    sigs = json.loads((Path(__file__).parent / "golden" / "reference_signatures.json").read_text())["numba"]
    for name, params in sigs.items():
        op = getattr(torch.ops.autojax_gb300, name).default
        got = [a.name for a in op._schema.arguments][: len(params)]
        assert got == params, (name, got, params)


@pytest.mark.gpu
def test_drop_in_ops_match_the_functions():
    """The ops return what the drop-in functions return (same C-ABI calls), on golden inputs."""
    import autojax_gb300 as aj

    d = gu.full_inputs("cfg1")
    dev = "cuda"
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in d.items() if isinstance(v, np.ndarray)}
    ops = torch.ops.autojax_gb300
    S = d["pixels"]
    idx, w = t["pix_indexes_for_sub_slim_index"], t["pix_weights_for_sub_slim_index"]
    T = ops.mapping_matrix_from(idx, w, S)
    assert torch.equal(T, aj.mapping_matrix_from(idx, w, S))
    F = ops.curvature_matrix_via_w_wilde_sparse_mapping_matrix_from(t["w_tilde"], idx, w, S)
    assert torch.equal(F, aj.curvature_matrix_via_w_wilde_sparse_mapping_matrix_from(t["w_tilde"], idx, w, S))
    wc = ops.w_compact_curvature_interferometer_from(d["grid_size"], t["noise_map_real"], t["uv_wavelengths"],
                                                     d["pixel_scale"])
    np.testing.assert_allclose(wc.cpu().numpy(), d["w_compact"], rtol=1e-10, atol=1e-11 * np.abs(d["w_compact"]).max())
    H = ops.constant_regularization_matrix_from(0.7, t["neighbors"], t["neighbors_sizes"])
    D = ops.data_vector_from(T, t["dirty_image"])
    s = ops.reconstruction_positive_negative_from(D, (F + H).contiguous())
    assert s.shape == (S,) and torch.isfinite(s).all()
    logE = ops.log_likelihood_function_via_w_tilde_from(t["dirty_image"], t["data"], t["noise_map"], t["w_tilde"], idx,
                                                         w, t["neighbors"], t["neighbors_sizes"])
    exp = float(gu.expected("cfg1", "numba__log_likelihood_function_via_w_tilde_from"))
    assert logE.shape == () and abs(float(logE) - exp) <= 1e-10 * abs(exp)
    mask = ops.mask_2d_circular_from([30, 30], [0.1, 0.1], 1.2, [0.0, 0.0])
    assert mask.dtype == torch.bool and mask.shape == (30, 30)
    torch.library.opcheck(ops.curvature_matrix_via_w_tilde_from.default, (t["w_tilde"], T),
                          test_utils=("test_schema", "test_faketensor"))
