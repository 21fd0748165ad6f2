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
