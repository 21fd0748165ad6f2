"""The reference's LU semantics (np.linalg.solve / slogdet, numba.py:731, 849-850) for matrices that
are not positive definite: aj_lu_solve, and the drop-in functions that fall back to it.

Tolerances: the solve against LAPACK's at cond(A) * 1e-15 (forward error), log|det| at 1e-11 of
S * max(1, |log|det||); the likelihood at the float64 path's rel 1e-10.
"""

from __future__ import annotations

import numpy as np
import pytest

import golden_util as gu
from oracle import numpy_port as ref

pytestmark = pytest.mark.gpu


def _lu(A, b):
    import torch

    from autojax_gb300 import _lib

    lib = _lib.load()
    S = b.shape[0]
    At = torch.from_numpy(A).cuda()
    bt = torch.from_numpy(b).cuda()
    x = torch.empty(S, dtype=torch.float64, device="cuda")
    ld = torch.empty(1, dtype=torch.float64, device="cuda")
    info = torch.zeros(2, dtype=torch.int32, device="cuda")
    ws = torch.empty(lib.aj_lu_solve_workspace_size(S), dtype=torch.uint8, device="cuda")
    _lib.check(lib.aj_lu_solve(bt.data_ptr(), At.data_ptr(), S, x.data_ptr(), ld.data_ptr(), ws.data_ptr(), ws.numel(),
                               info.data_ptr(), torch.cuda.current_stream().cuda_stream), "aj_lu_solve")
    torch.cuda.synchronize()
    return x.cpu().numpy(), float(ld[0]), int(info[0])


@pytest.mark.parametrize("S", [1, 2, 31, 32, 33, 100, 257, 700])
def test_lu_solve_and_logabsdet_match_lapack(S):
    rng = np.random.default_rng(S)
    A = rng.standard_normal((S, S))  # general, nonsymmetric
    b = rng.standard_normal(S)
    x, ld, info = _lu(A, b)
    assert info == 0
    exp = np.linalg.solve(A, b)
    cond = np.linalg.cond(A)
    assert np.linalg.norm(x - exp) / np.linalg.norm(exp) <= max(1e-13, 1e-15 * cond)
    sign, e_ld = np.linalg.slogdet(A)
    assert abs(ld - e_ld) <= 1e-11 * S * max(1.0, abs(e_ld))


def test_lu_reports_singular():
    A = np.ones((40, 40))
    _, _, info = _lu(A, np.ones(40))
    from autojax_gb300 import _lib

    assert info == _lib.AJ_INFO_SINGULAR


def test_indefinite_solve_falls_back_to_lu():
    import autojax_gb300 as aj

    rng = np.random.default_rng(5)
    S = 120
    Q, _ = np.linalg.qr(rng.standard_normal((S, S)))
    ev = np.concatenate([np.linspace(1, 10, S - 20), -np.linspace(1, 5, 20)])
    A = (Q * ev) @ Q.T  # symmetric, indefinite, well conditioned
    b = rng.standard_normal(S)
    s = aj.reconstruction_positive_negative_from(b, A)
    np.testing.assert_allclose(s, np.linalg.solve(A, b), rtol=1e-11, atol=1e-12)
    with pytest.raises(np.linalg.LinAlgError):
        aj.reconstruction_positive_negative_from(b, np.zeros((S, S)))


@pytest.mark.parametrize("case", ["cfg1", "edge"])
def test_likelihood_with_indefinite_curvature_matches_reference(case):
    """A negated w_tilde makes F + H indefinite: the reference still returns a log-evidence (LU
    solve, log|det| by LU), and so does the drop-in function (through its LU fallback)."""
    import autojax_gb300 as aj

    d = gu.full_inputs(case)
    W = -np.ascontiguousarray(d["w_tilde"])
    args = (d["dirty_image"], d["data"], d["noise_map"], W, d["pix_indexes_for_sub_slim_index"],
            d["pix_weights_for_sub_slim_index"], d["neighbors"], d["neighbors_sizes"])
    exp = ref.log_likelihood_function_via_w_tilde_from(*args)
    got = aj.log_likelihood_function_via_w_tilde_from(*args)
    assert abs(got - exp) <= 1e-10 * abs(exp), (got, exp)
    wc = -np.ascontiguousarray(d["w_compact"])
    cargs = (d["dirty_image"], d["data"], d["noise_map"], wc, d["native_index_for_slim_index"], *args[4:])
    exp_c = ref.log_likelihood_function_via_w_compact_from(*cargs)
    got_c = aj.log_likelihood_function_via_w_compact_from(*cargs)
    assert abs(got_c - exp_c) <= 1e-10 * abs(exp_c), (got_c, exp_c)
