"""The no-allocation solve entry point, called through the C ABI.

aj_spd_solve_noalloc serves callers that cannot allocate device memory (a
plugin or foreign-function host that only holds device pointers its host
application gave it): it takes no workspace and keeps its scratch in a fixed
device array for systems up to AJ_NOALLOC_SOLVE_MAX_S.  This file is collected
last so that a run stopping at the first failure has run every other test.
"""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _spd(S, seed):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((S, S))
    return X @ X.T + S * np.eye(S), rng.standard_normal(S)


def _solve_with_workspace(lib, A, b):
    import torch

    from autojax_gb300 import _lib

    S = b.shape[0]
    ws = torch.empty(lib.aj_spd_solve_workspace_size(S), dtype=torch.uint8, device="cuda")
    out = torch.empty(S, dtype=torch.float64, device="cuda")
    info = torch.zeros(2, dtype=torch.int32, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    _lib.check(lib.aj_spd_solve(b.data_ptr(), A.data_ptr(), S, out.data_ptr(), ws.data_ptr(), ws.numel(),
                                info.data_ptr(), st), "aj_spd_solve")
    torch.cuda.synchronize()
    assert int(info[0]) == 0
    return out.cpu().numpy()


def test_noalloc_solve_matches_workspace_solve_twice():
    import torch

    from autojax_gb300 import _lib

    lib = _lib.load()
    st = torch.cuda.current_stream().cuda_stream
    # calls in a row, different sizes (the capacity itself first): the shared scratch keeps the
    # previous call's contents
    for S, seed in ((_lib.AJ_NOALLOC_SOLVE_MAX_S, 3), (1000, 1), (257, 2)):
        A_np, b_np = _spd(S, seed)
        A = torch.from_numpy(A_np).cuda()
        b = torch.from_numpy(b_np).cuda()
        out = torch.full((S,), float("nan"), dtype=torch.float64, device="cuda")
        info = torch.zeros(2, dtype=torch.int32, device="cuda")
        rc = lib.aj_spd_solve_noalloc(b.data_ptr(), A.data_ptr(), S, out.data_ptr(), info.data_ptr(), st)
        assert rc == _lib.AJ_OK
        torch.cuda.synchronize()
        assert int(info[0]) == 0
        ref = _solve_with_workspace(lib, A, b)
        np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=1e-11, atol=1e-13)


def test_noalloc_solve_rejects_sizes_above_capacity():
    import torch

    from autojax_gb300 import _lib

    lib = _lib.load()
    S = _lib.AJ_NOALLOC_SOLVE_MAX_S + 1
    rc = lib.aj_spd_solve_noalloc(None, None, S, None, None, torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.AJ_ERR_TOO_LARGE


def test_noalloc_solve_requires_info():
    """A non-positive-definite A is reported only through info, so a NULL info is rejected."""
    import torch

    from autojax_gb300 import _lib

    lib = _lib.load()
    S = 8
    A = torch.eye(S, dtype=torch.float64, device="cuda")
    b = torch.ones(S, dtype=torch.float64, device="cuda")
    out = torch.empty(S, dtype=torch.float64, device="cuda")
    rc = lib.aj_spd_solve_noalloc(b.data_ptr(), A.data_ptr(), S, out.data_ptr(), None,
                                  torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.AJ_ERR_ARG
