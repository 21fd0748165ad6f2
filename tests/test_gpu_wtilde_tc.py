"""The tensor-core digit product behind the mixed direct w_tilde (csrc/wtilde_tc.cu).

aj_digit_syrk_probe runs the tcgen05 kernel on digit planes given directly, so
these tests check the shared-memory descriptors, the TMEM level accumulators
and their fold against exact arithmetic: every level sum is an integer below
2^24 (float64 holds it exactly), and the double-float result must match
sum_L 2^-7L level_L to ~2^-46 of its scale.  The adversarial case puts every
digit at its bound (+64), where each level sum reaches its largest value.
"""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DIGITS = 7
BITS = 7


def _bf16_bits(a: np.ndarray) -> np.ndarray:
    """bf16 bit patterns of small integers (exact: the top half of their float32 pattern)."""
    return (a.astype(np.float32).view(np.uint32) >> 16).astype(np.uint16)


def _exact(Dg: np.ndarray, M: int) -> np.ndarray:
    """sum over levels L = d + e <= 6 of 2^-7L sum_r D_d[i, r] D_e[j, r] (level sums exact in float64)."""
    X = Dg[:, :M, :].astype(np.float64)
    out = np.zeros((M, M))
    for L in range(DIGITS):
        acc = np.zeros((M, M))
        for d in range(L + 1):
            acc += X[d] @ X[L - d].T
        out += acc * 2.0 ** (-BITS * L)
    return out


def _run(Dg: np.ndarray, M: int, rows: int, calls: int = 1):
    import torch

    from autojax_gb300 import _lib

    lib = _lib.load()
    dev = torch.device("cuda", 0)
    d = torch.from_numpy(_bf16_bits(Dg).view(np.int16)).to(dev)
    oh = torch.zeros((M, M), dtype=torch.float32, device=dev)
    ol = torch.zeros((M, M), dtype=torch.float32, device=dev)
    scale = torch.ones(1, dtype=torch.float32, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    st = torch.cuda.current_stream().cuda_stream
    for c in range(calls):
        _lib.check(lib.aj_digit_syrk_probe(d.data_ptr(), rows, M, oh.data_ptr(), ol.data_ptr(), scale.data_ptr(),
                                           1 if c else 0, err.data_ptr(), st), "aj_digit_syrk_probe")
    torch.cuda.synchronize()
    assert int(err[0]) == 0
    return oh.double().cpu().numpy() + ol.double().cpu().numpy()


def _lower(a):
    return np.tril(a)


@pytest.mark.parametrize("M,rows", [(200, 512), (128, 256), (333, 768)])
def test_digit_product_matches_exact(M, rows):
    rng = np.random.default_rng(M + rows)
    Mp = (M + 127) // 128 * 128
    Dg = rng.integers(-64, 65, size=(DIGITS, Mp, rows))
    Dg[:, M:, :] = 0
    got = _run(Dg, M, rows)
    exp = _exact(Dg, M)
    scale = np.abs(exp).max()
    np.testing.assert_allclose(_lower(got), _lower(exp), rtol=0, atol=2.0**-44 * scale)
    assert np.all(np.triu(got, 1) == 0)  # only the lower triangle is written


def test_digit_product_at_the_exactness_bound():
    """All digits +64 (and a sign-alternating block): each level sum reaches (L + 1) * 256 * 2^12."""
    M, rows = 130, 512
    Mp = 256
    Dg = np.full((DIGITS, Mp, rows), 64, dtype=np.int64)
    Dg[:, 64:96, 256:] = -64
    Dg[:, M:, :] = 0
    got = _run(Dg, M, rows)
    exp = _exact(Dg, M)
    scale = np.abs(exp).max()
    np.testing.assert_allclose(_lower(got), _lower(exp), rtol=0, atol=2.0**-44 * scale)


def test_digit_product_accumulates_across_calls():
    M, rows = 160, 256
    rng = np.random.default_rng(3)
    Dg = rng.integers(-64, 65, size=(DIGITS, 256, rows))
    Dg[:, M:, :] = 0
    got = _run(Dg, M, rows, calls=3)
    exp = 3.0 * _exact(Dg, M)
    np.testing.assert_allclose(_lower(got), _lower(exp), rtol=0, atol=2.0**-44 * np.abs(exp).max())
