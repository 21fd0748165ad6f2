"""The seeded synthetic inputs the bench and the GPU tests use (host logic, no device): the same
seed gives the same arrays, and the arrays have the stated shapes and distributions.

- uv uniform in the annulus r in [1e3, 5e5] wavelengths;
- sigma lognormal(ln 0.3, 0.5), the same for the real and imaginary parts;
- mapping rows with indices in [0, S) or -1 and live weights summing to 1;
- neighbour lists that form a graph Laplacian: mirrored, no self-loops, sizes equal to the entries
  (the likelihood's deflation of H's constant mode checks for exactly this).
"""

from __future__ import annotations

import numpy as np
import pytest

from autojax_gb300 import synthetic


def _check_mesh(idx, w, nb, nsz, S):
    assert ((idx >= -1) & (idx < S)).all()
    live = np.cumprod(idx != -1, axis=1).astype(bool)
    np.testing.assert_allclose(np.where(live, w, 0.0).sum(axis=1), 1.0, rtol=0, atol=1e-12)
    assert np.array_equal(nsz, (nb != -1).sum(axis=1))
    for i in range(S):
        row = nb[i][nb[i] != -1]
        assert i not in row
        for k in row:
            assert i in nb[k][nb[k] != -1], (i, k)


@pytest.fixture(scope="module")
def cfg1():
    return synthetic.make_dataset("cfg1", K=3000, seed=4)


def test_same_seed_same_arrays(cfg1):
    again = synthetic.make_dataset("cfg1", K=3000, seed=4)
    for key, v in cfg1.items():
        if isinstance(v, np.ndarray):
            assert np.array_equal(v, again[key]), key
    other = synthetic.make_dataset("cfg1", K=3000, seed=5)
    assert not np.array_equal(other["uv_wavelengths"], cfg1["uv_wavelengths"])


def test_visibility_and_noise_distributions(cfg1):
    uv = cfg1["uv_wavelengths"]
    r = np.hypot(uv[:, 0], uv[:, 1])
    assert uv.shape == (3000, 2) and r.min() >= 1e3 and r.max() <= 5e5
    sigma = cfg1["noise_map"].real
    assert np.array_equal(sigma, cfg1["noise_map"].imag)
    assert 0.28 < np.median(sigma) < 0.32 and 0.45 < np.log(sigma).std() < 0.55
    assert cfg1["data"].shape == (3000,) and cfg1["dirty_image"].shape == (cfg1["M"],)


def test_mapping_and_neighbours(cfg1):
    _check_mesh(cfg1["pix_indexes_for_sub_slim_index"], cfg1["pix_weights_for_sub_slim_index"],
                cfg1["neighbors"], cfg1["neighbors_sizes"], cfg1["S"])


def test_lens_models_stay_in_their_ranges(cfg1):
    models = synthetic.lens_models(cfg1, 3, S_range=(40, 120), einstein_range=(0.6, 1.2), lam_range=(1e-3, 1e3),
                                   seed=9)
    for m in models:
        assert 40 <= m["S"] <= 120 and 0.6 <= m["einstein_radius"] <= 1.2
        assert 1e-3 <= m["coefficient"] ** 2 <= 1e3
        _check_mesh(m["pix_indexes_for_sub_slim_index"], m["pix_weights_for_sub_slim_index"], m["neighbors"],
                    m["neighbors_sizes"], m["S"])
