"""Restatement of the reference's deterministic test data (test infrastructure).

``src/autojax/tests.py`` cannot be imported here (it imports jax at line 12),
so its ``DataGenerated`` fixture (tests.py:455-529) is restated: the same
md5-derived seeds (tests.py:64-67), the same draws in the same order, the same
geometry (tests.py:203-306).  Where the reference data generator runs under
numba, this runs the same steps as NumPy; ``tests/golden/make_golden.py``
records the arrays it produced next to the reference outputs, so the fixtures
and not this file are the pinned inputs.
"""

from __future__ import annotations

import hashlib
from dataclasses import dataclass, field

import numpy as np

from . import numpy_port as ref


def deterministic_seed(string: str, *numbers: int) -> int:
    """tests.py:64-67 — md5 of repr((name, sizes)) reduced mod 2**32."""
    digest = hashlib.md5(repr((string, numbers)).encode()).hexdigest()
    return int(digest, 16) % (2**32)


def gen_neighbors(S: int, P: int, rng) -> np.ndarray:
    """tests.py:84-132 — random symmetric neighbour lists, -1 padded, sorted per row."""
    if S <= 0 or P <= 0 or (S * P) % 2:
        raise ValueError("S, P must be positive with S*P even")
    stubs = np.repeat(np.arange(S, dtype=np.int64), P)
    rng.shuffle(stubs)
    pairs = stubs.reshape(-1, 2)
    nb = np.empty((S, P), dtype=np.int64)
    fill = np.zeros(S, dtype=np.int64)
    for a, b in pairs:
        nb[a, fill[a]] = b
        fill[a] += 1
        nb[b, fill[b]] = a
        fill[b] += 1
    sentinel = S
    nb[nb == np.arange(S)[:, None]] = sentinel
    for i in range(S):
        uniq = np.unique(nb[i])
        if uniq.size < P:
            nb[i, : uniq.size] = uniq
            nb[i, uniq.size :] = sentinel
    nb.sort()
    nb[nb == sentinel] = -1
    return nb


def gen_pix_indexes_for_sub_slim_index(M: int, S: int, B: int) -> np.ndarray:
    """tests.py:136-151 — banded source indices: B consecutive pixels from m*S//M."""
    lo = (np.arange(M) * S) // M
    lo = np.minimum(lo, S - B)
    return (lo[:, None] + np.arange(B)[None, :]).astype(np.int64)


@dataclass
class DataGenerated:
    """tests.py:154-529 with the environment defaults of tests.py:26-30."""

    N: int = 30
    B: int = 3
    K: int = 1024
    P: int = 32
    S: int = 256
    pixel_scale: float = 0.2
    coefficient: float = 1.0
    arrays: dict = field(default_factory=dict, init=False)

    def __post_init__(self):
        N, ps = self.N, self.pixel_scale
        radius = ((N + 1) // 2) * ps  # tests.py:211-213
        pixel_scales = (ps, ps)
        centre = (0.0, 0.0)
        mask = ref.mask_2d_circular_from((N, N), pixel_scales, radius, centre)  # tests.py:275-277
        native = np.ascontiguousarray(np.argwhere(~mask))  # tests.py:279-281
        arcsec = np.pi / 648000
        d = ps * arcsec
        g000 = 9.9 * arcsec  # tests.py:296
        I, J = np.mgrid[:N, :N]
        g = np.empty((N, N, 2))
        g[:, :, 0] = -d * I + g000
        g[:, :, 1] = d * J - g000
        slim = g[~mask]
        M = slim.shape[0]
        K, S, B, P = self.K, self.S, self.B, self.P
        dirty = np.random.default_rng(deterministic_seed("dirty_image", M)).random(M)
        uv = np.random.default_rng(deterministic_seed("uv_wavelengths", K, 2)).random((K, 2))
        pidx = gen_pix_indexes_for_sub_slim_index(M, S, B)
        pw = 0.01 + np.random.default_rng(deterministic_seed("pix_weights_for_sub_slim_index", M, S, B)).random((M, B))
        pw /= pw.sum(axis=1).reshape(-1, 1)
        nb = gen_neighbors(S, P, np.random.default_rng(deterministic_seed("neighbors", S, P)))
        nsz = (nb != -1).sum(axis=1)
        data = np.random.default_rng(deterministic_seed("data", K)).random(2 * K).view(np.complex128)
        noise = np.random.default_rng(deterministic_seed("noise_map", K)).random(2 * K).view(np.complex128)
        self.arrays = {
            "grid_size": N,
            "pixel_scale": ps,
            "pixel_scales": pixel_scales,
            "centre": centre,
            "radius": radius,
            "shape_native": (M, M),  # tests.py:236-238 (sic)
            "shape_masked_pixels_2d": (N, N),
            "coefficient": self.coefficient,
            "pixels": S,
            "pix_pixels": S,
            "total_mask_pixels": M,
            "real_space_mask": mask,
            "native_index_for_slim_index": native,
            "grid_radians_2d": g,
            "grid_radians_slim": np.ascontiguousarray(slim),
            "dirty_image": dirty,
            "uv_wavelengths": uv,
            "pix_indexes_for_sub_slim_index": pidx,
            "pix_weights_for_sub_slim_index": pw,
            "pix_size_for_sub_slim_index": np.full(M, B, dtype=np.int64),
            "slim_index_for_sub_slim_index": np.arange(M),
            "sub_fraction": np.ones(M),
            "neighbors": nb,
            "neighbors_sizes": nsz,
            "data": data,
            "noise_map": noise,
            "noise_map_real": np.ascontiguousarray(noise.real),
            "visibilities_real": np.ascontiguousarray(data.real),
        }
