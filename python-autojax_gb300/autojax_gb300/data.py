"""The reference's dataset file format (``DataLoaded``, tests.py:397-452).

An ``.npz`` holding the eight arrays a likelihood evaluation needs, under the
reference's parameter names; M, K, P and S follow from their shapes as
tests.py:404-418 derives them.  ``load_npz`` returns them as C-contiguous
arrays of the reference's dtypes (the numba signatures reject anything else),
ready for the functions of this package.
"""

from __future__ import annotations

from pathlib import Path

import numpy as np

NPZ_KEYS = {
    "dirty_image": np.float64,
    "data": np.complex128,
    "noise_map": np.complex128,
    "uv_wavelengths": np.float64,
    "neighbors": np.int64,
    "neighbors_sizes": np.int64,
    "pix_indexes_for_sub_slim_index": np.int64,
    "pix_weights_for_sub_slim_index": np.float64,
}


def load_npz(path) -> dict:
    """The arrays of a DataLoaded-format file plus M, K, P and S (tests.py:404-418)."""
    with np.load(Path(path)) as z:
        missing = [k for k in NPZ_KEYS if k not in z.files]
        if missing:
            raise KeyError(f"{path}: missing arrays {missing}")
        out = {k: np.ascontiguousarray(z[k], dtype=dt) for k, dt in NPZ_KEYS.items()}
    out["M"] = out["pix_indexes_for_sub_slim_index"].shape[0]
    out["K"] = out["uv_wavelengths"].shape[0]
    out["P"] = out["neighbors"].shape[1]
    out["S"] = out["neighbors_sizes"].size
    if out["pix_weights_for_sub_slim_index"].shape != out["pix_indexes_for_sub_slim_index"].shape:
        raise ValueError("pix_weights_for_sub_slim_index and pix_indexes_for_sub_slim_index differ in shape")
    if out["dirty_image"].shape != (out["M"],) or out["data"].shape != (out["K"],) or \
            out["noise_map"].shape != (out["K"],) or out["neighbors"].shape[0] != out["S"]:
        raise ValueError("inconsistent array shapes")
    return out


def save_npz(path, d: dict) -> None:
    """Write the eight arrays of ``d`` (keyed by the reference's names) in the DataLoaded format."""
    np.savez(Path(path), **{k: np.ascontiguousarray(d[k], dtype=dt) for k, dt in NPZ_KEYS.items()})


__all__ = ["NPZ_KEYS", "load_npz", "save_npz"]
