"""Load the golden fixtures written by ``tests/golden/make_golden.py`` and compare against them."""

from __future__ import annotations

import inspect
from functools import lru_cache
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = ("refgen", "cfg1", "edge")
TUPLE_KEYS = {"pixel_scales", "centre", "shape_native", "shape_masked_pixels_2d"}
INT_KEYS = {"grid_size", "pixels", "pix_pixels", "total_mask_pixels"}
FLOAT_KEYS = {"pixel_scale", "radius", "coefficient"}


@lru_cache(maxsize=None)
def raw(case: str) -> dict:
    with np.load(GOLDEN / f"{case}.npz") as z:
        return {k: z[k] for k in z.files}


def inputs(case: str) -> dict:
    """Reference-named inputs of a case, plus the derived arrays the signatures need (from the oracle)."""
    from oracle import numpy_port as ref

    r = raw(case)
    d = {}
    for k, v in r.items():
        if not k.startswith("in__"):
            continue
        name = k[4:]
        if name in TUPLE_KEYS:
            d[name] = tuple(v.tolist())
        elif name in INT_KEYS:
            d[name] = int(v)
        elif name in FLOAT_KEYS:
            d[name] = float(v)
        else:
            d[name] = np.ascontiguousarray(v)
    S = d["pixels"]
    d.setdefault("pix_pixels", S)
    d.setdefault("total_mask_pixels", d["grid_radians_slim"].shape[0])
    return d


@lru_cache(maxsize=None)
def derived(case: str) -> dict:
    """Derived inputs (w_tilde, w_compact, preload, mapping matrix, ...) computed by the oracle."""
    from oracle import numpy_port as ref

    d = inputs(case)
    out = {}
    out["w_tilde"] = ref.w_tilde_curvature_interferometer_from(d["noise_map_real"], d["uv_wavelengths"], d["grid_radians_slim"])
    out["w_compact"] = ref.w_compact_curvature_interferometer_from(d["grid_size"], d["noise_map_real"], d["uv_wavelengths"], d["pixel_scale"])
    out["w_tilde_preload"] = ref.w_tilde_curvature_preload_interferometer_from(
        d["noise_map_real"], d["uv_wavelengths"], d["shape_masked_pixels_2d"], d["grid_radians_2d"]
    )
    out["curvature_preload"] = out["w_tilde_preload"]
    T = ref.mapping_matrix_from(d["pix_indexes_for_sub_slim_index"], d["pix_weights_for_sub_slim_index"], d["pixels"])
    out["mapping_matrix"] = T
    out["matrix"] = T
    out["data_vector"] = ref.data_vector_from(T, d["dirty_image"])
    F = ref.curvature_matrix_via_w_tilde_from(out["w_tilde"], T)
    H = ref.constant_regularization_matrix_from(d["coefficient"], d["neighbors"], d["neighbors_sizes"])
    out["curvature_reg_matrix"] = F + H
    # inputs recorded bit-exact by the generator win over the recomputed ones
    for k in ("curvature_reg_matrix", "data_vector"):
        if k in d:
            out[k] = d[k]
    return out


def full_inputs(case: str) -> dict:
    d = inputs(case)
    d.update(derived(case))
    return d


def call(func, d: dict, **extra):
    """Call ``func`` with its positional parameters looked up by name in ``d`` (tests.py:564-567)."""
    sig = inspect.signature(func)
    pos = (inspect.Parameter.POSITIONAL_ONLY, inspect.Parameter.POSITIONAL_OR_KEYWORD)
    args = [d[k] for k, p in sig.parameters.items() if p.kind in pos and k in d and k not in extra]
    return func(*args, **extra)


def expected_keys(case: str, prefix: str) -> list[str]:
    r = raw(case)
    names = set()
    for k in r:
        if k.startswith(prefix + "__"):
            names.add(k[len(prefix) + 2 :])
        elif k.startswith("fp__" + prefix + "__"):
            names.add(k[len("fp__" + prefix + "__") :].rsplit("__", 1)[0])
    return sorted(names)


def expected(case: str, key: str):
    """Stored value (array or fingerprint dict) of an output key such as ``numba__mapping_matrix_from``."""
    r = raw(case)
    if key in r:
        return r[key]
    fp = {}
    for part in ("rows_idx", "rows", "proj", "projT"):
        fp[part] = r[f"fp__{key}__{part}"]
    return fp


def fingerprint_of(a: np.ndarray, seed: int = 12345) -> dict:
    a = np.asarray(a, dtype=np.float64)
    rng = np.random.default_rng(seed)
    rows = np.unique(np.linspace(0, a.shape[0] - 1, 16).astype(np.int64))
    return {
        "rows_idx": rows,
        "rows": a[rows],
        "proj": a @ rng.standard_normal((a.shape[1], 4)),
        "projT": a.T @ rng.standard_normal((a.shape[0], 4)),
    }


def assert_matches(actual, exp, rtol: float, atol_frac: float = 1e-12, what: str = ""):
    """Compare an array with a stored array or fingerprint.

    ``atol`` is ``atol_frac`` times the largest stored magnitude, so entries that
    cancel to ~0 are judged against the scale of the result, not against themselves.
    """
    if isinstance(exp, dict):
        fa = fingerprint_of(np.asarray(actual))
        np.testing.assert_array_equal(fa["rows_idx"], exp["rows_idx"])
        for part in ("rows", "proj", "projT"):
            e = exp[part]
            atol = atol_frac * max(1e-300, float(np.max(np.abs(e))))
            np.testing.assert_allclose(fa[part], e, rtol=rtol, atol=atol, err_msg=f"{what} [{part}]")
        return
    a = np.asarray(actual)
    e = np.asarray(exp)
    if e.dtype == bool or e.dtype.kind in "iu":
        np.testing.assert_array_equal(a, e, err_msg=what)
        return
    atol = atol_frac * max(1e-300, float(np.max(np.abs(e)))) if e.size else 0.0
    np.testing.assert_allclose(a, e, rtol=rtol, atol=atol, err_msg=what)
