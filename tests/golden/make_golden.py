"""Generate the golden fixtures by running the reference implementation itself.

Run here, where the reference source is mounted (not on a GPU host):

    python tests/golden/make_golden.py /root/reference

The reference (ickc/python-autojax, ``src/autojax/numba.py`` and
``src/autojax/original.py``) is imported in place.  numba is not installed, so a
pass-through shim stands in for it (``jit`` returns the function unchanged,
``prange`` is ``range``): the reference's own Python source then runs as plain
NumPy, with its own loops, in its own order.

Cases (each written as ``<case>.npz`` next to this script):

* ``refgen``   — the reference's ``DataGenerated`` fixture at its defaults
                 (N=30, B=3, K=1024, P=32, S=256; tests.py:26-30, 455-529);
                 outputs of every function in the reference's test list
                 (tests.py:41-61), taken from ``original`` except the four
                 names tests.py:34-39 takes from ``numba``, plus the ``numba``
                 outputs of the functions whose signatures differ.
* ``cfg1``     — the small benchmark configuration (K=2000, 30x30 at 0.1",
                 r=1.2", 16x16 bilinear source, lambda=1) through ``numba``.
* ``edge``     — a tiny case with ragged (-1 padded) mapping rows, a repeated
                 source index in a row, and ragged neighbour rows, through
                 ``numba``; plus likelihoods at two other regularisation
                 coefficients assembled from the reference's own functions.
"""

from __future__ import annotations

import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "python-autojax_gb300"))


def _install_numba_shim():
    try:
        import numba  # noqa: F401

        return
    except ImportError:
        pass
    shim = types.ModuleType("numba")

    def jit(*args, **kwargs):
        if len(args) == 1 and callable(args[0]) and not kwargs:
            return args[0]
        return lambda f: f

    shim.jit = jit
    shim.njit = jit
    shim.prange = range
    sys.modules["numba"] = shim


def _import_reference(ref_root: Path):
    _install_numba_shim()
    sys.path.insert(0, str(ref_root / "src"))
    from autojax import numba as ref_numba
    from autojax import original as ref_original

    return ref_numba, ref_original


def _call(func, d):
    import inspect

    sig = inspect.signature(func)
    return func(*[d[k] for k in sig.parameters])


REF_TESTS = [
    "constant_regularization_matrix_from",
    "curvature_matrix_via_w_compact_sparse_mapping_matrix_from",
    "curvature_matrix_via_w_tilde_curvature_preload_interferometer_from",
    "curvature_matrix_via_w_tilde_from",
    "data_vector_from",
    "log_likelihood_function_via_w_compact_from",
    "log_likelihood_function_via_w_tilde_from",
    "mapping_matrix_from",
    "mask_2d_circular_from",
    "noise_normalization_complex_from",
    "reconstruction_positive_negative_from",
    "sparse_mapping_matrix_transpose_matmul",
    "w_compact_curvature_interferometer_from",
    "w_tilde_curvature_interferometer_from",
    "w_tilde_curvature_preload_interferometer_from",
    "w_tilde_data_interferometer_from",
    "w_tilde_via_compact_from",
    "w_tilde_via_preload_from",
]
REF_TESTS_NUMBA = {
    "curvature_matrix_via_w_compact_sparse_mapping_matrix_from",
    "sparse_mapping_matrix_transpose_matmul",
    "w_compact_curvature_interferometer_from",
    "w_tilde_via_compact_from",
}
# numba.py functions whose outputs are recorded under "numba__<name>"
NUMBA_FUNCS = [
    "mask_2d_circular_from",
    "w_tilde_data_interferometer_from",
    "w_tilde_curvature_interferometer_from",
    "w_compact_curvature_interferometer_from",
    "w_tilde_via_compact_from",
    "w_tilde_via_preload_from",
    "mapping_matrix_from",
    "data_vector_from",
    "curvature_matrix_via_w_tilde_from",
    "curvature_matrix_via_w_compact_sparse_mapping_matrix_direct_from",
    "_w_compact_matmul_sparse_mapping_matrix_from",
    "sparse_mapping_matrix_transpose_matmul",
    "curvature_matrix_via_w_wilde_sparse_mapping_matrix_from",
    "curvature_matrix_via_w_compact_sparse_mapping_matrix_from",
    "constant_regularization_matrix_from",
    "reconstruction_positive_negative_from",
    "noise_normalization_complex_from",
    "log_likelihood_function_via_w_tilde_from",
    "log_likelihood_function_via_w_compact_from",
]
INPUT_KEYS = [
    "grid_size",
    "pixel_scale",
    "pixel_scales",
    "centre",
    "radius",
    "shape_native",
    "shape_masked_pixels_2d",
    "coefficient",
    "pixels",
    "real_space_mask",
    "native_index_for_slim_index",
    "grid_radians_2d",
    "grid_radians_slim",
    "dirty_image",
    "uv_wavelengths",
    "pix_indexes_for_sub_slim_index",
    "pix_weights_for_sub_slim_index",
    "pix_size_for_sub_slim_index",
    "slim_index_for_sub_slim_index",
    "sub_fraction",
    "neighbors",
    "neighbors_sizes",
    "data",
    "noise_map",
    "noise_map_real",
    "visibilities_real",
]


def _complete(d: dict, ref_numba, ref_original) -> dict:
    """Add the derived inputs that the reference's fixture computes (tests.py:255-394)."""
    d = dict(d)
    S = d["pixels"]
    M = d["grid_radians_slim"].shape[0]
    d.setdefault("pix_pixels", S)
    d.setdefault("total_mask_pixels", M)
    # entries before the first -1, so original.py's pix_size loops see the rows numba.py's breaks see
    d.setdefault("pix_size_for_sub_slim_index", np.cumprod(np.asarray(d["pix_indexes_for_sub_slim_index"]) != -1, axis=1).sum(axis=1))
    d.setdefault("slim_index_for_sub_slim_index", np.arange(M))
    d.setdefault("sub_fraction", np.ones(M))
    d.setdefault("pixel_scales", (d["pixel_scale"], d["pixel_scale"]))
    d.setdefault("centre", (0.0, 0.0))
    d.setdefault("shape_masked_pixels_2d", (d["grid_size"], d["grid_size"]))
    d.setdefault("coefficient", 1.0)
    d["mapping_matrix"] = ref_numba.mapping_matrix_from(d["pix_indexes_for_sub_slim_index"], d["pix_weights_for_sub_slim_index"], S)
    d["matrix"] = d["mapping_matrix"]
    d["w_tilde"] = ref_numba.w_tilde_curvature_interferometer_from(d["noise_map_real"], d["uv_wavelengths"], d["grid_radians_slim"])
    d["w_compact"] = ref_numba.w_compact_curvature_interferometer_from(d["grid_size"], d["noise_map_real"], d["uv_wavelengths"], d["pixel_scale"])
    d["w_tilde_preload"] = ref_original.w_tilde_curvature_preload_interferometer_from(
        d["noise_map_real"], d["uv_wavelengths"], d["shape_masked_pixels_2d"], d["grid_radians_2d"]
    )
    d["curvature_preload"] = d["w_tilde_preload"]
    d["data_vector"] = ref_numba.data_vector_from(d["mapping_matrix"], d["dirty_image"])
    F = ref_numba.curvature_matrix_via_w_tilde_from(d["w_tilde"], d["mapping_matrix"])
    H = ref_numba.constant_regularization_matrix_from(d["coefficient"], d["neighbors"], d["neighbors_sizes"])
    d["curvature_reg_matrix"] = F + H
    return d


def _outputs(d, ref_numba, ref_original, with_original: bool) -> dict:
    out = {}
    for name in NUMBA_FUNCS:
        out["numba__" + name] = np.asarray(_call(getattr(ref_numba, name), d))
        print("  numba", name, flush=True)
    if with_original:
        for name in REF_TESTS:
            if name == "w_tilde_curvature_interferometer_from":
                # original.py:166-226 is an O(M^2 K) pure-Python loop without numba; the
                # reference's tests accept numba's vectorised form at rtol 5e-6 (tests.py:631)
                out["ref__" + name] = out["numba__" + name]
                continue
            mod = ref_numba if name in REF_TESTS_NUMBA else ref_original
            out["ref__" + name] = np.asarray(_call(getattr(mod, name), d))
            print("  ref", name, flush=True)
    out["original__w_tilde_curvature_preload_interferometer_from"] = d["w_tilde_preload"]
    out["original__curvature_matrix_via_w_tilde_curvature_preload_interferometer_from"] = np.asarray(
        _call(ref_original.curvature_matrix_via_w_tilde_curvature_preload_interferometer_from, d)
    )
    out["original__mapping_matrix_from"] = np.asarray(_call(ref_original.mapping_matrix_from, d))
    out["original__w_tilde_via_preload_from"] = np.asarray(_call(ref_original.w_tilde_via_preload_from, d))
    return out


def _likelihood_at(d, ref_numba, coefficient: float) -> float:
    """numba.py:818-857 with the regularisation coefficient changed (the reference hard-codes 1.0)."""
    S = d["neighbors_sizes"].size
    T = ref_numba.mapping_matrix_from(d["pix_indexes_for_sub_slim_index"], d["pix_weights_for_sub_slim_index"], S)
    F = ref_numba.curvature_matrix_via_w_tilde_from(d["w_tilde"], T)
    H = ref_numba.constant_regularization_matrix_from(coefficient, d["neighbors"], d["neighbors_sizes"])
    A = F + H
    D = ref_numba.data_vector_from(T, d["dirty_image"])
    s = ref_numba.reconstruction_positive_negative_from(D, A)
    chi = d["data"].view(np.float64) / d["noise_map"].view(np.float64)
    return float(
        -0.5
        * (
            chi @ chi
            - s @ D
            + np.linalg.slogdet(A)[1]
            - np.linalg.slogdet(H)[1]
            + ref_numba.noise_normalization_complex_from(d["noise_map"])
        )
    )


def fingerprint(a: np.ndarray, seed: int = 12345) -> dict:
    """Size-independent fingerprint of a large matrix: sampled rows and random projections.

    A matrix that matches 16 sampled rows and its products with 4 random vectors
    from both sides matches the reference everywhere up to the test tolerance
    (any single wrong entry moves a projection).
    """
    a = np.asarray(a, dtype=np.float64)
    rng = np.random.default_rng(seed)
    rows = np.unique(np.linspace(0, a.shape[0] - 1, 16).astype(np.int64))
    return {
        "rows_idx": rows,
        "rows": a[rows],
        "proj": a @ rng.standard_normal((a.shape[1], 4)),
        "projT": a.T @ rng.standard_normal((a.shape[0], 4)),
    }


BIG = 60_000


def _save(name: str, d: dict, out: dict):
    payload = {}
    for k in INPUT_KEYS:
        if k in d:
            payload["in__" + k] = np.asarray(d[k])
    # the solve is ill-conditioned: its own inputs are kept bit-exact
    for k in ("curvature_reg_matrix", "data_vector"):
        payload["in__" + k] = np.asarray(d[k])
    for k, v in out.items():
        v = np.asarray(v)
        if v.dtype.kind == "f" and v.size > BIG and v.ndim == 2:
            for fk, fv in fingerprint(v).items():
                payload[f"fp__{k}__{fk}"] = fv
        else:
            payload[k] = v
    np.savez_compressed(HERE / f"{name}.npz", **payload)
    print("wrote", name, sum(v.nbytes for v in payload.values()) / 1e6, "MB raw", flush=True)


def make_edge(rng_seed: int = 7):
    """Ragged mapping rows, a repeated index, ragged neighbour rows, on a tiny grid."""
    from autojax_gb300 import synthetic

    rng = np.random.default_rng(rng_seed)
    N, ps = 8, 0.3
    mask = synthetic.mask_circular(N, ps, 1.1)
    native = np.ascontiguousarray(np.argwhere(~mask).astype(np.int64))
    g2d = synthetic.grid_radians_2d(N, ps)
    slim = np.ascontiguousarray(g2d[~mask])
    M = slim.shape[0]
    K, S, B = 50, 12, 4
    uv = synthetic.annulus_uv(rng, K, 1e3, 2e5)
    sigma = np.exp(np.log(0.3) + 0.5 * rng.standard_normal(K))
    noise = sigma + 1j * sigma
    data = rng.standard_normal(K) + 1j * rng.standard_normal(K)
    pidx = rng.integers(0, S, size=(M, B)).astype(np.int64)
    pw = rng.uniform(0.05, 1.0, size=(M, B))
    pidx[3, 2:] = -1  # ragged row
    pidx[5, 1:] = -1  # single entry
    pidx[7, 1] = -1  # entries after the first -1 are ignored
    pidx[7, 2] = 4
    pidx[9, 3] = pidx[9, 0]  # repeated index: assign keeps the last, sums add both
    # symmetric neighbour graph on a ring plus chords, ragged rows
    nbl = [set() for _ in range(S)]
    for s in range(S):
        for t in ((s + 1) % S, (s + 5) % S):
            nbl[s].add(t)
            nbl[t].add(s)
    P = max(len(x) for x in nbl) + 1
    nb = -np.ones((S, P), dtype=np.int64)
    for s in range(S):
        v = sorted(nbl[s])
        nb[s, : len(v)] = v
    nsz = (nb != -1).sum(axis=1)
    return {
        "grid_size": N,
        "pixel_scale": ps,
        "radius": 1.1,
        "shape_native": (N, N),
        "real_space_mask": mask,
        "native_index_for_slim_index": native,
        "grid_radians_2d": g2d,
        "grid_radians_slim": slim,
        "uv_wavelengths": uv,
        "noise_map": noise,
        "noise_map_real": np.ascontiguousarray(noise.real),
        "data": data,
        "visibilities_real": np.ascontiguousarray(data.real),
        "dirty_image": rng.standard_normal(M),
        "pix_indexes_for_sub_slim_index": pidx,
        "pix_weights_for_sub_slim_index": pw,
        "neighbors": nb,
        "neighbors_sizes": nsz,
        "pixels": S,
    }


def write_signatures(ref_numba, ref_original):
    """Parameter lists of every public function of numba.py and original.py (util/mod_diff.py:25-57 idea)."""
    import inspect
    import json

    out = {}
    for modname, mod in (("numba", ref_numba), ("original", ref_original)):
        sigs = {}
        for name, obj in vars(mod).items():
            if callable(obj) and getattr(obj, "__module__", "") == mod.__name__:
                sigs[name] = list(inspect.signature(obj).parameters)
        # module-level aliases (numba.py:651-653)
        for name, obj in vars(mod).items():
            if callable(obj) and name not in sigs and getattr(obj, "__module__", "") == mod.__name__:
                sigs[name] = list(inspect.signature(obj).parameters)
        if modname == "numba":
            sigs["curvature_matrix_via_w_tilde_curvature_preload_interferometer_from"] = list(
                inspect.signature(mod.curvature_matrix_via_w_tilde_curvature_preload_interferometer_from).parameters
            )
        out[modname] = dict(sorted(sigs.items()))
    (HERE / "reference_signatures.json").write_text(json.dumps(out, indent=1) + "\n")
    print("wrote reference_signatures.json", flush=True)


def main(ref_root: str):
    ref_numba, ref_original = _import_reference(Path(ref_root))
    write_signatures(ref_numba, ref_original)
    if "--signatures-only" in sys.argv:
        return
    from oracle import refdata
    from autojax_gb300 import synthetic

    print("case refgen", flush=True)
    d = _complete(refdata.DataGenerated().arrays, ref_numba, ref_original)
    out = _outputs(d, ref_numba, ref_original, with_original=True)
    _save("refgen", d, out)

    print("case cfg1", flush=True)
    c = synthetic.make_dataset("cfg1")
    c = {k: v for k, v in c.items() if k not in ("config", "M", "K", "S")}
    c["shape_native"] = (c["grid_size"], c["grid_size"])
    c["radius"] = synthetic.CONFIGS["cfg1"].mask_radius
    c = _complete(c, ref_numba, ref_original)
    out = _outputs(c, ref_numba, ref_original, with_original=False)
    for coef in (0.1, 3.0):
        out[f"numba__log_likelihood_coefficient_{coef}"] = np.asarray(_likelihood_at(c, ref_numba, coef))
    _save("cfg1", c, out)

    print("case edge", flush=True)
    e = _complete(make_edge(), ref_numba, ref_original)
    out = _outputs(e, ref_numba, ref_original, with_original=False)
    for coef in (0.5, 2.0):
        out[f"numba__log_likelihood_coefficient_{coef}"] = np.asarray(_likelihood_at(e, ref_numba, coef))
    _save("edge", e, out)


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    if len(args) != 1:
        sys.exit("usage: make_golden.py <path of the ickc/python-autojax checkout>")
    main(args[0])
