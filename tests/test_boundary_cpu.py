"""The C-ABI boundary without a GPU: the library builds, loads, and exports every declared symbol;
the Python API keeps the reference's names and parameter lists."""

from __future__ import annotations

import inspect
import json
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "autojax_gb300.h"


def _declared_functions() -> set[str]:
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"\b(aj_[a-z0-9_]+)\s*\(", text)) - {"aj_problem"}


@pytest.fixture(scope="module")
def lib_path():
    from autojax_gb300 import build

    return build.build()


def test_library_exports_every_declared_symbol(lib_path):
    import ctypes

    lib = ctypes.CDLL(str(lib_path))
    missing = [name for name in sorted(_declared_functions()) if not hasattr(lib, name)]
    assert not missing, missing


def test_python_binding_covers_the_header(lib_path):
    from autojax_gb300 import _lib

    assert set(_lib.SIGNATURES) == _declared_functions()
    lib = _lib.load()
    assert lib.aj_version().decode().startswith("autojax_gb300")


def test_status_codes_match_header():
    from autojax_gb300 import _lib

    text = HEADER.read_text()
    for name in ("AJ_OK", "AJ_ERR_ARG", "AJ_ERR_CUDA", "AJ_ERR_WORKSPACE", "AJ_ERR_TOO_LARGE", "AJ_INFO_INDEX_RANGE",
                 "AJ_INFO_NOT_POSITIVE_DEFINITE", "AJ_INFO_SINGULAR", "AJ_FP64", "AJ_MIXED", "AJ_NOALLOC_SOLVE_MAX_S", "AJ_BATCH_BRANCHES"):
        m = re.search(rf"#define {name} \(?(-?\d+)\)?", text)
        assert m, name
        assert getattr(_lib, name) == int(m.group(1)), name


def test_workspace_sizes_are_callable_without_a_device(lib_path):
    from autojax_gb300 import _lib

    lib = _lib.load()
    assert lib.aj_spd_solve_workspace_size(1500) > 1500 * 1500 * 8
    assert lib.aj_sparse_workspace_size(9504, 3, 1500, 9504) > 0
    p = _lib.Problem(M=448, K=2000, S=256, B=4, P=4, N=0)
    # an incomplete problem (no pointers) sizes to 0 instead of crashing
    assert lib.aj_log_evidence_workspace_size(p, 0, 1) == 0


def test_api_keeps_reference_names_and_parameters():
    """mod_diff-style comparison (util/mod_diff.py:25-57) against the recorded reference signatures."""
    import autojax_gb300 as aj

    sigs = json.loads((ROOT / "tests" / "golden" / "reference_signatures.json").read_text())["numba"]
    for name in aj.NUMBA_API:
        assert name in sigs, name
        ours = [p.name for p in inspect.signature(getattr(aj, name)).parameters.values()
                if p.kind in (p.POSITIONAL_ONLY, p.POSITIONAL_OR_KEYWORD)]
        assert ours == sigs[name], (name, ours, sigs[name])
    assert set(aj.NUMBA_API) == set(sigs), set(sigs) ^ set(aj.NUMBA_API)


def test_original_preload_signature():
    import autojax_gb300 as aj

    sigs = json.loads((ROOT / "tests" / "golden" / "reference_signatures.json").read_text())["original"]
    name = "w_tilde_curvature_preload_interferometer_from"
    ours = [p.name for p in inspect.signature(getattr(aj, name)).parameters.values() if p.kind == p.POSITIONAL_OR_KEYWORD]
    assert ours == sigs[name]


def test_calls_fail_loudly_without_a_device():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a device is visible")
    import numpy as np

    import autojax_gb300 as aj

    with pytest.raises(RuntimeError, match="no CUDA device"):
        aj.mapping_matrix_from(np.zeros((2, 3), np.int64), np.zeros((2, 3)), 4)


def test_numpy_dtype_is_checked_like_the_reference_signatures():
    import numpy as np

    import autojax_gb300 as aj

    with pytest.raises(TypeError):
        aj.mapping_matrix_from(np.zeros((2, 3), np.int32), np.zeros((2, 3)), 4)


def test_missing_library_raises_without_fallback(tmp_path, monkeypatch):
    """With the extension not built, the first call raises (there is no CPU path to fall back to)."""
    from autojax_gb300 import _lib

    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "libautojax_gb300.so"))
    with pytest.raises(_lib.LibraryError, match="no CPU fallback"):
        _lib.load()
