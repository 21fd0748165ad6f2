"""The reference's dataset file format (DataLoaded, tests.py:397-452): write, read back, derive sizes."""

from __future__ import annotations

import numpy as np
import pytest


def test_npz_round_trip(tmp_path):
    from autojax_gb300 import data, synthetic

    d = synthetic.make_dataset("cfg1", K=300, seed=2)
    p = tmp_path / "data.npz"
    data.save_npz(p, d)
    got = data.load_npz(p)
    for k in data.NPZ_KEYS:
        np.testing.assert_array_equal(got[k], d[k])
        assert got[k].flags.c_contiguous
    assert (got["M"], got["K"], got["S"], got["P"]) == (d["M"], d["K"], d["S"], d["neighbors"].shape[1])


def test_npz_rejects_missing_and_inconsistent(tmp_path):
    from autojax_gb300 import data, synthetic

    d = synthetic.make_dataset("cfg1", K=50, seed=2)
    p = tmp_path / "bad.npz"
    np.savez(p, **{k: d[k] for k in list(data.NPZ_KEYS)[:-1]})
    with pytest.raises(KeyError):
        data.load_npz(p)
    bad = dict(d)
    bad["dirty_image"] = d["dirty_image"][:-1]
    data.save_npz(p, bad)
    with pytest.raises(ValueError):
        data.load_npz(p)
