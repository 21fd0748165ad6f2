"""The end-to-end call's staging layout (host logic, no device): one buffer of 8-byte slots holds a
model's inputs, each segment 16-byte aligned, none overlapping, and numpy views of a host copy of
the buffer write exactly where the device views of the same layout read."""

from __future__ import annotations

import itertools

import numpy as np
import torch

from autojax_gb300.inversion import staging_layout


def test_segments_are_aligned_disjoint_and_sized():
    for M, B, S, P in itertools.product((1, 5, 448, 9504), (1, 3, 4), (1, 7, 256, 1500), (1, 3, 10)):
        seg, n = staging_layout(M, B, S, P)
        sizes = {"idx": M * B, "w": M * B, "nb": S * P, "nsz": S, "coef": 1}
        spans = sorted((sl.start, sl.stop) for sl in seg.values())
        for name, sl in seg.items():
            assert sl.stop - sl.start == sizes[name], (name, M, B, S, P)
            assert sl.start % 2 == 0  # 16-byte boundary in 8-byte slots
        for (a0, a1), (b0, _) in zip(spans, spans[1:]):
            assert a1 <= b0
        assert spans[-1][1] <= n <= spans[-1][1] + 1


def test_host_views_write_where_device_views_read():
    M, B, S, P = 5, 3, 7, 4
    seg, n = staging_layout(M, B, S, P)
    host = torch.zeros(n, dtype=torch.int64)
    h = host.numpy()
    h_idx = h[seg["idx"]].reshape(M, B)
    h_w = h[seg["w"]].view(np.float64).reshape(M, B)
    h_nb = h[seg["nb"]].reshape(S, P)
    h_nsz = h[seg["nsz"]]
    h_coef = h[seg["coef"]].view(np.float64)
    rng = np.random.default_rng(3)
    idx, w = rng.integers(-1, S, (M, B)), rng.random((M, B))
    nb, nsz = rng.integers(-1, S, (S, 3)), rng.integers(0, 4, S)
    h_idx[...] = idx
    h_w[...] = w
    h_nb[...] = -1
    h_nb[:, :3] = nb
    h_nsz[...] = nsz
    h_coef[0] = 0.37
    # the "device" buffer: a copy of the host one, read through torch views of the same slices
    dev = host.clone()
    assert np.array_equal(dev[seg["idx"]].view(M, B).numpy(), idx)
    assert np.array_equal(dev[seg["w"]].view(torch.float64).view(M, B).numpy(), w)
    got_nb = dev[seg["nb"]].view(S, P).numpy()
    assert np.array_equal(got_nb[:, :3], nb) and (got_nb[:, 3] == -1).all()
    assert np.array_equal(dev[seg["nsz"]].numpy(), nsz)
    assert dev[seg["coef"]].view(torch.float64).item() == 0.37
