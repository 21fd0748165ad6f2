"""The mixed-precision path (double-float on the float32 pipe) against the float64 oracle.

Tolerances (stated per result, as the mixed path promises): logE rel 1e-8;
dlogE/dlambda within 1e-6 of the scale of its two cancelling traces
(tr(H^-1 L) ~ S / lambda) plus 1e-5 relative; weight gradient 1e-5 of its
largest entry, or 2e-15 cond(A) of it when larger (the gradient goes through
A^-1).  Double-float keeps ~2^-47 per operation; the fixtures reach condition
numbers near 1e11, which is where these bounds come from.
"""

from __future__ import annotations

import numpy as np
import pytest

import golden_util as gu
from oracle import adjoint

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def aj():
    import autojax_gb300

    return autojax_gb300


def _args(d):
    return (d["dirty_image"], d["data"], d["noise_map"], d["w_tilde"], d["pix_indexes_for_sub_slim_index"],
            d["pix_weights_for_sub_slim_index"], d["neighbors"], d["neighbors_sizes"])


@pytest.mark.parametrize("case", gu.CASES)
@pytest.mark.parametrize("coef", [0.05, 1.0, 20.0])
def test_mixed_matches_oracle(aj, case, coef):
    d = gu.full_inputs(case)
    logE, dlam, gw = aj.log_evidence_and_grad(*_args(d), coefficient=coef, precision="mixed")
    r_logE, r_dlam, r_gw = adjoint.log_evidence_and_grad(*_args(d), coefficient=coef)
    assert abs(logE - r_logE) <= 1e-8 * abs(r_logE), (logE, r_logE)
    trace_scale = d["pixels"] / coef**2
    assert abs(dlam - r_dlam) <= 1e-6 * trace_scale + 1e-5 * abs(r_dlam), (dlam, r_dlam)
    # the weight gradient goes through A^-1: its error scales with cond(A) (refgen reaches ~1e11)
    from oracle import numpy_port as ref

    T = ref.mapping_matrix_from(d["pix_indexes_for_sub_slim_index"], d["pix_weights_for_sub_slim_index"], d["pixels"])
    ev = np.linalg.eigvalsh(T.T @ d["w_tilde"] @ T + ref.constant_regularization_matrix_from(coef, d["neighbors"],
                                                                                              d["neighbors_sizes"]))
    cond = ev[-1] / ev[0]
    np.testing.assert_allclose(gw, r_gw, rtol=0, atol=max(1e-5, 2e-15 * cond) * np.abs(r_gw).max())


@pytest.mark.parametrize("case", ["cfg1", "edge"])
def test_mixed_compact_matches_oracle(aj, case):
    d = gu.full_inputs(case)
    a = _args(d)
    got = aj.log_likelihood_function_via_w_compact_from(a[0], a[1], a[2], d["w_compact"],
                                                        d["native_index_for_slim_index"], *a[4:], precision="mixed")
    exp = float(gu.expected(case, "numba__log_likelihood_function_via_w_compact_from"))
    assert abs(got - exp) <= 1e-8 * abs(exp)


def test_evaluator_graph_replay_matches_direct(aj):
    import torch

    from autojax_gb300.inversion import LogEvidence

    d = gu.full_inputs("cfg1")
    a = _args(d)
    ev = LogEvidence(a[0], a[1], a[2], a[3], S=d["pixels"], B=a[4].shape[1], P=a[6].shape[1], precision="mixed")
    ev.set_model(a[4], a[5], a[6], a[7], coefficient=0.7)
    ev.capture()
    for coef in (0.7, 0.2, 3.0):
        logE, dlam, gw = ev.evaluate_host(a[4], a[5], a[6], a[7], coef)
        r = adjoint.log_evidence_and_grad(*a, coefficient=coef)
        assert abs(logE - r[0]) <= 1e-8 * abs(r[0])
        assert abs(dlam - r[1]) <= 1e-7 * d["pixels"] / coef**2 + 1e-6 * abs(r[1])
    assert ev.launches_per_eval and ev.launches_per_eval > 10


def test_evaluate_host_reports_bad_index_then_recovers(aj):
    """The end-to-end call reads the info word from its one device-to-host copy: an out-of-range
    mapping index raises IndexError, and the next good call through the same graph is exact."""
    from autojax_gb300.inversion import LogEvidence

    d = gu.full_inputs("cfg1")
    a = _args(d)
    ev = LogEvidence(a[0], a[1], a[2], a[3], S=d["pixels"], B=a[4].shape[1], P=a[6].shape[1], precision="mixed")
    ev.set_model(a[4], a[5], a[6], a[7], coefficient=0.7)
    ev.capture()
    bad = a[4].copy()
    bad[3, 1] = d["pixels"]
    with pytest.raises(IndexError, match=str(3 * a[4].shape[1] + 1)):
        ev.evaluate_host(bad, a[5], a[6], a[7], 0.7)
    logE, dlam, gw = ev.evaluate_host(a[4], a[5], a[6], a[7], 0.7)
    r = adjoint.log_evidence_and_grad(*a, coefficient=0.7)
    assert abs(logE - r[0]) <= 1e-8 * abs(r[0])
    assert gw.shape == a[4].shape
    assert ev.h2d_bytes() >= (a[4].size * 2 + a[6].size + d["pixels"] + 1) * 8
    assert ev.d2h_bytes() == (4 + a[4].size) * 8


def test_autograd_function(aj):
    import torch

    from autojax_gb300.inversion import LogEvidence, log_evidence

    d = gu.full_inputs("edge")
    a = _args(d)
    ev = LogEvidence(a[0], a[1], a[2], a[3], S=d["pixels"], B=a[4].shape[1], P=a[6].shape[1], precision="fp64")
    ev.set_model(a[4], a[5], a[6], a[7], coefficient=1.0)
    w = torch.tensor(a[5], device="cuda", requires_grad=True)
    c = torch.tensor(1.3, dtype=torch.float64, device="cuda", requires_grad=True)
    out = log_evidence(w, c, ev)
    out.backward()
    r = adjoint.log_evidence_and_grad(*a, coefficient=1.3)
    assert abs(float(out) - r[0]) <= 1e-10 * abs(r[0])
    np.testing.assert_allclose(w.grad.cpu().numpy(), r[2], rtol=1e-8, atol=1e-9 * np.abs(r[2]).max())
    assert abs(float(c.grad) - 2 * 1.3 * r[1]) <= 1e-7 * max(1.0, abs(2 * 1.3 * r[1]))


@pytest.mark.parametrize("M,K", [(33, 65), (448, 2000), (300, 7)])
def test_mixed_w_tilde_matches_oracle(aj, M, K):
    """The double-float w_tilde build: float64 panel, double-float product (~1e-13 relative)."""
    from oracle import numpy_port as ref

    rng = np.random.default_rng(M + K)
    g = rng.standard_normal((M, 2)) * 1e-5
    uv = rng.uniform(-5e5, 5e5, (K, 2))
    n = rng.uniform(0.1, 1.0, K)
    W, P = aj.w_tilde_curvature_interferometer_from(n, uv, g, precision="mixed", planes=True)
    exp = ref.w_tilde_curvature_interferometer_from(n, uv, g)
    scale = np.abs(exp).max()
    np.testing.assert_allclose(W, exp, rtol=0, atol=1e-12 * scale)
    np.testing.assert_allclose(P[0].astype(np.float64) + P[1].astype(np.float64), W, rtol=0, atol=1e-15 * scale)


def _spd_with_condition(S, cond, seed):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.standard_normal((S, S)))
    ev = np.logspace(0.0, np.log10(cond), S)
    return (Q * ev) @ Q.T


@pytest.mark.parametrize("S", [1, 31, 32, 33, 100, 257, 1000])
def test_mixed_spd_inverse_matches_numpy(S):
    """aj_spd_inverse_mixed (double-float Cholesky, L^-1 and L^-T L^-1) against float64 LAPACK.

    Tolerance: each double-float operation keeps ~2^-47, so the inverse is good
    to ~S 2^-47 cond(A) of its largest entry; log det to ~S 2^-47 cond(A).
    """
    import torch

    from autojax_gb300 import _lib

    lib = _lib.load()
    cond = 1e6
    A = _spd_with_condition(S, cond, 7 + S)
    At = torch.from_numpy(A).cuda()
    inv = torch.empty_like(At)
    logdet = torch.zeros(1, dtype=torch.float64, device="cuda")
    info = torch.zeros(2, dtype=torch.int32, device="cuda")
    ws = torch.empty(lib.aj_spd_inverse_mixed_workspace_size(S), dtype=torch.uint8, device="cuda")
    _lib.check(lib.aj_spd_inverse_mixed(At.data_ptr(), S, inv.data_ptr(), logdet.data_ptr(), ws.data_ptr(),
                                        ws.numel(), info.data_ptr(), torch.cuda.current_stream().cuda_stream),
               "aj_spd_inverse_mixed")
    torch.cuda.synchronize()
    assert int(info[0]) == 0
    ref = np.linalg.inv(A)
    got = inv.cpu().numpy()
    tol = max(S, 32) * 2.0**-47 * cond * np.abs(ref).max()
    assert np.abs(got - ref).max() <= tol
    assert np.abs(got - got.T).max() == 0.0
    sign, ld = np.linalg.slogdet(A)
    assert sign > 0
    assert abs(float(logdet[0]) - ld) <= max(S, 32) * 2.0**-47 * cond * max(1.0, abs(ld))


@pytest.mark.parametrize("S", [130, 600, 1500])
def test_mixed_spd_inverse_with_graded_scales(S):
    """A = D B D with D = diag(2^u), u in [-20, 20]: the columns of L^-1 span 2^80, so the tensor-core
    L^-T L^-1 (digits cut per column at its own power of two, groups above a tile's first row
    skipped) must keep each entry to its own scale, |err_ij| <= tol sqrt(A^-1_ii A^-1_jj), with
    tol ~ S 2^-46 cond(B) (the double-float bound of the factorisation and inverse)."""
    import torch

    from autojax_gb300 import _lib

    lib = _lib.load()
    rng = np.random.default_rng(S)
    cond = 1e3
    Bm = _spd_with_condition(S, cond, 100 + S)
    d = 2.0 ** rng.integers(-20, 21, size=S).astype(np.float64)
    A = (d[:, None] * Bm) * d[None, :]
    At = torch.from_numpy(A).cuda()
    inv = torch.empty_like(At)
    logdet = torch.zeros(1, dtype=torch.float64, device="cuda")
    info = torch.zeros(2, dtype=torch.int32, device="cuda")
    ws = torch.empty(lib.aj_spd_inverse_mixed_workspace_size(S), dtype=torch.uint8, device="cuda")
    _lib.check(lib.aj_spd_inverse_mixed(At.data_ptr(), S, inv.data_ptr(), logdet.data_ptr(), ws.data_ptr(),
                                        ws.numel(), info.data_ptr(), torch.cuda.current_stream().cuda_stream),
               "aj_spd_inverse_mixed")
    torch.cuda.synchronize()
    assert int(info[0]) == 0
    ref = (np.linalg.inv(Bm) / d[:, None]) / d[None, :]
    got = inv.cpu().numpy()
    scale = np.sqrt(np.outer(np.diag(ref), np.diag(ref)))
    tol = S * 2.0**-46 * cond
    assert np.max(np.abs(got - ref) / scale) <= tol
    assert np.abs(got - got.T).max() == 0.0


def test_mixed_spd_inverse_reports_not_positive_definite():
    import torch

    from autojax_gb300 import _lib

    lib = _lib.load()
    S = 70
    A = _spd_with_condition(S, 10.0, 3)
    A[40, 40] = -1.0  # leading minor 41 is indefinite
    At = torch.from_numpy(A).cuda()
    inv = torch.empty_like(At)
    logdet = torch.zeros(1, dtype=torch.float64, device="cuda")
    info = torch.zeros(2, dtype=torch.int32, device="cuda")
    ws = torch.empty(lib.aj_spd_inverse_mixed_workspace_size(S), dtype=torch.uint8, device="cuda")
    _lib.check(lib.aj_spd_inverse_mixed(At.data_ptr(), S, inv.data_ptr(), logdet.data_ptr(), ws.data_ptr(),
                                        ws.numel(), info.data_ptr(), torch.cuda.current_stream().cuda_stream),
               "aj_spd_inverse_mixed")
    torch.cuda.synchronize()
    assert int(info[0]) == _lib.AJ_INFO_NOT_POSITIVE_DEFINITE
    assert np.isnan(float(logdet[0]))


@pytest.mark.parametrize("config,K", [("cfg2", 3000)])
def test_mixed_matches_fp64_at_multi_chunk_sizes(aj, config, K):
    """M = 5,024 > 1,024: the double-float gathers run over several column chunks (the golden cases
    have M <= 1,024).  Mixed logE against the float64 path (itself pinned to the oracle) over the
    bench's lambda range."""
    import torch

    from autojax_gb300 import synthetic
    from autojax_gb300.inversion import Dataset, LogEvidence

    d = synthetic.make_dataset(config, K=K)
    dev = torch.device("cuda")
    wc = aj.w_compact_curvature_interferometer_from(d["grid_size"], torch.from_numpy(d["noise_map_real"]).to(dev),
                                                    torch.from_numpy(d["uv_wavelengths"]).to(dev), d["pixel_scale"])
    W = aj.w_tilde_via_compact_from(wc, torch.from_numpy(d["native_index_for_slim_index"]).to(dev))
    B, P = d["pix_indexes_for_sub_slim_index"].shape[1], d["neighbors"].shape[1]
    ev = {p: LogEvidence(S=d["S"], B=B, P=P, precision=p,
                         dataset=Dataset(d["dirty_image"], d["data"], d["noise_map"], W, precision=p))
          for p in ("mixed", "fp64")}
    for lam in (1e-3, 1e-1, 1e1, 1e3):
        out = {}
        for p, e in ev.items():
            e.set_model(d["pix_indexes_for_sub_slim_index"], d["pix_weights_for_sub_slim_index"], d["neighbors"],
                        d["neighbors_sizes"], np.sqrt(lam))
            e.launch()
            torch.cuda.synchronize()
            e.check()
            out[p] = e.out.cpu().numpy().copy()
        assert abs(out["mixed"][0] - out["fp64"][0]) <= 1e-7 * abs(out["fp64"][0]), (lam, out)


@pytest.mark.parametrize("M,S", [(1028, 997), (1032, 7), (1030, 257)])
def test_mixed_curvature_gather_edges(aj, M, S):
    """The mixed F through the double-float gathers against the float64 products, on inputs that
    reach their edge cases: an odd source-pixel count (the transposed gather's last block holds a
    single pixel), source pixels with more entries than one staging pass (several passes and a
    padded last group of four), rows ended early by -1 and repeated indices, and M not a multiple
    of 4 (the untransposed gather, then a transpose)."""
    rng = np.random.default_rng(M + S)
    W = rng.standard_normal((M, M))
    W = (W + W.T) / 2
    idx = rng.integers(0, S, size=(M, 3))
    idx[:300, 0] = 0  # source pixel 0 gets at least 300 entries
    idx[::7, 2] = -1
    w = rng.random((M, 3))
    F = aj.curvature_matrix_via_w_wilde_sparse_mapping_matrix_from(W, idx, w, S, precision="mixed")
    F64 = aj.curvature_matrix_via_w_wilde_sparse_mapping_matrix_from(W, idx, w, S)
    np.testing.assert_allclose(F, F64, rtol=0, atol=1e-12 * np.abs(F64).max())


def test_mixed_weight_gradient_ragged_rows(aj):
    """S = 101 (Omega's and A^-1's rows are not 16-byte aligned, so the gradient takes its scalar
    loads) and mapping rows padded to B = 7: later repeats that overwrite earlier entries, entries
    after an early -1, and rows with more live entries than one pass of the per-pixel products takes."""
    import torch

    from autojax_gb300 import synthetic

    cfg = synthetic.Config("ragged", 500, 30, 0.1, 1.2, 101, "delaunay", 0.8, 1.5, 1.0, 11)
    d = synthetic.make_dataset(cfg)
    S = d["S"]
    assert S % 4 != 0
    dev = torch.device("cuda")
    wc = aj.w_compact_curvature_interferometer_from(d["grid_size"], torch.from_numpy(d["noise_map_real"]).to(dev),
                                                    torch.from_numpy(d["uv_wavelengths"]).to(dev), d["pixel_scale"])
    W = aj.w_tilde_via_compact_from(wc, torch.from_numpy(d["native_index_for_slim_index"]).to(dev)).cpu().numpy()
    idx3, w3 = d["pix_indexes_for_sub_slim_index"], d["pix_weights_for_sub_slim_index"]
    M = idx3.shape[0]
    rng = np.random.default_rng(5)
    idx = np.full((M, 7), -1, np.int64)
    wts = np.zeros((M, 7))
    idx[:, :3], wts[:, :3] = idx3, w3
    for m in range(M):
        kind = m % 4
        if kind == 1:  # a repeat overwrites the earlier entry
            idx[m, 3:5] = [idx3[m, 0], rng.integers(S)]
            wts[m, 3:5] = rng.uniform(0.05, 0.5, 2)
        elif kind == 2:  # entries after an early -1 are ignored
            idx[m, 4:6] = rng.integers(S, size=2)
            wts[m, 4:6] = 0.4
        elif kind == 3:  # six live entries: a second pass of the dot products
            idx[m, 3:6] = [rng.integers(S), idx3[m, 1], rng.integers(S)]
            wts[m, 3:6] = rng.uniform(0.05, 0.3, 3)
    args = (d["dirty_image"], d["data"], d["noise_map"], W, idx, wts, d["neighbors"], d["neighbors_sizes"])
    coef = 0.5
    logE, dlam, gw = aj.log_evidence_and_grad(*args, coefficient=coef, precision="mixed")
    r_logE, r_dlam, r_gw = adjoint.log_evidence_and_grad(*args, coefficient=coef)
    assert abs(logE - r_logE) <= 1e-8 * abs(r_logE), (logE, r_logE)
    from oracle import numpy_port as ref

    T = ref.mapping_matrix_from(idx, wts, S)
    ev = np.linalg.eigvalsh(T.T @ W @ T + ref.constant_regularization_matrix_from(coef, d["neighbors"],
                                                                                   d["neighbors_sizes"]))
    cond = ev[-1] / ev[0]
    assert np.all(gw[idx == -1] == 0) and np.all(gw[:, 3:][(np.arange(M) % 4 == 2)] == 0)
    np.testing.assert_allclose(gw, r_gw, rtol=0, atol=max(1e-5, 2e-15 * cond) * np.abs(r_gw).max())


def test_tile_policy_does_not_change_results():
    """The 64 x 64 and 32 x 32 tile kernels add in the same order: any tile policy gives the same bits."""
    import torch

    from autojax_gb300 import _lib, tune

    lib = _lib.load()
    S = 700
    A = torch.from_numpy(_spd_with_condition(S, 1e5, 11)).cuda()
    ws = torch.empty(lib.aj_spd_inverse_mixed_workspace_size(S), dtype=torch.uint8, device="cuda")
    saved = tune.get_tile_policy()
    outs = []
    try:
        for pol in ((1, 1), (tune.NEVER,) * 2, (40, 200)):
            tune.set_tile_policy(*pol)
            inv = torch.empty_like(A)
            ld = torch.zeros(1, dtype=torch.float64, device="cuda")
            info = torch.zeros(2, dtype=torch.int32, device="cuda")
            _lib.check(lib.aj_spd_inverse_mixed(A.data_ptr(), S, inv.data_ptr(), ld.data_ptr(), ws.data_ptr(),
                                                ws.numel(), info.data_ptr(), torch.cuda.current_stream().cuda_stream),
                       "aj_spd_inverse_mixed")
            torch.cuda.synchronize()
            outs.append((inv.clone(), ld.clone()))
    finally:
        tune.set_tile_policy(*saved)
    for inv, ld in outs[1:]:
        assert torch.equal(inv, outs[0][0]) and torch.equal(ld, outs[0][1])


def _spd_inverse_mixed(A):
    import torch

    from autojax_gb300 import _lib

    lib = _lib.load()
    S = A.shape[0]
    At = torch.from_numpy(np.ascontiguousarray(A)).cuda()
    inv = torch.empty_like(At)
    logdet = torch.zeros(1, dtype=torch.float64, device="cuda")
    info = torch.zeros(2, dtype=torch.int32, device="cuda")
    ws = torch.empty(lib.aj_spd_inverse_mixed_workspace_size(S), dtype=torch.uint8, device="cuda")
    _lib.check(lib.aj_spd_inverse_mixed(At.data_ptr(), S, inv.data_ptr(), logdet.data_ptr(), ws.data_ptr(),
                                        ws.numel(), info.data_ptr(), torch.cuda.current_stream().cuda_stream),
               "aj_spd_inverse_mixed")
    torch.cuda.synchronize()
    assert int(info[0]) == 0
    return inv.cpu().numpy(), float(logdet[0])


@pytest.mark.parametrize("S", [96, 257, 500])
def test_mixed_spd_inverse_graded(S):
    """A = D B D with D spanning 1e-3 .. 1e3 (a graded matrix, cond(A) ~ 1e12 cond(B)).

    The panel's pre-update cuts each row of L into 8-bit digits relative to that row's largest
    entry; L = D chol(B) is graded by rows only, so the factorisation keeps the accuracy of B:
    each entry of A^-1 = D^-1 B^-1 D^-1 to ~S 2^-47 cond(B) of its own scale max|B^-1| / (d_i d_j),
    and log|A| to ~S 2^-47 cond(B).
    """
    cond = 1e6
    B = _spd_with_condition(S, cond, 101 + S)
    d = np.logspace(-3.0, 3.0, S)[np.random.default_rng(5).permutation(S)]
    A = (d[:, None] * B) * d[None, :]
    got, ld = _spd_inverse_mixed(A)
    ref = (np.linalg.inv(B) / d[:, None]) / d[None, :]
    scale = np.abs(np.linalg.inv(B)).max() / np.outer(d, d)
    tol = max(S, 32) * 2.0**-47 * cond
    assert np.max(np.abs(got - ref) / scale) <= tol
    ld_ref = np.linalg.slogdet(B)[1] + 2.0 * np.log(d).sum()
    assert abs(ld - ld_ref) <= tol * max(1.0, abs(ld_ref))


def test_mixed_spd_inverse_ill_conditioned():
    """cond(A) = 1e10 at S = 500 (16 panels through the tensor-core pre-update): the inverse to
    ~S 2^-47 cond(A) of its largest entry and log|A| to ~S 2^-47 cond(A), as for a double-float
    factorisation."""
    S, cond = 500, 1e10
    A = _spd_with_condition(S, cond, 77)
    got, ld = _spd_inverse_mixed(A)
    ref = np.linalg.inv(A)
    tol = S * 2.0**-47 * cond
    assert np.abs(got - ref).max() <= tol * np.abs(ref).max()
    # |d log|A|| = |tr(A^-1 dA)| <= S cond(A) |dA| / |A|
    assert abs(ld - np.linalg.slogdet(A)[1]) <= S * 2.0**-47 * cond
