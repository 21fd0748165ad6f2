"""Repeated log-evidence evaluations against one resident dataset (the MCMC inner loop).

``LogEvidence`` keeps the dataset (dirty image, visibilities, noise, and the
shared w_tilde or compact table) on the device, owns persistent input buffers
and one workspace, and evaluates logE (and its adjoint) with a single C-ABI
call per evaluation.  ``capture()`` records that call into a CUDA graph so a
step replays ~300 kernel launches as one graph launch; the regularisation
coefficient lives in device memory, so replays may change it.

``LogEvidenceFunction`` exposes the same evaluation to ``torch.autograd`` with
gradients for the mapping weights and the regularisation coefficient.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from ._device import PRECISIONS, precision_code


def _as_dev(x, dtype, device):
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=dtype).contiguous()
    return torch.as_tensor(np.ascontiguousarray(x), dtype=dtype).to(device)


def _complex_real(x, device):
    if isinstance(x, torch.Tensor):
        return torch.view_as_real(x.to(device=device, dtype=torch.complex128).contiguous()).contiguous()
    a = np.ascontiguousarray(x, dtype=np.complex128)
    return torch.from_numpy(a.view(np.float64).reshape(-1, 2)).to(device)


class Dataset:
    """The arrays every evaluation of one observation shares, resident on the device.

    The dirty image (M,), visibilities and noise (K,) complex128, and either
    w_tilde (M, M) or the compact table w_compact (N, 2N-1) with
    native_index_for_slim_index (M, 2), as the reference's likelihoods take
    them (numba.py:761-857, 866-967).  For the mixed path the double-float
    planes of w_tilde are split once here and reused by every evaluation.
    """

    def __init__(self, dirty_image, data, noise_map, w_tilde=None, *, w_compact=None, native_index_for_slim_index=None,
                 precision: str = "mixed", device=None):
        if not torch.cuda.is_available():
            raise RuntimeError("autojax_gb300 needs a CUDA device (it has no CPU path)")
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        dev = self.device
        self.lib = _lib.load()
        self.precision = precision
        self.pc = precision_code(precision)
        self.dirty = _as_dev(dirty_image, torch.float64, dev)
        self.data = _complex_real(data, dev)
        self.noise = _complex_real(noise_map, dev)
        self.M = self.dirty.shape[0]
        self.K = self.data.shape[0]
        self.w_tilde = _as_dev(w_tilde, torch.float64, dev) if w_tilde is not None else None
        self.w_compact = _as_dev(w_compact, torch.float64, dev) if w_compact is not None else None
        self.native = (_as_dev(native_index_for_slim_index, torch.int64, dev)
                       if native_index_for_slim_index is not None else None)
        if self.w_tilde is None and (self.w_compact is None or self.native is None):
            raise ValueError("pass w_tilde, or w_compact with native_index_for_slim_index")
        self.w_hi = self.w_lo = None
        if self.w_tilde is not None and self.pc == _lib.AJ_MIXED:
            self.w_hi = torch.empty(self.w_tilde.shape, dtype=torch.float32, device=dev)
            self.w_lo = torch.empty(self.w_tilde.shape, dtype=torch.float32, device=dev)
            _lib.check(self.lib.aj_split_f64(self.w_tilde.data_ptr(), self.w_tilde.numel(), self.w_hi.data_ptr(),
                                             self.w_lo.data_ptr(), torch.cuda.current_stream(dev).cuda_stream),
                       "aj_split_f64")

    def fill(self, p: _lib.Problem) -> None:
        """Set the shared fields of an aj_problem."""
        p.M, p.K = self.M, self.K
        p.dirty_image = self.dirty.data_ptr()
        p.data = self.data.data_ptr()
        p.noise_map = self.noise.data_ptr()
        if self.w_tilde is not None:
            p.w_tilde64 = self.w_tilde.data_ptr()
            if self.w_hi is not None:
                p.w_tilde_hi = self.w_hi.data_ptr()
                p.w_tilde_lo = self.w_lo.data_ptr()
        else:
            p.w_compact = self.w_compact.data_ptr()
            p.native_index = self.native.data_ptr()
            p.N = self.w_compact.shape[0]


def staging_layout(M: int, B: int, S: int, P: int) -> tuple[dict, int]:
    """Slices of one model's inputs in the buffer of 8-byte slots that an end-to-end call copies at
    once: mapping indexes and weights (M x B), neighbours (S x P), neighbour counts (S) and the
    regularisation coefficient (1).  Each segment starts on a 16-byte boundary.  Returns the
    slices by name ("idx", "w", "nb", "nsz", "coef") and the buffer's length in slots."""
    seg = {}
    n = 0
    for name, size in (("idx", M * B), ("w", M * B), ("nb", S * P), ("nsz", S), ("coef", 1)):
        seg[name] = slice(n, n + size)
        n += size + (size & 1)
    return seg, n


class LogEvidence:
    """Resident-dataset evaluator of the log-evidence and its gradient.

    Parameters mirror ``log_likelihood_function_via_w_tilde_from``
    (numba.py:761-857): pass ``w_tilde`` (M, M), or ``w_compact`` (N, 2N-1)
    with ``native_index_for_slim_index`` for the compact form (numba.py:866-967).
    Shapes of the per-model arrays (M x B mapping, S x P neighbours) are fixed
    at construction by ``B``, ``S`` and ``P``.  Evaluators of several models
    share one ``Dataset`` when it is passed as ``dataset`` (the other dataset
    arguments are then omitted).
    """

    def __init__(self, dirty_image=None, data=None, noise_map=None, w_tilde=None, *, w_compact=None,
                 native_index_for_slim_index=None, S: int, B: int, P: int, precision: str = "mixed",
                 with_grad: bool = True, device=None, dataset: Dataset | None = None):
        if dataset is None:
            dataset = Dataset(dirty_image, data, noise_map, w_tilde, w_compact=w_compact,
                              native_index_for_slim_index=native_index_for_slim_index, precision=precision,
                              device=device)
        elif precision_code(precision) != dataset.pc:
            raise ValueError("precision differs from the dataset's")
        self.dataset = ds = dataset
        self.device = dev = ds.device
        self.lib = ds.lib
        self.precision = ds.precision
        self.pc = ds.pc
        self.with_grad = bool(with_grad)
        self.M, self.K = ds.M, ds.K
        self.S, self.B, self.P = int(S), int(B), int(P)
        # persistent per-model inputs (graph replays read these addresses), views of one buffer of
        # 8-byte slots so an end-to-end call moves them with one copy
        M, B, S, P = self.M, self.B, self.S, self.P
        seg, n_in = staging_layout(M, B, S, P)
        self._in = torch.zeros(n_in, dtype=torch.int64, device=dev)
        self.pix_indexes = self._in[seg["idx"]].view(M, B)
        self.pix_weights = self._in[seg["w"]].view(torch.float64).view(M, B)
        self.neighbors = self._in[seg["nb"]].view(S, P)
        self.neighbors_sizes = self._in[seg["nsz"]]
        self.coefficient = self._in[seg["coef"]].view(torch.float64)
        self.neighbors.fill_(-1)
        self.coefficient.fill_(1.0)
        # outputs, packed likewise: logE and dlogE/dlambda, the info word (two int32), the gradient
        self._outbuf = torch.zeros(4 + M * B, dtype=torch.float64, device=dev)
        self.out = self._outbuf[0:2]
        self.info = self._outbuf[2:3].view(torch.int32)
        self.grad_weights = self._outbuf[4:].view(M, B)
        self.reconstruction = torch.zeros(self.S, dtype=torch.float64, device=dev)
        self.problem = self._problem()
        nbytes = self.lib.aj_log_evidence_workspace_size(self.problem, self.pc, int(self.with_grad))
        if nbytes == 0:
            raise ValueError("inconsistent problem dimensions")
        self.workspace = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        self.graph = None
        self.launches_per_eval = None
        # pinned staging for host inputs/outputs (end-to-end calls), laid out like the device buffers
        self._h_in = torch.zeros(n_in, dtype=torch.int64).pin_memory()
        self._h_outbuf = torch.zeros(4 + M * B, dtype=torch.float64).pin_memory()
        hi = self._h_in.numpy()
        self._h_idx = hi[seg["idx"]].reshape(M, B)
        self._h_w = hi[seg["w"]].view(np.float64).reshape(M, B)
        self._h_nb = hi[seg["nb"]].reshape(S, P)
        self._h_nsz = hi[seg["nsz"]]
        self._h_coef = hi[seg["coef"]].view(np.float64)

    def _problem(self) -> _lib.Problem:
        p = _lib.Problem()
        self.dataset.fill(p)
        p.S, p.B, p.P = self.S, self.B, self.P
        p.pix_indexes = self.pix_indexes.data_ptr()
        p.pix_weights = self.pix_weights.data_ptr()
        p.neighbors = self.neighbors.data_ptr()
        p.neighbors_sizes = self.neighbors_sizes.data_ptr()
        p.coefficient = 1.0
        p.coefficient_dev = self.coefficient.data_ptr()
        return p

    # ---------------------------------------------------------------- inputs

    def set_model(self, pix_indexes, pix_weights, neighbors, neighbors_sizes, coefficient=1.0):
        """Copy one lens model's arrays into the persistent device buffers (device-to-device for tensors)."""
        self.pix_indexes.copy_(_as_dev(pix_indexes, torch.int64, self.device))
        self.pix_weights.copy_(_as_dev(pix_weights, torch.float64, self.device))
        nb = _as_dev(neighbors, torch.int64, self.device)
        self.neighbors.fill_(-1)
        self.neighbors[:, : nb.shape[1]].copy_(nb)
        self.neighbors_sizes.copy_(_as_dev(neighbors_sizes, torch.int64, self.device))
        self.set_coefficient(coefficient)

    def set_coefficient(self, coefficient):
        if isinstance(coefficient, torch.Tensor):
            self.coefficient.copy_(coefficient.reshape(1).to(self.coefficient))
        else:
            self.coefficient.fill_(float(coefficient))

    # ------------------------------------------------------------- execution

    def launch(self):
        """Enqueue one evaluation on the current stream (no synchronisation)."""
        stream = torch.cuda.current_stream(self.device).cuda_stream
        self.info.zero_()
        rc = self.lib.aj_log_evidence(self.problem, self.pc, int(self.with_grad), self.out.data_ptr(),
                                      self.grad_weights.data_ptr() if self.with_grad else None,
                                      self.reconstruction.data_ptr(), self.workspace.data_ptr(),
                                      self.workspace.numel(), self.info.data_ptr(), stream)
        _lib.check(rc, "aj_log_evidence")

    def capture(self):
        """Record one evaluation into a CUDA graph (after a warm-up call); step() then replays it.

        The capture goes through the library (aj_graph_begin/end) rather than
        torch.cuda.graph: the library instantiates the graph so replays keep
        the stream priorities of its factorisation lanes.  Nothing allocates
        while capturing (all buffers exist already).
        """
        if self.graph is not None:
            self.release_graph()
        cap = torch.cuda.Stream(self.device)
        cap.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(cap):
            self.launch()  # warm-up on the capture stream: creates its side streams
        torch.cuda.synchronize(self.device)
        before = self.lib.aj_launch_count()
        _lib.check(self.lib.aj_graph_begin(cap.cuda_stream), "aj_graph_begin")
        exec_ = ctypes.c_void_p()
        try:
            with torch.cuda.stream(cap):
                self.launch()
        except BaseException:
            if self.lib.aj_graph_end(cap.cuda_stream, ctypes.byref(exec_)) == _lib.AJ_OK:
                self.lib.aj_graph_destroy(exec_)
            raise
        _lib.check(self.lib.aj_graph_end(cap.cuda_stream, ctypes.byref(exec_)), "aj_graph_end")
        self.launches_per_eval = int(self.lib.aj_launch_count() - before)
        self._capture_stream = cap
        self.graph = exec_
        return exec_

    def release_graph(self):
        if self.graph is not None:
            self.lib.aj_graph_destroy(self.graph)
            self.graph = None

    def __del__(self):
        try:
            self.release_graph()
        except Exception:
            pass

    def step(self):
        """One evaluation: graph replay when captured, else a direct launch."""
        if self.graph is not None:
            _lib.check(self.lib.aj_graph_launch(self.graph, torch.cuda.current_stream(self.device).cuda_stream),
                       "aj_graph_launch")
        else:
            self.launch()

    def check(self):
        code, where = (int(v) for v in self.info.tolist())
        self._raise_info(code, where)

    @staticmethod
    def _raise_info(code: int, where: int):
        if code == _lib.AJ_INFO_NOT_POSITIVE_DEFINITE:
            raise np.linalg.LinAlgError(f"curvature_reg_matrix is not positive definite (pivot {where})")
        if code == _lib.AJ_INFO_INDEX_RANGE:
            raise IndexError(f"index out of range (flat position {where})")


    # --------------------------------------------------------- host facing

    def evaluate_host(self, pix_indexes, pix_weights, neighbors, neighbors_sizes, coefficient=1.0):
        """End-to-end call with host NumPy inputs: H2D from pinned memory, one evaluation, D2H of the results.

        Returns (logE, dlogE/dlambda, dlogE/dpix_weights) as NumPy values.
        """
        self._h_idx[...] = pix_indexes
        self._h_w[...] = pix_weights
        nb = np.asarray(neighbors)
        if nb.shape[1] == self._h_nb.shape[1]:
            self._h_nb[...] = nb
        else:
            self._h_nb[...] = -1
            self._h_nb[:, : nb.shape[1]] = nb
        self._h_nsz[...] = neighbors_sizes
        self._h_coef[0] = coefficient
        self._in.copy_(self._h_in, non_blocking=True)
        self.step()
        n_out = self._n_out()
        self._h_outbuf[:n_out].copy_(self._outbuf[:n_out], non_blocking=True)
        torch.cuda.current_stream(self.device).synchronize()
        o = self._h_outbuf.numpy()
        code, where = (int(v) for v in o[2:3].view(np.int32))
        self._raise_info(code, where)
        return float(o[0]), float(o[1]), (o[4:n_out].reshape(self.M, self.B).copy() if self.with_grad else None)

    def _n_out(self) -> int:
        return self._outbuf.numel() if self.with_grad else 4

    def h2d_bytes(self) -> int:
        return self._h_in.numel() * 8

    def d2h_bytes(self) -> int:
        return self._n_out() * 8


class LogEvidenceBatch:
    """Many lens models against one ``Dataset``, evaluated by one call.

    Each model has its own source-pixel count (``S_list``), mapping,
    neighbours and coefficient; ``B`` and ``P`` bound the mapping and
    neighbour widths of every model.  ``launch()`` enqueues all evaluations
    through ``aj_log_evidence_batched`` as concurrent branches of the current
    stream; ``capture()`` records that into one CUDA graph, so ``step()``
    evaluates the whole batch with one graph launch.  Results: ``out`` (n, 2)
    holds logE and dlogE/dlambda per model, ``evals[i].grad_weights`` the
    weight gradients.
    """

    def __init__(self, dataset: Dataset, S_list, *, B: int, P: int, with_grad: bool = True):
        self.dataset = dataset
        self.lib = dataset.lib
        self.device = dataset.device
        self.with_grad = bool(with_grad)
        self.evals = [LogEvidence(S=int(S), B=B, P=P, precision=dataset.precision, with_grad=with_grad,
                                  dataset=dataset) for S in S_list]
        n = self.n = len(self.evals)
        self.out = torch.zeros((n, 2), dtype=torch.float64, device=self.device)
        self.info = torch.zeros((n, 2), dtype=torch.int32, device=self.device)
        self._problems = (_lib.Problem * n)(*[e.problem for e in self.evals])
        self._grads = (ctypes.c_void_p * n)(*[e.grad_weights.data_ptr() for e in self.evals])
        self._recons = (ctypes.c_void_p * n)(*[e.reconstruction.data_ptr() for e in self.evals])
        self._ws = (ctypes.c_void_p * n)(*[e.workspace.data_ptr() for e in self.evals])
        self._ws_bytes = (ctypes.c_size_t * n)(*[e.workspace.numel() for e in self.evals])
        self.graph = None
        self.launches_per_batch = None

    def set_model(self, i, pix_indexes, pix_weights, neighbors, neighbors_sizes, coefficient=1.0):
        self.evals[i].set_model(pix_indexes, pix_weights, neighbors, neighbors_sizes, coefficient)

    def launch(self):
        """Enqueue every evaluation on the current stream (no synchronisation)."""
        stream = torch.cuda.current_stream(self.device).cuda_stream
        self.info.zero_()
        rc = self.lib.aj_log_evidence_batched(self._problems, self.n, self.dataset.pc, int(self.with_grad),
                                              self.out.data_ptr(), ctypes.cast(self._grads, ctypes.c_void_p),
                                              ctypes.cast(self._recons, ctypes.c_void_p),
                                              ctypes.cast(self._ws, ctypes.c_void_p),
                                              ctypes.cast(self._ws_bytes, ctypes.c_void_p), self.info.data_ptr(),
                                              stream)
        _lib.check(rc, "aj_log_evidence_batched")

    def capture(self):
        """Record one batch into a CUDA graph (after a warm-up call on the capture stream)."""
        if self.graph is not None:
            self.release_graph()
        cap = torch.cuda.Stream(self.device)
        cap.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(cap):
            self.launch()
        torch.cuda.synchronize(self.device)
        before = self.lib.aj_launch_count()
        exec_ = ctypes.c_void_p()
        _lib.check(self.lib.aj_graph_begin(cap.cuda_stream), "aj_graph_begin")
        try:
            with torch.cuda.stream(cap):
                self.launch()
        except BaseException:
            if self.lib.aj_graph_end(cap.cuda_stream, ctypes.byref(exec_)) == _lib.AJ_OK:
                self.lib.aj_graph_destroy(exec_)
            raise
        _lib.check(self.lib.aj_graph_end(cap.cuda_stream, ctypes.byref(exec_)), "aj_graph_end")
        self.launches_per_batch = int(self.lib.aj_launch_count() - before)
        self._capture_stream = cap
        self.graph = exec_
        return exec_

    def release_graph(self):
        if self.graph is not None:
            self.lib.aj_graph_destroy(self.graph)
            self.graph = None

    def __del__(self):
        try:
            self.release_graph()
        except Exception:
            pass

    def step(self):
        if self.graph is not None:
            _lib.check(self.lib.aj_graph_launch(self.graph, torch.cuda.current_stream(self.device).cuda_stream),
                       "aj_graph_launch")
        else:
            self.launch()

    def check(self):
        for i, (code, where) in enumerate(self.info.tolist()):
            if code == _lib.AJ_INFO_NOT_POSITIVE_DEFINITE:
                raise np.linalg.LinAlgError(f"model {i}: curvature_reg_matrix is not positive definite (pivot {where})")
            if code == _lib.AJ_INFO_INDEX_RANGE:
                raise IndexError(f"model {i}: index out of range (flat position {where})")



class LogEvidenceFunction(torch.autograd.Function):
    """logE(pix_weights, coefficient) for a LogEvidence evaluator with its model indices set.

    Backward returns dlogE/dpix_weights and dlogE/dcoefficient = 2 c dlogE/dlambda.
    """

    @staticmethod
    def forward(ctx, pix_weights: torch.Tensor, coefficient: torch.Tensor, evaluator: LogEvidence):
        ev = evaluator
        ev.pix_weights.copy_(pix_weights.detach())
        ev.set_coefficient(coefficient.detach())
        ev.step()
        ev.check()
        ctx.save_for_backward(coefficient.detach().clone().reshape(()))
        ctx.grads = (ev.grad_weights.clone(), ev.out[1].clone())
        return ev.out[0].clone()

    @staticmethod
    def backward(ctx, g):
        (c,) = ctx.saved_tensors
        gw, dlam = ctx.grads
        return g * gw, (g * dlam * 2.0 * c).reshape(()), None


def log_evidence(pix_weights: torch.Tensor, coefficient: torch.Tensor, evaluator: LogEvidence) -> torch.Tensor:
    """Differentiable logE (see LogEvidenceFunction)."""
    return LogEvidenceFunction.apply(pix_weights, coefficient, evaluator)


__all__ = ["Dataset", "LogEvidence", "LogEvidenceBatch", "LogEvidenceFunction", "log_evidence", "PRECISIONS"]
