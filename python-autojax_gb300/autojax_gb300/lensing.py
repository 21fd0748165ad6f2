"""Lens parameters to logE and back, on the device.

The reference's likelihood takes a finished mapping (``pix_indexes``,
``pix_weights``, numba.py:761-857); a lens-model sampler has to produce that
mapping from its parameters every step.  This module does that on the GPU and
carries the adjoint the other way:

    theta_E, source points, coefficient
        -> beta = SIS trace of the image grid          (aj_sis_trace)
        -> barycentric weights in the fixed triangulation (aj_delaunay_weights)
        -> logE, dlogE/dlambda, dlogE/dpix_weights    (aj_log_evidence)
        -> dlogE/dpoints, dlogE/dbeta                 (aj_delaunay_weights_vjp)
        -> dlogE/dtheta_E                             (aj_sis_trace_vjp)

The triangulation (and so the neighbour lists of the regularisation) is fixed
at construction from the starting points: gradients are those of the
weights for that topology, as a sampler that keeps the mesh's connectivity
uses them.  Coordinates are (y, x) in arcsec.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from ._device import Call, ptr
from .inversion import Dataset, LogEvidence


def _lib_call(name, *args):
    _lib.check(getattr(_lib.load(), name)(*args), name)


def sis_trace(theta, einstein_radius):
    """beta = theta - theta_E theta / |theta| for theta (M, 2) in arcsec."""
    c = Call("sis_trace")
    t = c.arr(theta, torch.float64, 2, "theta")
    beta = c.empty(tuple(t.shape))
    _lib_call("aj_sis_trace", ptr(t), t.shape[0], float(einstein_radius), None, ptr(beta), c.stream())
    return c.out(beta)


def delaunay_weights(beta, points, simplices):
    """(pix_indexes (M, 3), pix_weights (M, 3)) of beta in the triangulation of points."""
    c = Call("delaunay_weights")
    b = c.arr(beta, torch.float64, 2, "beta")
    P = c.arr(points, torch.float64, 2, "points")
    tri = c.arr(simplices, torch.int64, 2, "simplices")
    M = b.shape[0]
    idx = c.empty((M, 3), torch.int64)
    w = c.empty((M, 3))
    info = c.info()
    _lib_call("aj_delaunay_weights", ptr(b), M, ptr(P), P.shape[0], ptr(tri), tri.shape[0], ptr(idx), ptr(w),
              ptr(info), c.stream())
    c.check_info(info)
    return c.out(idx), c.out(w)


def bilinear_weights(beta, n, half_width):
    """(pix_indexes (M, 4), pix_weights (M, 4)) on the n x n mesh over [-half_width, half_width]^2."""
    c = Call("bilinear_weights")
    b = c.arr(beta, torch.float64, 2, "beta")
    M = b.shape[0]
    idx = c.empty((M, 4), torch.int64)
    w = c.empty((M, 4))
    _lib_call("aj_bilinear_weights", ptr(b), M, int(n), float(half_width), ptr(idx), ptr(w), c.stream())
    return c.out(idx), c.out(w)


def delaunay_weights_vjp(beta, points, pix_indexes, grad_weights):
    """(dL/dpoints (S, 2), dL/dbeta (M, 2)) from dL/dpix_weights (M, 3)."""
    c = Call("delaunay_weights_vjp")
    b = c.arr(beta, torch.float64, 2, "beta")
    P = c.arr(points, torch.float64, 2, "points")
    idx = c.arr(pix_indexes, torch.int64, 2, "pix_indexes")
    G = c.arr(grad_weights, torch.float64, 2, "grad_weights")
    gP = c.empty(tuple(P.shape))
    gB = c.empty(tuple(b.shape))
    _lib_call("aj_delaunay_weights_vjp", ptr(b), b.shape[0], ptr(P), P.shape[0], ptr(idx), ptr(G), ptr(gP), ptr(gB),
              c.stream())
    return c.out(gP), c.out(gB)


def bilinear_weights_vjp(beta, n, half_width, grad_weights):
    c = Call("bilinear_weights_vjp")
    b = c.arr(beta, torch.float64, 2, "beta")
    G = c.arr(grad_weights, torch.float64, 2, "grad_weights")
    gB = c.empty(tuple(b.shape))
    _lib_call("aj_bilinear_weights_vjp", ptr(b), b.shape[0], int(n), float(half_width), ptr(G), ptr(gB), c.stream())
    return c.out(gB)


def sis_trace_vjp(theta, grad_beta):
    """dL/dtheta_E from dL/dbeta (M, 2)."""
    c = Call("sis_trace_vjp")
    t = c.arr(theta, torch.float64, 2, "theta")
    g = c.arr(grad_beta, torch.float64, 2, "grad_beta")
    out = c.zeros(1)
    _lib_call("aj_sis_trace_vjp", ptr(t), t.shape[0], ptr(g), ptr(out), c.stream())
    return float(out.cpu()[0]) if c.numpy_out else out[0]


def triangulate(points):
    """Host Delaunay triangulation: (simplices (T, 3), neighbours (S, P) -1 padded, sizes (S,))."""
    from scipy.spatial import Delaunay

    pts = np.asarray(points, dtype=np.float64)
    tri = Delaunay(pts)
    indptr, indices = tri.vertex_neighbor_vertices
    deg = np.diff(indptr)
    nb = -np.ones((pts.shape[0], int(deg.max())), dtype=np.int64)
    for s in range(pts.shape[0]):
        nb[s, : deg[s]] = np.sort(indices[indptr[s] : indptr[s + 1]])
    return np.ascontiguousarray(tri.simplices.astype(np.int64)), nb, deg.astype(np.int64)


class LensedEvidence:
    """logE and its gradients in (theta_E, source points, coefficient) for one dataset.

    ``theta`` (M, 2) is the image grid in arcsec (the dataset's slim grid);
    ``points`` (S, 2) the starting source points, whose Delaunay triangulation
    fixes the mesh topology and the regularisation neighbours.  ``step()``
    enqueues trace -> weights -> evaluation -> adjoint on the current stream;
    ``capture()`` records that as one CUDA graph (theta_E, points and the
    coefficient live in device memory, so replays take new values).
    """

    def __init__(self, dataset: Dataset, theta, points, *, with_grad: bool = True):
        self.dataset = ds = dataset
        self.device = dev = ds.device
        self.lib = ds.lib
        self.theta = torch.as_tensor(np.ascontiguousarray(theta, dtype=np.float64)).to(dev)
        self.M = self.theta.shape[0]
        if self.M != ds.M:
            raise ValueError("theta must have one row per image pixel of the dataset")
        simplices, nb, nsz = triangulate(np.asarray(points))
        self.S = nb.shape[0]
        self.simplices = torch.from_numpy(simplices).to(dev)
        self.points = torch.as_tensor(np.ascontiguousarray(points, dtype=np.float64)).to(dev)
        self.einstein_radius = torch.zeros(1, dtype=torch.float64, device=dev)
        self.beta = torch.empty((self.M, 2), dtype=torch.float64, device=dev)
        self.ev = LogEvidence(S=self.S, B=3, P=nb.shape[1], precision=ds.precision, with_grad=with_grad, dataset=ds)
        self.ev.neighbors.copy_(torch.from_numpy(nb))
        self.ev.neighbors_sizes.copy_(torch.from_numpy(nsz))
        self.with_grad = bool(with_grad)
        self.grad_points = torch.zeros((self.S, 2), dtype=torch.float64, device=dev)
        self.grad_beta = torch.zeros((self.M, 2), dtype=torch.float64, device=dev)
        self.grad_einstein_radius = torch.zeros(1, dtype=torch.float64, device=dev)
        self.weight_info = torch.zeros(2, dtype=torch.int32, device=dev)
        self.graph = None

    def set_params(self, einstein_radius, points=None, coefficient=None):
        if isinstance(einstein_radius, torch.Tensor):
            self.einstein_radius.copy_(einstein_radius.reshape(1).to(self.einstein_radius))
        else:
            self.einstein_radius.fill_(float(einstein_radius))
        if points is not None:
            self.points.copy_(torch.as_tensor(points, dtype=torch.float64).reshape(self.S, 2))
        if coefficient is not None:
            self.ev.set_coefficient(coefficient)

    def launch(self):
        st = torch.cuda.current_stream(self.device).cuda_stream
        lib = self.lib
        _lib.check(lib.aj_sis_trace(self.theta.data_ptr(), self.M, 0.0, self.einstein_radius.data_ptr(),
                                    self.beta.data_ptr(), st), "aj_sis_trace")
        self.weight_info.zero_()
        _lib.check(lib.aj_delaunay_weights(self.beta.data_ptr(), self.M, self.points.data_ptr(), self.S,
                                           self.simplices.data_ptr(), self.simplices.shape[0],
                                           self.ev.pix_indexes.data_ptr(), self.ev.pix_weights.data_ptr(),
                                           self.weight_info.data_ptr(), st), "aj_delaunay_weights")
        self.ev.launch()
        if self.with_grad:
            _lib.check(lib.aj_delaunay_weights_vjp(self.beta.data_ptr(), self.M, self.points.data_ptr(), self.S,
                                                   self.ev.pix_indexes.data_ptr(), self.ev.grad_weights.data_ptr(),
                                                   self.grad_points.data_ptr(), self.grad_beta.data_ptr(), st),
                       "aj_delaunay_weights_vjp")
            _lib.check(lib.aj_sis_trace_vjp(self.theta.data_ptr(), self.M, self.grad_beta.data_ptr(),
                                            self.grad_einstein_radius.data_ptr(), st), "aj_sis_trace_vjp")

    def capture(self):
        """Record one step (trace -> weights -> evaluation -> adjoint) into a CUDA graph."""
        if self.graph is not None:
            self.release_graph()
        cap = torch.cuda.Stream(self.device)
        cap.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(cap):
            self.launch()
        torch.cuda.synchronize(self.device)
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
        self._capture_stream = cap
        self.graph = exec_

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
        code, where = (int(v) for v in self.weight_info.tolist())
        if code == _lib.AJ_INFO_INDEX_RANGE:
            raise IndexError(f"simplex index out of range (flat position {where})")
        self.ev.check()

    def evaluate(self, einstein_radius, points=None, coefficient=None):
        """One evaluation; returns (logE, dlogE/dtheta_E, dlogE/dpoints (S, 2) numpy, dlogE/dlambda)."""
        self.set_params(einstein_radius, points, coefficient)
        self.step()
        torch.cuda.current_stream(self.device).synchronize()
        self.check()
        out = self.ev.out.cpu().numpy()
        return (float(out[0]), float(self.grad_einstein_radius.cpu()[0]), self.grad_points.cpu().numpy(),
                float(out[1]))


class LensedLogEvidenceFunction(torch.autograd.Function):
    """logE(theta_E, points, coefficient) through a LensedEvidence evaluator, differentiable in all three."""

    @staticmethod
    def forward(ctx, einstein_radius, points, coefficient, evaluator: LensedEvidence):
        ev = evaluator
        ev.set_params(einstein_radius.detach(), points.detach(), coefficient.detach())
        ev.step()
        ev.check()
        ctx.save_for_backward(coefficient.detach().clone().reshape(()))
        ctx.grads = (ev.grad_einstein_radius.clone().reshape(einstein_radius.shape), ev.grad_points.clone(),
                     ev.ev.out[1].clone())
        return ev.ev.out[0].clone()

    @staticmethod
    def backward(ctx, g):
        (c,) = ctx.saved_tensors
        g_te, g_pts, dlam = ctx.grads
        return g * g_te, g * g_pts, (g * dlam * 2.0 * c).reshape(()), None


__all__ = ["sis_trace", "sis_trace_vjp", "delaunay_weights", "delaunay_weights_vjp", "bilinear_weights",
           "bilinear_weights_vjp", "triangulate", "LensedEvidence", "LensedLogEvidenceFunction"]
