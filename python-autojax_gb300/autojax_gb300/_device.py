"""Host-side plumbing between NumPy/torch arrays and the C ABI (device memory, streams, status words)."""

from __future__ import annotations

import numpy as np
import torch

from . import _lib

PRECISIONS = {"fp64": _lib.AJ_FP64, "mixed": _lib.AJ_MIXED}

_NP_DTYPES = {
    torch.float64: np.float64,
    torch.int64: np.int64,
    torch.float32: np.float32,
    torch.uint8: np.uint8,
}


def precision_code(precision: str) -> int:
    try:
        return PRECISIONS[precision]
    except KeyError:
        raise ValueError(f"precision must be one of {sorted(PRECISIONS)}, got {precision!r}") from None


class Call:
    """Collects the inputs of one drop-in call, moves them to the GPU and returns outputs in the caller's type.

    NumPy inputs are checked like the reference's typed signatures (dtype and
    C-contiguity, else TypeError) and copied to the device; torch tensors are
    used in place when already on the device with the right dtype.
    """

    def __init__(self, name: str):
        self.name = name
        self.numpy_out = True
        self.device = None
        self.keep = []

    def _pick_device(self):
        if self.device is None:
            if not torch.cuda.is_available():
                raise RuntimeError(f"{self.name}: no CUDA device is visible (autojax_gb300 has no CPU path)")
            self.device = torch.device("cuda", torch.cuda.current_device())
        return self.device

    def arr(self, x, dtype: torch.dtype, ndim: int | None = None, name: str = "array") -> torch.Tensor:
        if isinstance(x, torch.Tensor):
            self.numpy_out = False
            if self.device is None and x.is_cuda:
                self.device = x.device
            dev = self._pick_device()
            t = x.to(device=dev, dtype=dtype).contiguous()
        else:
            a = np.asarray(x)
            want = _NP_DTYPES.get(dtype)
            if dtype == torch.complex128:
                want = np.complex128
            if a.dtype != want:
                raise TypeError(f"{self.name}: {name} must be {np.dtype(want).name}, got {a.dtype.name}")
            if not a.flags.c_contiguous:
                raise TypeError(f"{self.name}: {name} must be C-contiguous")
            dev = self._pick_device()
            t = torch.from_numpy(a).to(dev)
        if ndim is not None and t.dim() != ndim:
            raise TypeError(f"{self.name}: {name} must be {ndim}-D, got shape {tuple(t.shape)}")
        self.keep.append(t)
        return t

    def complex_as_real(self, x, name: str) -> torch.Tensor:
        t = self.arr(x, torch.complex128, 1, name)
        return torch.view_as_real(t).contiguous()

    def empty(self, shape, dtype=torch.float64) -> torch.Tensor:
        return torch.empty(shape, dtype=dtype, device=self._pick_device())

    def zeros(self, shape, dtype=torch.float64) -> torch.Tensor:
        return torch.zeros(shape, dtype=dtype, device=self._pick_device())

    def workspace(self, nbytes: int) -> torch.Tensor:
        t = torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=self._pick_device())
        self.keep.append(t)
        return t

    def info(self) -> torch.Tensor:
        t = torch.zeros(2, dtype=torch.int32, device=self._pick_device())
        self.keep.append(t)
        return t

    def stream(self) -> int:
        return torch.cuda.current_stream(self._pick_device()).cuda_stream

    def check_info(self, info: torch.Tensor) -> None:
        code, where = (int(v) for v in info.tolist())
        if code == _lib.AJ_INFO_INDEX_RANGE:
            raise IndexError(f"{self.name}: index out of range (flat position {where})")
        if code == _lib.AJ_INFO_NOT_POSITIVE_DEFINITE:
            raise np.linalg.LinAlgError(f"{self.name}: matrix is not positive definite (pivot {where})")
        if code == _lib.AJ_INFO_SINGULAR:
            raise np.linalg.LinAlgError(f"{self.name}: Singular matrix (zero pivot {where})")

    def out(self, t: torch.Tensor):
        return t.cpu().numpy() if self.numpy_out else t

    def scalar(self, t: torch.Tensor):
        return float(t.item()) if self.numpy_out else t.reshape(())


def ptr(t) -> int | None:
    return None if t is None else t.data_ptr()
