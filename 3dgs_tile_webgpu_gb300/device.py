"""Device-memory plumbing for Python callers: scene upload and zero-copy views
of the library's device pointers as torch tensors (``__cuda_array_interface__``)."""
from __future__ import annotations

import numpy as np

from .abi import GaussianData

_TYPESTR = {np.dtype(np.uint32): "<u4", np.dtype(np.float32): "<f4", np.dtype(np.uint16): "<u2",
            np.dtype(np.int32): "<i4", np.dtype(np.float16): "<f2"}


class _Interface:
    def __init__(self, ptr: int, shape, dtype):
        self.__cuda_array_interface__ = {"shape": tuple(int(s) for s in shape), "typestr": _TYPESTR[np.dtype(dtype)],
                                         "data": (int(ptr), False), "version": 2, "strides": None}


def view(ptr: int, shape, dtype=np.uint32):
    """A torch tensor aliasing ``shape`` elements at device address ``ptr``."""
    import torch
    if int(np.prod(shape)) == 0:
        return torch.empty(tuple(shape), dtype={np.dtype(np.uint32): torch.int32, np.dtype(np.float32): torch.float32}
                           .get(np.dtype(dtype), torch.int32), device="cuda")
    return torch.as_tensor(_Interface(ptr, shape, dtype), device="cuda")


def to_numpy(ptr: int, shape, dtype=np.uint32) -> np.ndarray:
    t = view(ptr, shape, dtype)
    return t.cpu().numpy().view(dtype).reshape(shape)


class DeviceScene:
    """Packed scene buffers resident on the GPU (the Store's role)."""

    def __init__(self, scene: dict, device: str = "cuda"):
        import torch
        self.scene = scene
        self.means = torch.from_numpy(np.ascontiguousarray(scene["means"], np.float32)).to(device)
        self.shape = torch.from_numpy(np.ascontiguousarray(scene["shape"], np.uint32).view(np.int32)).to(device)
        self.rot = torch.from_numpy(np.ascontiguousarray(scene["rotations"], np.uint32).view(np.int32)).to(device)
        self.sh = torch.from_numpy(np.ascontiguousarray(scene["sh"], np.uint32).view(np.int32)).to(device)
        self.count = int(scene["count"])
        self.active_count = int(scene["active_count"])
        self.sh_degree = int(scene["sh_degree"])

    def data(self) -> GaussianData:
        d = GaussianData()
        d.count, d.active_count, d.sh_degree = self.count, self.active_count, self.sh_degree
        d.means, d.scales_opacity = self.means.data_ptr(), self.shape.data_ptr()
        d.rotations, d.sh_coefficients = self.rot.data_ptr(), self.sh.data_ptr()
        return d

    def nbytes(self) -> int:
        return sum(t.numel() * t.element_size() for t in (self.means, self.shape, self.rot, self.sh))
