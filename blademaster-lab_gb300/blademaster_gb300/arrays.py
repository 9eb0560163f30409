"""Reference-shaped views of the solver's device buffers.

The reference exposes Warp arrays that callers read with ``.numpy()`` and
write with ``.assign()``, ``.zero_()`` and ``.fill_()``
(e.g. blademaster_warp/paper_freefall.py:78-79, tests/test_single_field.py:10-13).
Here the device layout differs from the API shape (particles are in cell
order and structure-of-arrays; the knife state is float64), so each view
carries a reader and a writer that translate between the two.
"""

import numpy as np


class DeviceArray:
    """A device buffer seen in the reference's shape and dtype."""

    def __init__(self, shape, dtype, read, write=None, on_write=None, name=""):
        self.shape = tuple(shape)
        self.dtype = np.dtype(dtype)
        self._read = read
        self._write = write
        self._on_write = on_write
        self.name = name

    def numpy(self):
        return np.asarray(self._read(), dtype=self.dtype).reshape(self.shape)

    def assign(self, data):
        if self._write is None:
            raise ValueError(f"{self.name} is read-only")
        value = np.asarray(data, dtype=self.dtype)
        if value.size != int(np.prod(self.shape)):
            raise ValueError(f"{self.name}: expected shape {self.shape}, got {value.shape}")
        self._write(value.reshape(self.shape))
        if self._on_write is not None:
            self._on_write()

    def zero_(self):
        self.assign(np.zeros(self.shape, self.dtype))

    def fill_(self, value):
        self.assign(np.full(self.shape, value, self.dtype))

    def __len__(self):
        return self.shape[0]

    def __repr__(self):
        return f"DeviceArray({self.name}, shape={self.shape}, dtype={self.dtype})"


def particle_view(tensor, order_t, rank_t, components, dtype, name, on_write=None, leading=None):
    """View of a [components][n] (or [leading][components][n]) device tensor as (n, ...) in reference order."""
    import torch

    n = tensor.shape[-1]
    comp_shape = () if components is None else tuple(components)
    ncomp = int(np.prod(comp_shape)) if comp_shape else 1
    api_shape = (n, *comp_shape) if leading is None else (leading, n, *comp_shape)

    def read():
        t = tensor.reshape(-1, ncomp, n) if leading is not None else tensor.reshape(ncomp, n)
        t = t.index_select(-1, rank_t)
        if leading is not None:
            return t.permute(0, 2, 1).reshape(api_shape).cpu().numpy()
        return t.t().reshape(api_shape).cpu().numpy()

    def write(value):
        v = torch.as_tensor(np.ascontiguousarray(value), device=tensor.device).to(tensor.dtype)
        if leading is not None:
            v = v.reshape(leading, n, ncomp).index_select(1, order_t).permute(0, 2, 1)
        else:
            v = v.reshape(n, ncomp).index_select(0, order_t).t()
        tensor.copy_(v.reshape(tensor.shape))

    return DeviceArray(api_shape, dtype, read, write, on_write, name)


def plain_view(tensor, shape, dtype, name, on_write=None, writable=True):
    """View of a device tensor whose layout already matches the API (reshaped only)."""
    import torch

    def read():
        return tensor.reshape(shape).cpu().numpy()

    def write(value):
        tensor.copy_(torch.as_tensor(np.ascontiguousarray(value), device=tensor.device).to(tensor.dtype).reshape(tensor.shape))

    return DeviceArray(shape, dtype, read, write if writable else None, on_write, name)


def soa_view(tensor, count, name, on_write=None):
    """View of a [3][count] device tensor as (count, 3)."""
    import torch

    def read():
        return tensor.reshape(3, count).t().cpu().numpy()

    def write(value):
        tensor.copy_(torch.as_tensor(np.ascontiguousarray(value), device=tensor.device).to(tensor.dtype).t().reshape(tensor.shape))

    return DeviceArray((count, 3), np.float32, read, write, on_write, name)
