"""Raw float32 files in the layouts of the reference's drivers.

``read_binary_dataset`` keeps both of the reference's signatures:

* ``read_binary_dataset(file, [H, W])`` -> float32 [-1, H, W], C order
  (test.py:10-15: images [slice][y][x] or sinograms [slice][view][col]);
* ``read_binary_dataset(file, num_samples, nview, ncol)`` -> float32
  [num_samples, nview, ncol] (FDK/FDK_test_training.py:9-16).

``write_raw`` writes an array's bytes in C order, as the drivers'
``f.write(bytearray(array))`` does (test.py:24-26, FDK/FDK_test_training.py:
130-133); torch tensors are moved to the host first.
"""
from __future__ import annotations

import os

import numpy as np


def read_binary_dataset(file_name, *dims) -> np.ndarray:
    """float32 array of a raw file, shaped as one of the reference drivers does."""
    data = np.fromfile(file_name, dtype=np.float32, count=-1)
    if len(dims) == 1:
        h, w = (int(d) for d in dims[0])
        if data.size % (h * w):
            raise ValueError(f"{file_name}: {data.size} floats is not a whole number of "
                             f"{h}x{w} slices")
        return np.reshape(data, (-1, h, w), order="C")
    if len(dims) == 3:
        s, v, c = (int(d) for d in dims)
        if data.size != s * v * c:
            raise ValueError(f"{file_name}: {data.size} floats, expected {s}x{v}x{c}")
        return np.reshape(data, (s, v, c), order="C")
    raise TypeError("read_binary_dataset(file, [H, W]) or (file, num_samples, nview, ncol)")


def write_raw(file_name, array) -> int:
    """Writes the array's float32 bytes in C order; returns the byte count."""
    try:
        import torch
        if isinstance(array, torch.Tensor):
            array = array.detach().cpu().numpy()
    except ImportError:  # pragma: no cover
        pass
    a = np.ascontiguousarray(array)
    d = os.path.dirname(os.fspath(file_name))
    if d:
        os.makedirs(d, exist_ok=True)
    with open(file_name, "wb") as f:
        f.write(a.tobytes(order="C"))
    return a.nbytes
