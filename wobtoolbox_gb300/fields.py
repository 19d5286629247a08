"""raw_data field files of the reference: a uint32 grid size followed by the raw little-endian
array (runtime_utils.cuh:34-81), e.g. potential{N}.scalar (float32) and gradient{N}.vector2/3
(float32 x 2/3). NaN marks points that were not evaluated (apps/general_2d.cu:45-47)."""
from __future__ import annotations

import numpy as np


def save_field(path: str, field: np.ndarray, grid_size: int) -> None:
    with open(path, "wb") as f:
        f.write(np.uint32(grid_size).tobytes())
        f.write(np.ascontiguousarray(field, dtype=np.float32).tobytes())


def load_field(path: str, components: int = 1):
    """Returns (grid_size, array [n] or [n, components])."""
    with open(path, "rb") as f:
        grid = int(np.frombuffer(f.read(4), dtype=np.uint32)[0])
        data = np.frombuffer(f.read(), dtype=np.float32)
    if components > 1:
        data = data.reshape(-1, components)
    return grid, data
