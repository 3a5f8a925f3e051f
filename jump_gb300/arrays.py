"""Per-particle matrix arrays in the layout the C ABI reads.

A Julia ``Vector{SMatrix{d,d,Float64}}`` stores each particle's matrix
column-major.  ``matrix_array`` returns an (n, d, d) array indexed
``A[p, i, j]`` (row i, column j) whose memory is that column-major layout, so
the descriptors hand its buffer to the library without a transposed copy.
"""
from __future__ import annotations

import numpy as np


def matrix_array(n: int, d: int, identity: bool = False) -> np.ndarray:
    store = np.zeros((int(n), d, d))  # store[p, j, i] = A_ij: column j contiguous
    if identity:
        store[:, np.arange(d), np.arange(d)] = 1.0
    return store.transpose(0, 2, 1)
