"""Grid2D / Grid3D: the background grid of jump (Grid.jl:64-268), host side.

The fields keep the reference's names and values.  Node arrays are numpy
arrays with one row per node; node index lists (bottomNodes, ...) are
0-based, where the reference's are 1-based (Grid.jl:134-144, 226-249).
``fixedNodes`` has the reference's shape (dim, nodeCount) and its
column-major memory layout, so it crosses the C ABI without a copy.
The dense nodeCount^2 mass matrix ``M`` (Grid.jl:118) serves only the MUSL
solver and is not allocated.
"""
from __future__ import annotations

import numpy as np


class Grid2D:
    dim = 2

    def __init__(self, xmin, xmax, ymin, ymax, iN_x, iN_y):
        xmin, xmax, ymin, ymax = float(xmin), float(xmax), float(ymin), float(ymax)
        iN_x, iN_y = int(iN_x), int(iN_y)
        if iN_x < 2 or iN_y < 2:
            raise ValueError("Grid2D needs at least 2 nodes per axis")
        dx = (xmax - xmin) / (float(iN_x) - 1.0)  # Grid.jl:105
        dy = (ymax - ymin) / (float(iN_y) - 1.0)
        self.xmin, self.ymin = xmin, ymin
        self.xmax, self.ymax = xmax, ymax  # kept so dx is rebuilt bit-exactly across the ABI
        self.lx, self.ly = xmax - xmin, ymax - ymin
        self.dx, self.dy = dx, dy
        self.dxI, self.dyI = 1.0 / dx, 1.0 / dy
        self.nodeCountX, self.nodeCountY = iN_x, iN_y
        self.nodeCount = iN_x * iN_y
        self.cellCount = (iN_x - 1) * (iN_y - 1)
        n = self.nodeCount
        self.mass = np.zeros(n)
        self.momentum0 = np.zeros((n, 2))
        self.momentum = np.zeros((n, 2))
        self.momentum2 = np.zeros((n, 2))
        self.force = np.zeros((n, 2))
        xs = xmin + np.arange(iN_x, dtype=np.float64) * dx  # pos = xmin + (i-1)*dx, Grid.jl:149-152
        ys = ymin + np.arange(iN_y, dtype=np.float64) * dy
        self.pos = np.empty((n, 2))
        self.pos[:, 0] = np.tile(xs, iN_y)
        self.pos[:, 1] = np.repeat(ys, iN_x)
        self.fixedNodes = np.zeros((2, n), dtype=np.int64, order="F")
        i = np.arange(iN_x)
        self.bottomNodes = i.copy()
        self.topNodes = i + iN_x * (iN_y - 1)
        j = np.arange(1, iN_y + 1)
        self.rightNodes = iN_x * j - 1
        self.leftNodes = iN_x * (j - 1)

    @property
    def lengths(self):
        return (self.lx, self.ly)

    def extents(self):
        return (self.xmin, self.xmin + self.lx), (self.ymin, self.ymin + self.ly)


class Grid3D:
    dim = 3

    def __init__(self, xmin, xmax, ymin, ymax, zmin, zmax, iN_x, iN_y, iN_z):
        xmin, xmax = float(xmin), float(xmax)
        ymin, ymax = float(ymin), float(ymax)
        zmin, zmax = float(zmin), float(zmax)
        iN_x, iN_y, iN_z = int(iN_x), int(iN_y), int(iN_z)
        if min(iN_x, iN_y, iN_z) < 2:
            raise ValueError("Grid3D needs at least 2 nodes per axis")
        dx = (xmax - xmin) / (float(iN_x) - 1.0)  # Grid.jl:199-201
        dy = (ymax - ymin) / (float(iN_y) - 1.0)
        dz = (zmax - zmin) / (float(iN_z) - 1.0)
        self.xmin, self.ymin, self.zmin = xmin, ymin, zmin
        self.xmax, self.ymax, self.zmax = xmax, ymax, zmax
        self.lx, self.ly, self.lz = xmax - xmin, ymax - ymin, zmax - zmin
        self.dx, self.dy, self.dz = dx, dy, dz
        self.dxI, self.dyI, self.dzI = 1.0 / dx, 1.0 / dy, 1.0 / dz
        self.nodeCountX, self.nodeCountY, self.nodeCountZ = iN_x, iN_y, iN_z
        self.nodeCountXY = iN_x * iN_y
        self.nodeCount = iN_x * iN_y * iN_z
        n = self.nodeCount
        self.mass = np.zeros(n)
        self.momentum0 = np.zeros((n, 3))
        self.momentum = np.zeros((n, 3))
        self.momentum2 = np.zeros((n, 3))
        self.force = np.zeros((n, 3))
        xs = xmin + np.arange(iN_x, dtype=np.float64) * dx  # Grid.jl:253-264
        ys = ymin + np.arange(iN_y, dtype=np.float64) * dy
        zs = zmin + np.arange(iN_z, dtype=np.float64) * dz
        self.pos = np.empty((n, 3))
        self.pos[:, 0] = np.tile(xs, iN_y * iN_z)
        self.pos[:, 1] = np.tile(np.repeat(ys, iN_x), iN_z)
        self.pos[:, 2] = np.repeat(zs, iN_x * iN_y)
        self.fixedNodes = np.zeros((3, n), dtype=np.int64, order="F")
        nxy = self.nodeCountXY
        k = np.arange(iN_z)
        i = np.arange(iN_x)
        # bottom/top are the y faces, left/right the x faces, front/back the z faces
        self.bottomNodes = (i[None, :] + k[:, None] * nxy).ravel()
        self.topNodes = (i[None, :] + iN_x * (iN_y - 1) + k[:, None] * nxy).ravel()
        j = np.arange(1, iN_y + 1)
        self.rightNodes = (iN_x * j[None, :] - 1 + k[:, None] * nxy).ravel()
        self.leftNodes = (iN_x * (j[None, :] - 1) + k[:, None] * nxy).ravel()
        self.frontNodes = np.arange(nxy)
        self.backNodes = np.arange(nxy) + (iN_z - 1) * nxy

    @property
    def lengths(self):
        return (self.lx, self.ly, self.lz)


def to_1D_index(i, j, grid, k=None):
    """1-based node index of 1-based (i, j[, k]) (Grid.jl:275-291)."""
    if k is None:
        return grid.nodeCountX * (j - 1) + i
    return grid.nodeCountXY * (k - 1) + grid.nodeCountX * (j - 1) + i
