"""Grid Dirichlet conditions: fix_Dirichlet_grid (Dirichlet.jl:28-82)."""
from __future__ import annotations

import numpy as np


def fix_Dirichlet_grid(grid, data, ghostcell: bool = False):
    """Set grid.fixedNodes[:, face] .= mask for each (face, mask) of data["dirichlet_grid"].

    Faces: "bottom"/"top" (y), "left"/"right" (x) and, on a Grid3D, "front"/"back" (z).
    With ghostcell=True on a Grid2D the next node row inwards is fixed too
    (Dirichlet.jl:60-78).
    """
    if "dirichlet_grid" not in data:
        return
    d = grid.dim
    for bnd, fix in data["dirichlet_grid"]:
        mask = np.asarray(fix, dtype=np.int64).reshape(d, 1)
        if bnd == "bottom":
            nodes = [grid.bottomNodes] + ([grid.bottomNodes + grid.nodeCountX] if (ghostcell and d == 2) else [])
        elif bnd == "top":
            nodes = [grid.topNodes] + ([grid.topNodes - grid.nodeCountX] if (ghostcell and d == 2) else [])
        elif bnd == "left":
            nodes = [grid.leftNodes] + ([grid.leftNodes + 1] if (ghostcell and d == 2) else [])
        elif bnd == "right":
            nodes = [grid.rightNodes] + ([grid.rightNodes - 1] if (ghostcell and d == 2) else [])
        elif bnd == "front" and d == 3:
            nodes = [grid.frontNodes]
        elif bnd == "back" and d == 3:
            nodes = [grid.backNodes]
        else:
            raise ValueError("Not recognized grid faces!!!")
        for idx in nodes:
            grid.fixedNodes[:, idx] = mask
