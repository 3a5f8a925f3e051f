"""Algorithm tags (Algorithm.jl:13-45), basis tags (Basis.jl:37-48) and body
forces (BodyForce.jl:56-91) of the explicit step, host side."""
from __future__ import annotations

import numpy as np


class AlgorithmType:
    pass


class USL(AlgorithmType):
    """Update-stress-last; ``tolerance`` is the nodal-mass cutoff of G2P (Algorithm.jl:16-18)."""

    def __init__(self, tolerance):
        self.tolerance = float(tolerance)


class MUSL(AlgorithmType):
    """Modified USL with FLIP/PIC blend ``alpha`` (Algorithm.jl:37-39): particle
    velocities v <- alpha v + sum N (v_I - alpha v0_I) before the kinematics."""

    def __init__(self, alpha):
        self.alpha = float(alpha)


class BasisType:
    pass


class LinearBasis(BasisType):
    """Linear hat functions (Basis.jl:39), 2 nodes per axis."""


class QuadBsplineBasis(BasisType):
    """Modified quadratic B-splines, 3 nodes per axis (Basis.jl:374-592, Bsplines.jl:18-80)."""


class CubicBsplineBasis(BasisType):
    """Modified cubic B-splines, 4 nodes per axis (Basis.jl:594-820, Bsplines.jl:86-172)."""


class BodyForceType:
    pass


class ConstantBodyForce2D(BodyForceType):
    """``body .= g`` for every particle (BodyForce.jl:56-58, 85-87)."""

    def __init__(self, g):
        self.g = np.asarray(g, dtype=np.float64).reshape(2)

    def __call__(self, body, x, t):
        body[:] = self.g


class ConstantBodyForce3D(BodyForceType):
    """BodyForce.jl:60-62, 89-91."""

    def __init__(self, g):
        self.g = np.asarray(g, dtype=np.float64).reshape(3)

    def __call__(self, body, x, t):
        body[:] = self.g
