"""Solid2D / Solid3D particle containers and the particle generators of jump
(Solid.jl:67-125, 267-297, 322-537), host side.

Particle fields keep the reference's names.  Vectors are (parCount, d) numpy
arrays and matrices (parCount, d, d) with ``A[p, i, j]`` the (i, j) entry;
their memory is column-major per particle (the layout of a Julia
``SMatrix``, which the C ABI reads), so they pass to the library uncopied.

Extension beyond the reference: ``youngs`` (None or a parCount array) gives
a per-particle Young's modulus, used by inverse problems that recover E per
particle.
"""
from __future__ import annotations

from fractions import Fraction
import math

import numpy as np

from .arrays import matrix_array
from .material import RigidMaterial


def julia_range(start: float, step: float, stop: float) -> np.ndarray:
    """Elements of the Julia float range ``start:step:stop``.

    The length follows Base's fallback rule (round((stop-start)/step) + 1,
    minus one on overshoot); every element is the double nearest to
    start + k*step, evaluated exactly, as Julia's twice-precision ranges do.
    """
    start, step, stop = float(start), float(step), float(stop)
    if step == 0:
        raise ValueError("range step cannot be zero")
    lf = (stop - start) / step
    if lf < 0:
        n = 0
    elif lf == 0:
        n = 1
    else:
        n = int(round(lf)) + 1
        last = start + (n - 1) * step
        n -= int(start < stop < last) + int(start > stop > last)
    fs, fst = Fraction(start), Fraction(step)
    return np.array([float(fs + k * fst) for k in range(n)], dtype=np.float64)


def buildParticleForCircle(fCenter, fRadius: float, fOffset: float) -> np.ndarray:
    """Lattice points strictly inside a circle (Solid.jl:322-337)."""
    fRadius = math.floor(fRadius / fOffset) * fOffset
    r = julia_range(-fRadius + 0.5 * fOffset, fOffset, +fRadius - 0.5 * fOffset)
    fy, fx = np.meshgrid(r, r, indexing="ij")  # fy outer loop, fx inner
    keep = (fx * fx + fy * fy) < fRadius * fRadius
    return np.stack([fCenter[0] + fx[keep], fCenter[1] + fy[keep]], axis=1)


def buildParticleForRing(fCenter, innerRad, outerRad, fOffset) -> np.ndarray:
    """Lattice points inside an annulus (Solid.jl:339-354)."""
    fRadius = math.floor(outerRad / fOffset) * fOffset
    r = julia_range(-fRadius + 0.5 * fOffset, fOffset, +fRadius - 0.5 * fOffset)
    fy, fx = np.meshgrid(r, r, indexing="ij")
    r2 = fx * fx + fy * fy
    keep = (r2 < outerRad * outerRad) & (r2 > innerRad * innerRad)
    return np.stack([fCenter[0] + fx[keep], fCenter[1] + fy[keep]], axis=1)


def buildParticleForSphere(fCenter, fRadius: float, fOffset: float) -> np.ndarray:
    """Lattice points strictly inside a sphere (Solid.jl:356-373)."""
    fRadius = math.floor(fRadius / fOffset) * fOffset
    r = julia_range(-fRadius + 0.5 * fOffset, fOffset, +fRadius - 0.5 * fOffset)
    fz, fy, fx = np.meshgrid(r, r, r, indexing="ij")
    keep = (fx * fx + fy * fy + fz * fz) < fRadius * fRadius
    return np.stack([fCenter[0] + fx[keep], fCenter[1] + fy[keep], fCenter[2] + fz[keep]], axis=1)


def buildParticleForCylinder(fCenter, fRadius, fLength, fOffsetX, fOffsetZ, axis: int = 1) -> np.ndarray:
    """Lattice points inside a cylinder of half-length ``fLength`` (Solid.jl:447-465).

    The reference's cylinder runs along y (axis=1); ``axis`` selects another
    axis with the same loop order (length outermost, then the two cross axes).
    """
    fRadius = math.floor(fRadius / fOffsetX) * fOffsetX
    rl = julia_range(-fLength + 0.5 * fOffsetZ, fOffsetZ, +fLength - 0.5 * fOffsetZ)
    rc = julia_range(-fRadius + 0.5 * fOffsetX, fOffsetX, +fRadius - 0.5 * fOffsetX)
    fl, fz, fx = np.meshgrid(rl, rc, rc, indexing="ij")
    keep = (fx * fx + fz * fz) < fRadius * fRadius
    fl, fz, fx = fl[keep], fz[keep], fx[keep]
    if axis == 1:
        comps = (fx, fl, fz)
    elif axis == 2:
        comps = (fx, fz, fl)
    else:
        comps = (fl, fx, fz)
    return np.stack([fCenter[0] + comps[0], fCenter[1] + comps[1], fCenter[2] + comps[2]], axis=1)


def buildParticleForRectangle(fCenter, fWidth: float, fHeight: float, fOffset: float) -> np.ndarray:
    """Lattice points of a rectangle (Solid.jl:471-486)."""
    fWidth = math.floor(fWidth / fOffset) * fOffset
    fHeight = math.floor(fHeight / fOffset) * fOffset
    ry = julia_range(-0.5 * fHeight + 0.5 * fOffset, fOffset, +0.5 * fHeight - 0.5 * fOffset)
    rx = julia_range(-0.5 * fWidth + 0.5 * fOffset, fOffset, +0.5 * fWidth - 0.5 * fOffset)
    fy, fx = np.meshgrid(ry, rx, indexing="ij")
    return np.stack([fCenter[0] + fx.ravel(), fCenter[1] + fy.ravel()], axis=1)


def buildParticleForBlock(fCenter, fWidth, fHeight, fThickness, fOffset) -> np.ndarray:
    """Lattice points of a box (Solid.jl:492-509); the thickness is not snapped, as in the reference."""
    fWidth = math.floor(fWidth / fOffset) * fOffset
    fHeight = math.floor(fHeight / fOffset) * fOffset
    rz = julia_range(-0.5 * fThickness + 0.5 * fOffset, fOffset, +0.5 * fThickness - 0.5 * fOffset)
    ry = julia_range(-0.5 * fHeight + 0.5 * fOffset, fOffset, +0.5 * fHeight - 0.5 * fOffset)
    rx = julia_range(-0.5 * fWidth + 0.5 * fOffset, fOffset, +0.5 * fWidth - 0.5 * fOffset)
    fz, fy, fx = np.meshgrid(rz, ry, rx, indexing="ij")
    return np.stack([fCenter[0] + fx.ravel(), fCenter[1] + fy.ravel(), fCenter[2] + fz.ravel()], axis=1)


class _SolidBase:
    dim = 0

    def __init__(self, coords, mat):
        coords = np.ascontiguousarray(np.asarray(coords, dtype=np.float64).reshape(-1, self.dim))
        d = self.dim
        n = coords.shape[0]
        self.parCount = n
        self.mat = mat
        self.mass = np.full(n, float(mat.density))
        self.volumeInitial = np.zeros(n)
        self.volume = np.zeros(n)
        self.pos = coords.copy()
        self.pos0 = coords.copy()
        self.velocity = np.zeros((n, d))
        self.deformationGradient = matrix_array(n, d, identity=True)
        self.strain = matrix_array(n, d)
        self.stress = matrix_array(n, d)
        self.rigid = isinstance(mat, RigidMaterial)
        self.youngs = None
        # Solid.jl:93-96: surface classification, damage and crack force of the
        # TLMPM/phase-field solvers; written by the 2D dump, zeros here
        self.color = np.zeros(n)
        self.damage = np.zeros(n)
        self.crackForce = np.zeros(n)


class Solid2D(_SolidBase):
    """Solid2D(coords, mat), Solid.jl:104-125."""
    dim = 2


class Solid3D(_SolidBase):
    """Solid3D(coords, mat), Solid.jl:283-296."""
    dim = 3


def assign_velocity(solid, v0):
    """Solid.jl:532-537."""
    solid.velocity[:] = np.asarray(v0, dtype=np.float64).reshape(1, solid.dim)


def move(solid, dx):
    """Solid.jl:550-555."""
    solid.pos += np.asarray(dx, dtype=np.float64).reshape(1, solid.dim)
