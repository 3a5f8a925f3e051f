"""Problem set-ups of the benchmark workloads, written like jump's driver
scripts (Main_TwoDisks.jl:40-116, Main_TaylorBar.jl, Main_VibratingBeam.jl)
on the mirrored types.  Each returns (grid, solids, alg, data); inputs are
synthetic, generated from the stated geometry with seeded randomness.
"""
from __future__ import annotations

import math

import numpy as np

from .algorithm import USL, ConstantBodyForce2D, ConstantBodyForce3D
from .dirichlet import fix_Dirichlet_grid
from .grid import Grid2D, Grid3D
from .material import ElasticMaterial, ElastoPlasticMaterial, NeoHookeanMaterial
from .solid import (Solid2D, Solid3D, assign_velocity, buildParticleForCircle,
                    buildParticleForCylinder, buildParticleForRectangle)


def _scale(solid, off, d):
    vol = off ** d
    solid.mass *= vol  # solid.mass .*= dx*dx  (Main_TwoDisks.jl:69-71)
    solid.volume[:] = vol
    solid.volumeInitial[:] = vol


def two_disks(nodes: int = 21, ppc: int = 2, radius: float = 0.2, speed: float = 0.1,
              E: float = 1000.0, nu: float = 0.3, rho: float = 1000.0, dt: float = 1e-3,
              total_time: float = 3.0, fixed_boundary: bool = True, material: str = "elastic",
              centers=((0.2, 0.2), (0.8, 0.8))):
    """Two elastic disks colliding on [0,1]^2 (Main_TwoDisks.jl:40-116, linear basis)."""
    grid = Grid2D(0.0, 1.0, 0.0, 1.0, nodes, nodes)
    off = grid.dx / ppc
    c1 = buildParticleForCircle(list(centers[0]), radius, off)
    c2 = buildParticleForCircle(list(centers[1]), radius, off)
    if material == "elastic":
        mat = ElasticMaterial(E, nu, rho, 0, 0, len(c1))
        mats = (mat, mat)
    elif material == "neohookean":
        mats = (NeoHookeanMaterial(E, nu, rho, len(c1)), NeoHookeanMaterial(E, nu, rho, len(c2)))
    else:
        mats = (ElastoPlasticMaterial(E, nu, rho, 1.0, 10.0, len(c1)),
                ElastoPlasticMaterial(E, nu, rho, 1.0, 10.0, len(c2)))
    s1, s2 = Solid2D(c1, mats[0]), Solid2D(c2, mats[1])
    for s in (s1, s2):
        _scale(s, off, 2)
    assign_velocity(s1, [speed, speed])
    assign_velocity(s2, [-speed, -speed])
    data = {"total_time": total_time, "dt": dt, "time": 0.0,
            "bodyforce": ConstantBodyForce2D([0.0, 0.0])}
    if fixed_boundary:
        data["dirichlet_grid"] = [("bottom", (1, 1)), ("top", (1, 1)), ("left", (1, 1)), ("right", (1, 1))]
    return grid, [s1, s2], USL(1e-9), data


def taylor_bar(h: float = 2.5e-4, ppc: int = 2, radius: float = 3.2e-3, length: float = 32.4e-3,
               width: float = 16e-3, height: float = 40e-3, gap: float = 0.0, speed: float = 190.0,
               E: float = 117e9, nu: float = 0.35, rho: float = 8930.0, fy: float = 400e6,
               k1: float = 100e6, cfl: float = 0.2):
    """Copper Taylor bar along z striking a rigid wall at z = 0 (J2, linear hardening).

    Grid cells of size h over width x width x height, a cylinder of the given
    radius and length built with buildParticleForCylinder (Solid.jl:447-465,
    half-length argument) at ppc particles per cell and axis, the z = 0 face
    fixed in z (the wall), dt = cfl*h/c with c the dilatational wave speed.
    """
    nx = int(round(width / h)) + 1
    nz = int(round(height / h)) + 1
    grid = Grid3D(0.0, width, 0.0, width, 0.0, height, nx, nx, nz)
    off = h / ppc
    center = [0.5 * width, 0.5 * width, gap + 0.5 * length]
    coords = buildParticleForCylinder(center, radius, 0.5 * length, off, off, axis=2)
    mat = ElastoPlasticMaterial(E, nu, rho, fy, k1, len(coords))
    s = Solid3D(coords, mat)
    _scale(s, off, 3)
    assign_velocity(s, [0.0, 0.0, -speed])
    c = math.sqrt((mat.lambda_ + 2 * mat.mu) / rho)
    dt = cfl * h / c
    data = {"total_time": 80e-6, "dt": dt, "time": 0.0,
            "bodyforce": ConstantBodyForce3D([0.0, 0.0, 0.0]),
            "dirichlet_grid": [("front", (0, 0, 1))]}
    # Nodal-mass cutoff of 1e-3 particle masses: with USL(0.) near-empty nodes at
    # the mushrooming impact face give runaway velocities after ~110 steps.
    return grid, [s], USL(1e-3 * float(s.mass[0])), data


TAYLOR_MATERIALS = ("j2", "jc", "jcdamage")


def taylor_material(solid, material: str, h: float = 2.5e-4) -> str:
    """Replace the Taylor bar's J2 copper by another of the reference drivers'
    materials (SI units, cellsize one grid cell h); returns a label.

    jc:       the Johnson-Cook copper of Main_TaylorBar.jl:43-56
    jcdamage: the Johnson-Cook steel with damage of Main_Taylor_Bar_Frac_FEMP.jl:41-61
    """
    from .material import JohnsonCookDamage, JohnsonCookMaterial, JohnsonCookMaterialWithDamage
    n = solid.parCount
    if material == "j2":
        return "J2 linear hardening"
    if material == "jc":
        solid.mat = JohnsonCookMaterial(115e9, 0.31, 8940.0, 65e6, 356e6, 0.0, 0.37, 1e-3, 0.0, 0.0, 0.0, h, n)
        return "Johnson-Cook (A 65 MPa, B 356 MPa, n 0.37, C 0)"
    if material == "jcdamage":
        st = JohnsonCookMaterial(200e9, 0.33, 7850.0, 490e6, 383e6, 0.0123, 0.45, 0.5, 0.94, 0.9, 452.0, h, n)
        solid.mat = JohnsonCookMaterialWithDamage(st, JohnsonCookDamage(0.0705, 1.732, -0.54, 0.015, 0.0, 0.5,
                                                                        293.0, 1800.0, n))
        return "Johnson-Cook with damage (steel: A 490 MPa, B 383 MPa, n 0.45, C 0.0123; D1-D4)"
    raise ValueError(f"unknown Taylor-bar material {material}")


def cantilever(h: float = 0.0625, ppc: int = 4, length: float = 4.0, depth: float = 1.0,
               E_range=(0.5e6, 2e6), nu: float = 0.3, rho: float = 1050.0, g: float = -10.0,
               dt: float = 1e-4, seed: int = 0):
    """A 4 m x 1 m neo-Hookean beam clamped at x = 0 under gravity, with a
    per-particle Young's modulus drawn log-uniform in E_range (seeded)."""
    nx = int(round(4.5 / h)) + 1
    ny = int(round(4.0 / h)) + 1
    grid = Grid2D(0.0, 4.5, 0.0, 4.0, nx, ny)
    off = h / ppc
    coords = buildParticleForRectangle([0.5 * length, 2.5], length, depth, off)
    mat = NeoHookeanMaterial(math.sqrt(E_range[0] * E_range[1]), nu, rho, len(coords))
    s = Solid2D(coords, mat)
    _scale(s, off, 2)
    rng = np.random.default_rng(seed)
    s.youngs = np.exp(rng.uniform(math.log(E_range[0]), math.log(E_range[1]), len(coords)))
    data = {"total_time": 2000 * dt, "dt": dt, "time": 0.0,
            "bodyforce": ConstantBodyForce2D([0.0, g]),
            "dirichlet_grid": [("left", (1, 1))]}
    return grid, [s], USL(1e-9), data


def ensemble_member(i: int, seed: int = 0, gap=None):
    """Instance i of the seeded two-disk ensemble: radii in [0.1, 0.25],
    20..80 cells per axis, 4 particles per cell, E in [500, 5000], speed in
    [0.05, 0.2], dt = 5e-4.  The disks start at (0.3, 0.3) and (0.7, 0.7), or,
    with ``gap``, along that diagonal with their rims ``gap`` apart.  The nodal
    mass cutoff is 1e-3 particle masses (with 1e-9 some seeded problems run
    away once the disks collide)."""
    rng = np.random.default_rng([seed, i])
    r1, r2 = rng.uniform(0.1, 0.25, 2)
    cells = int(rng.integers(20, 81))
    E = float(rng.uniform(500.0, 5000.0))
    speed = float(rng.uniform(0.05, 0.2))
    grid = Grid2D(0.0, 1.0, 0.0, 1.0, cells + 1, cells + 1)
    off = grid.dx / 2
    p1, p2 = (0.3, 0.3), (0.7, 0.7)
    if gap is not None:
        d = (float(r1) + float(r2) + gap) / math.sqrt(2.0)
        p1, p2 = (0.5 - 0.5 * d, 0.5 - 0.5 * d), (0.5 + 0.5 * d, 0.5 + 0.5 * d)
    c1 = buildParticleForCircle(list(p1), float(r1), off)
    c2 = buildParticleForCircle(list(p2), float(r2), off)
    mat = ElasticMaterial(E, 0.3, 1000.0, 0, 0, max(len(c1), len(c2)))
    s1, s2 = Solid2D(c1, mat), Solid2D(c2, mat)
    for s in (s1, s2):
        _scale(s, off, 2)
    assign_velocity(s1, [speed, speed])
    assign_velocity(s2, [-speed, -speed])
    data = {"total_time": 1000 * 5e-4, "dt": 5e-4, "time": 0.0,
            "bodyforce": ConstantBodyForce2D([0.0, 0.0]),
            "dirichlet_grid": [("bottom", (1, 1)), ("top", (1, 1)), ("left", (1, 1)), ("right", (1, 1))]}
    return grid, [s1, s2], USL(1e-3 * float(s1.mass[0])), data


def apply_dirichlet(grid, data):
    fix_Dirichlet_grid(grid, data, ghostcell="ghostcell" in data)


def sphere_plate(h: float = 5e-4, ppc: int = 2, radius: float = 5e-3, speed: float = 50.0,
                 E_sphere: float = 200e9, rho_sphere: float = 7800.0, E_plate: float = 5e9,
                 rho_plate: float = 1200.0, nu: float = 0.3, plate=(20e-3, 20e-3, 4e-3), margin: float = 2e-3,
                 cfl: float = 0.2, gap=None):
    """An elastic steel sphere striking a neo-Hookean plate (two bodies, contact mode).

    The plate rests on the z = 0 face (fixed in z); the sphere starts one cell
    above it (``gap``, default one cell).  Contact uses one velocity field per body with the frictionless
    normal correction.  The plate density is not given by the workload
    description; 1200 kg/m^3 is used.
    """
    from .material import ElasticMaterial
    from .solid import buildParticleForBlock, buildParticleForSphere
    wx, wy, tz = plate
    gap = h if gap is None else gap
    lx = wx + 2 * margin
    lz = tz + 2 * radius + h + 2 * margin
    nx = int(round(lx / h)) + 1
    nz = int(round(lz / h)) + 1
    grid = Grid3D(0.0, lx, 0.0, lx, 0.0, (nz - 1) * h, nx, nx, nz)
    off = h / ppc
    cs = buildParticleForSphere([0.5 * lx, 0.5 * lx, tz + gap + radius], radius, off)
    cp = buildParticleForBlock([0.5 * lx, 0.5 * lx, 0.5 * tz], wx, wy, tz, off)
    ms = ElasticMaterial(E_sphere, nu, rho_sphere, len(cs))
    mp = NeoHookeanMaterial(E_plate, nu, rho_plate, len(cp))
    s1, s2 = Solid3D(cs, ms), Solid3D(cp, mp)
    for s in (s1, s2):
        _scale(s, off, 3)
    assign_velocity(s1, [0.0, 0.0, -speed])
    c = math.sqrt((ms.lambda_ + 2 * ms.mu) / rho_sphere)
    data = {"total_time": 1e-4, "dt": cfl * h / c, "time": 0.0,
            "bodyforce": ConstantBodyForce3D([0.0, 0.0, 0.0]),
            "dirichlet_grid": [("front", (0, 0, 1))], "contact": True, "friction": 0.0}
    return grid, [s1, s2], USL(1e-3 * float(s2.mass[0])), data


def impact_member(i: int, seed: int = 0, h: float = 5e-4, gap: float = 0.0):
    """Instance i of the seeded sphere-on-plate impact ensemble: the
    sphere_plate problem (steel sphere r = 5 mm, neo-Hookean plate 20x20x4 mm,
    2x2x2 particles per cell, two velocity fields with the frictionless
    contact correction) with the impact speed uniform in [10, 100] m/s and the
    plate's Young's modulus uniform in [1e9, 10e9] Pa.  The sphere starts
    touching the plate (``gap`` = 0) so that every step of a short solve is
    in contact."""
    rng = np.random.default_rng([seed, i])
    speed = float(rng.uniform(10.0, 100.0))
    E_plate = float(rng.uniform(1e9, 10e9))
    return sphere_plate(h=h, speed=speed, E_plate=E_plate, gap=gap)


def block_3d(h: float = 0.125, ppc: int = 2, size=(1.0, 0.25, 0.25), E_range=(0.5e6, 2e6), nu: float = 0.3,
             rho: float = 1050.0, g: float = -10.0, dt: float = 1e-4, seed: int = 0):
    """A neo-Hookean block clamped at x = 0 sagging under gravity, with a
    per-particle Young's modulus (log-uniform, seeded): the 3D counterpart of
    the cantilever inverse problem."""
    from .solid import buildParticleForBlock
    lx, ly, lz = size
    nx, ny, nz = int(round((lx + 0.25) / h)) + 1, int(round((ly + 0.75) / h)) + 1, int(round((lz + 0.25) / h)) + 1
    grid = Grid3D(0.0, (nx - 1) * h, 0.0, (ny - 1) * h, 0.0, (nz - 1) * h, nx, ny, nz)
    off = h / ppc
    coords = buildParticleForBlock([0.5 * lx, 0.5 + 0.5 * ly, 0.125 + 0.5 * lz], lx, ly, lz, off)
    mat = NeoHookeanMaterial(math.sqrt(E_range[0] * E_range[1]), nu, rho, len(coords))
    s = Solid3D(coords, mat)
    _scale(s, off, 3)
    rng = np.random.default_rng(seed)
    s.youngs = np.exp(rng.uniform(math.log(E_range[0]), math.log(E_range[1]), len(coords)))
    data = {"total_time": 200 * dt, "dt": dt, "time": 0.0, "bodyforce": ConstantBodyForce3D([0.0, g, 0.0]),
            "dirichlet_grid": [("left", (1, 1, 1))]}
    return grid, [s], USL(1e-9), data


def rigid_punch(dim: int = 2, h: float = 0.025, ppc: int = 2, radius: float = 0.2, speed: float = 0.1,
                E: float = 1000.0, nu: float = 0.3, rho: float = 1000.0, dt: float = 1e-3,
                material: str = "elastic"):
    """A rigid plate striking a deformable disk (sphere in 3D) that rests on a fixed
    rigid base, in the manner of the reference's lateral-compression drivers
    (Main_LateralCompressionTube.jl:116-117: a moving RigidMaterial punch and a
    still one).  The base fills y in [h, 3h] and is ``fixed`` (zero nodal momentum
    under it); the disk sits half a cell above it; the punch, 4h thick, starts
    1.5 cells above the disk and moves along -y at ``speed``.  Unit domain,
    h-spaced grid, every face fixed in every direction."""
    from .material import RigidMaterial
    from .solid import buildParticleForBlock, buildParticleForSphere
    n = int(round(1.0 / h)) + 1
    off = h / ppc
    cy = 3.5 * h + radius
    py = cy + radius + 1.5 * h + 2 * h
    if dim == 2:
        grid = Grid2D(0.0, 1.0, 0.0, 1.0, n, n)
        cd = buildParticleForCircle([0.5, cy], radius, off)
        cp = buildParticleForRectangle([0.5, py], 0.5, 4 * h, off)
        cb = buildParticleForRectangle([0.5, 2 * h], 0.6, 2 * h, off)
        S, v = Solid2D, [0.0, -speed]
        base = RigidMaterial(0.0, 0.0, 7800.0, fixed=True)
        punch = RigidMaterial(0.0, -speed, 7800.0)
        faces = [("bottom", (1, 1)), ("top", (1, 1)), ("left", (1, 1)), ("right", (1, 1))]
    else:
        grid = Grid3D(0.0, 1.0, 0.0, 1.0, 0.0, 1.0, n, n, n)
        cd = buildParticleForSphere([0.5, cy, 0.5], radius, off)
        cp = buildParticleForBlock([0.5, py, 0.5], 0.5, 4 * h, 0.5, off)
        cb = buildParticleForBlock([0.5, 2 * h, 0.5], 0.6, 2 * h, 0.6, off)
        S, v = Solid3D, [0.0, -speed, 0.0]
        base = RigidMaterial(0.0, 0.0, 0.0, 7800.0, fixed=True)
        punch = RigidMaterial(0.0, -speed, 0.0, 7800.0)
        faces = [("bottom", (1, 1, 1)), ("top", (1, 1, 1)), ("left", (1, 1, 1)), ("right", (1, 1, 1)),
                 ("front", (1, 1, 1)), ("back", (1, 1, 1))]
    if material == "elastic":
        mat = ElasticMaterial(E, nu, rho, len(cd))
    else:
        mat = NeoHookeanMaterial(E, nu, rho, len(cd))
    disk, pl, bs = S(cd, mat), S(cp, punch), S(cb, base)
    for s in (disk, pl, bs):
        _scale(s, off, dim)
    assign_velocity(pl, v)  # the punch's particles carry its velocity (energy records)
    bf = ConstantBodyForce2D([0.0, 0.0]) if dim == 2 else ConstantBodyForce3D([0.0, 0.0, 0.0])
    data = {"total_time": 200 * dt, "dt": dt, "time": 0.0, "bodyforce": bf, "dirichlet_grid": faces}
    return grid, [disk, pl, bs], USL(1e-9), data
