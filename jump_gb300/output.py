"""Particle output hooks (Output.jl:40-57, 146-290), host side.

``OvitoOutput`` writes the reference's LAMMPS dump text files from the
particle arrays downloaded before each hook.  Floats are printed the way
Julia's string interpolation prints a Float64.  PyPlot figures and VTK files
are not produced (graphics/plotting stacks are outside this build).
"""
from __future__ import annotations

import glob
import os


def jfloat(x: float) -> str:
    """Julia's shortest round-trip printing of a Float64 ("1.0e-5", "0.25", "3.0")."""
    x = float(x)
    s = repr(x)
    if s in ("inf", "-inf", "nan"):
        return {"inf": "Inf", "-inf": "-Inf", "nan": "NaN"}[s]
    if "e" in s:
        mant, exp = s.split("e")
        if "." not in mant:
            mant += ".0"
        return f"{mant}e{int(exp)}"
    return s


class OutputType:
    def __init__(self, interval: int):
        self.interval = int(interval)

    needs_particles = False

    def plot(self, solids, lims, ncells, counter):
        pass


class EmptyOutput(OutputType):
    """An output that only sets the hook interval."""


class OvitoOutput(OutputType):
    """OvitoOutput(interval, dir, outs): LAMMPS dumps dir * "dump_p.<counter>.LAMMPS"
    (Output.jl:40-57).  As in the reference, file names are the plain
    concatenation of dir and the name (dir normally ends in a separator), an
    existing dir loses its dir * "*.LAMMPS" files and a missing one is made
    with a one-level mkdir."""
    needs_particles = True

    def __init__(self, interval: int, dir: str, outs):
        super().__init__(interval)
        self.dir = dir
        self.outs = list(outs)
        if os.path.isdir(dir):
            for f in glob.glob(glob.escape(dir) + "*.LAMMPS"):
                os.remove(f)
        else:
            os.mkdir(dir)

    def plot(self, solids, lims, ncells, counter):
        d = solids[0].dim if solids else 2
        if d == 2:
            plotParticles_2D(self, solids, lims, ncells, counter)
        else:
            plotParticles_3D(self, solids, lims, ncells, counter)


def _header(f, parCount, lims, d, outs):
    f.write("ITEM: TIMESTEP \n0\nITEM: NUMBER OF ATOMS\n")
    f.write(f"{parCount} \n")
    f.write("ITEM: BOX BOUNDS sm sm sm\n")
    f.write(f"0 {jfloat(lims[0])}\n0 {jfloat(lims[1])}\n")
    f.write("0 0\n" if d == 2 else f"0 {jfloat(lims[2])}\n")
    f.write("ITEM: ATOMS id type x y z ")
    for v in outs:
        f.write(v + " ")
    f.write("\n")


def _elastic(mat):
    from .material import ElasticMaterial, RigidMaterial
    return isinstance(mat, (ElasticMaterial, RigidMaterial))


def plotParticles_2D(plot: OvitoOutput, solids, lims, ncells, counter: int):
    """Output.jl:146-222."""
    n = sum(s.parCount for s in solids)
    with open(plot.dir + f"dump_p.{int(counter)}.LAMMPS", "a") as f:
        _header(f, n, lims, 2, plot.outs)
        pid = 0
        for s, solid in enumerate(solids, start=1):
            el = _elastic(solid.mat)
            x, st, vel = solid.pos, solid.stress, solid.velocity
            for p in range(solid.parCount):
                pid += 1
                f.write(f"{pid} {s} {jfloat(x[p, 0])} {jfloat(x[p, 1])} 0 ")
                for v in plot.outs:
                    if v == "pstrain":
                        f.write("0 " if el else f"{jfloat(solid.mat.alpha[p])} ")
                    elif v == "vonMises":
                        f.write("0 " if el else f"{jfloat(solid.mat.vmStr[p])} ")
                    elif v == "sigmaxx":
                        f.write(f"{jfloat(st[p, 0, 0])} ")
                    elif v == "sigmayy":
                        f.write(f"{jfloat(st[p, 1, 1])} ")
                    elif v == "pressure":
                        f.write(f"{jfloat(st[p, 0, 0] + st[p, 1, 1])} ")
                    elif v == "vx":
                        f.write(f"{jfloat(vel[p, 0])}  ")
                    elif v == "vy":
                        f.write(f"{jfloat(vel[p, 1])}  ")
                    elif v == "damage":
                        f.write(f"{jfloat(solid.damage[p])}  ")
                    elif v == "crackforce":
                        f.write(f"{jfloat(solid.crackForce[p])}  ")
                    elif v == "color":
                        f.write(f"{jfloat(solid.color[p])}  ")
                f.write("\n")


def plotParticles_3D(plot: OvitoOutput, solids, lims, ncells, counter: int):
    """Output.jl:224-290."""
    n = sum(s.parCount for s in solids)
    with open(plot.dir + f"dump_p.{int(counter)}.LAMMPS", "a") as f:
        _header(f, n, lims, 3, plot.outs)
        pid = 0
        for s, solid in enumerate(solids, start=1):
            from .material import ElasticMaterial
            el = isinstance(solid.mat, ElasticMaterial)
            x, st, vel = solid.pos, solid.stress, solid.velocity
            for p in range(solid.parCount):
                pid += 1
                f.write(f"{pid} {s} {jfloat(x[p, 0])} {jfloat(x[p, 1])} {jfloat(x[p, 2])} ")
                for v in plot.outs:
                    if v == "pstrain":
                        f.write("0 " if el else f"{jfloat(solid.mat.alpha[p])} ")
                    elif v == "vonMises":
                        f.write("0 " if el else f"{jfloat(solid.mat.vmStr[p])} ")
                    elif v == "vx":
                        f.write(f"{jfloat(vel[p, 0])}  ")
                    elif v == "vy":
                        f.write(f"{jfloat(vel[p, 1])}  ")
                    elif v == "vz":
                        f.write(f"{jfloat(vel[p, 2])}  ")
                    elif v == "pressure":
                        f.write(f"{jfloat((st[p, 0, 0] + st[p, 1, 1]) + st[p, 2, 2])}  ")
                f.write("\n")
