"""Fixes: per-interval recorders called by the solver (Fix.jl:29-357).

``compute(fix, t)`` and ``closeFile(fix)`` keep the reference semantics and
text formats.  EnergiesFix can also be fed device-reduced sums
(``record``), which lets the solver skip a full particle download when no
other hook needs the particle arrays.
"""
from __future__ import annotations

import os

import numpy as np

from .output import jfloat


class FixBase:
    needs_particles = True

    def close(self):
        f = getattr(self, "file", None)
        if f is not None and not f.closed:
            f.close()


class EmptyFix(FixBase):
    """Fix.jl:34-35, 208-212: does nothing."""
    needs_particles = False

    def compute(self, time):
        pass


def _open_fresh(filename):
    """rm the file if it exists, then open it for appending (Fix.jl:61-67,
    111-114); a missing directory is an error, as there."""
    if os.path.isfile(filename):
        os.remove(filename)
    return open(filename, "a")


class EnergiesFix(FixBase):
    """KE = sum 1/2 m v.v and SE = sum 1/2 V sum(sigma .* eps), one line per call
    (Fix.jl:104-117, 248-270)."""
    needs_particles = False

    def __init__(self, solids, filename):
        self.solids = solids
        self.file = _open_fresh(filename)
        self.kinEnergy, self.strEnergy, self.recordTime = [], [], []

    def compute(self, time):
        # the reference's summation order: particles left to right across the solids,
        # dot(v, v) and sum(stress .* strain) over components in column-major order
        ke_terms, se_terms = [np.zeros(1)], [np.zeros(1)]
        for solid in self.solids:
            if solid.parCount == 0:
                continue
            v, st, ep = solid.velocity, solid.stress, solid.strain
            d = v.shape[1]
            dot = v[:, 0] * v[:, 0]
            for a in range(1, d):
                dot = dot + v[:, a] * v[:, a]
            ke_terms.append(0.5 * solid.mass * dot)
            se = st[:, 0, 0] * ep[:, 0, 0]
            for j in range(d):
                for i in range(d):
                    if i or j:
                        se = se + st[:, i, j] * ep[:, i, j]
            se_terms.append(0.5 * solid.volume * se)
        KE = float(np.cumsum(np.concatenate(ke_terms))[-1])
        SE = float(np.cumsum(np.concatenate(se_terms))[-1])
        self.record(time, KE, SE)

    def record(self, time, KE, SE):
        self.kinEnergy.append(KE)
        self.strEnergy.append(SE)
        self.recordTime.append(time)
        self.file.write(f"{jfloat(time)} {jfloat(KE)} {jfloat(SE)}\n")


class DisplacementFix(FixBase):
    """Position minus initial position of the particle found at ``point``
    (Fix.jl:37-102, 214-218).  As in the reference, the match uses x and y
    only, takes the first matching particle of a solid, and a later solid with
    a match replaces an earlier one."""

    def __init__(self, solids, point, dir):
        point = np.asarray(point, dtype=np.float64)
        self.solids = solids
        self.index = None
        for s, solid in enumerate(solids):
            dx = solid.pos[:, 0] - point[0]
            dy = solid.pos[:, 1] - point[1]
            hit = np.nonzero(np.sqrt(dx * dx + dy * dy) < 1e-10)[0]
            if hit.size:
                self.index = (s, int(hit[0]))
        if self.index is None:
            raise ValueError("No particle with that position found\n")
        self.file = _open_fresh(dir + "recorded-position.txt")  # string(dir, "recorded-position.txt")

    def compute(self, time):
        s, p = self.index
        solid = self.solids[s]
        x = solid.pos[p] - solid.pos0[p]
        self.file.write(f"{jfloat(time)} {jfloat(x[0])} {jfloat(x[1])}\n")


def compute(fixes, time):
    """compute(fix, t) on one fix or a list of fixes."""
    if isinstance(fixes, FixBase):
        fixes.compute(time)
        return
    for f in fixes:
        f.compute(time)


def closeFile(fixes):
    if isinstance(fixes, FixBase):
        fixes.close()
        return
    for f in fixes:
        f.close()


def as_list(fixes):
    return [fixes] if isinstance(fixes, FixBase) else list(fixes)
