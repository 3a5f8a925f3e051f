"""solve_explicit_dynamics_2D / 3D for USL or MUSL with the linear, quadratic or
cubic B-spline basis: the drop-in
for Problem.solve_explicit_dynamics_2D (USL SolveExplicitSolidMechanics2D.jl:335-585,
MUSL :24-329) and solve_explicit_dynamics_3D (USL
SolveExplicitSolidMechanics3D.jl:230-378, MUSL :14-223).

The time loop, the hook schedule and the in-place mutation of ``solids`` and
``grid`` follow the reference; the step itself runs in libjumpmpm.so.
Steps between two hooks run on the device without host round trips.  Before
each hook the particle arrays are downloaded into ``solids`` (skipped when
the only hooks are EmptyFix/EnergiesFix and a non-writing output, in which case
the energies are reduced on the device).  The per-step ``@printf`` of the 2D
reference (:375) is not reproduced.

Extra ``data`` keys (all optional): "precision" ("f64" | "f32" | "dw": FP64
fields with the P2G and G2P arithmetic in double-word FP32, 3D USL),
"contact" (bool) with "friction" (float), "sort_interval" (int).
"""
from __future__ import annotations

import numpy as np

from . import _capi
from .algorithm import MUSL, USL, CubicBsplineBasis, LinearBasis, QuadBsplineBasis
from .dirichlet import fix_Dirichlet_grid
from .engine import Descriptors, MPMContext
from .fix import EnergiesFix, as_list, closeFile
from .material import ElastoPlasticMaterial, ElasticMaterial


HOOK_CHUNK = 4096  # EnergiesFix records per mpm_step_energies call


def step_times(t: float, Tf: float, dt: float):
    """The `t` of every iteration of `while t < Tf ... t += dtime` (:373, :580)."""
    ts = []
    while t < Tf:
        ts.append(t)
        t += dt
    return ts


def write_back(solids, states):
    """Copy downloaded body states into the Solid objects (in place, like the reference)."""
    for solid, st in zip(solids, states):
        F, eps, sig = st.matrices()
        solid.pos[:] = st.pos
        solid.velocity[:] = st.velocity
        solid.volume[:] = st.volume
        solid.deformationGradient[:] = F
        solid.strain[:] = eps
        solid.stress[:] = sig
        m = solid.mat
        n = solid.parCount
        if isinstance(m, ElastoPlasticMaterial):
            m.alpha[:n] = st.alpha
            if solid.dim == 2:
                m.pstrain[:n] = st.pstrain.reshape(n, 3)
            else:
                m.pstrain_3D[:n] = st.pstrain.reshape(n, 3, 3).transpose(0, 2, 1)
            m.vmStr[:n] = st.vmstr
        elif isinstance(m, ElasticMaterial) and solid.dim == 3:
            m.vmStr[:n] = st.vmstr
        elif getattr(m, "alphadot", None) is not None:  # Johnson-Cook / Voce / Johnson-Cook with damage
            m.alpha[:n] = st.alpha
            m.alphadot[:n] = st.alphadot
            m.vmStr[:n] = st.vmstr
            if getattr(m, "damage_part", None) is not None:
                m.damage_init[:n] = st.damage_init
                m.dam[:n] = st.damage
                m.damage_part.temp[:n] = st.temperature


def _solve(dim, grid, solids, basis, alg, output, fixes, data):
    if not isinstance(basis, (LinearBasis, QuadBsplineBasis, CubicBsplineBasis)):
        raise _capi.MPMError(_capi.MPM_ERR_UNSUPPORTED,
                             "the accelerated path supports LinearBasis, QuadBsplineBasis and CubicBsplineBasis")
    basis_name = ("quad" if isinstance(basis, QuadBsplineBasis) else
                  "cubic" if isinstance(basis, CubicBsplineBasis) else "linear")
    if not isinstance(alg, (USL, MUSL)):
        raise _capi.MPMError(_capi.MPM_ERR_UNSUPPORTED, "the accelerated path supports USL and MUSL")
    musl = isinstance(alg, MUSL)
    if grid.dim != dim or any(s.dim != dim for s in solids):
        raise ValueError(f"solve_explicit_dynamics_{dim}D needs a Grid{dim}D and Solid{dim}D objects")
    Tf = float(data["total_time"])
    dt = float(data["dt"])
    t = float(data["time"])
    bodyforce = data["bodyforce"] if dim == 2 else data.get("bodyforce")
    ghostcell = "ghostcell" in data
    fix_Dirichlet_grid(grid, data, ghostcell=ghostcell)

    desc = Descriptors(grid, solids, tolerance=0.0 if musl else alg.tolerance, body_force=bodyforce, dt=dt,
                       precision=data.get("precision", "f64"), contact=bool(data.get("contact", False)),
                       friction=float(data.get("friction", 0.0)),
                       sort_interval=int(data.get("sort_interval", 0)),
                       algorithm="musl" if musl else "usl", alpha=alg.alpha if musl else 1.0,
                       basis=basis_name)
    fl = as_list(fixes)
    need_particles = output.needs_particles or any(f.needs_particles for f in fl)
    times = step_times(t, Tf, dt)
    interval = max(1, int(output.interval))
    lims = list(grid.lengths)
    ncells = [grid.nodeCountX, grid.nodeCountY] + ([grid.nodeCountZ] if dim == 3 else [])
    ctx = MPMContext(desc)
    try:
        done = 0
        nsteps = len(times)
        states = None  # host arrays of the downloads, reused from hook to hook
        efix = [f for f in fl if isinstance(f, EnergiesFix)]
        while done < nsteps:
            if not need_particles:
                # no hook reads particle arrays: the remaining steps in calls of at most
                # HOOK_CHUNK hooks, the EnergiesFix sums of each hook step formed on
                # the device and copied back once per call, with no host round trip
                # between steps
                first = (-done) % interval
                run = min(nsteps - done, first + HOOK_CHUNK * interval)
                if efix:
                    recs, _ = ctx.step_energies(run, interval, first)
                    for j, r in enumerate(recs):
                        th = times[done + first + j * interval]
                        for f in efix:
                            f.record(th, r[0], r[1])
                else:
                    ctx.step(run)
                done += run
                continue
            # next hook step: the first counter >= done with counter % interval == 0
            nxt = ((done + interval - 1) // interval) * interval
            run = min(nsteps, nxt + 1) - done
            ctx.step(run)
            done += run
            counter = done - 1
            if counter % interval == 0:
                th = times[counter]
                states = ctx.download_all(states)
                write_back(solids, states)
                output.plot(solids, lims, ncells, counter)
                for f in fl:
                    f.compute(th)
        write_back(solids, ctx.download_all(states))
        m, p0, p, f = ctx.download_grid(grid.nodeCount)
        grid.mass[:] = m
        grid.momentum0[:] = p0
        grid.momentum[:] = p
        grid.force[:] = f
    finally:
        ctx.close()
    closeFile(fixes)


def solve_explicit_dynamics_2D(grid, solids, basis, alg, output, fixes, data):
    """USL or MUSL explicit dynamics on a Grid2D (SolveExplicitSolidMechanics2D.jl:335, :24)."""
    return _solve(2, grid, solids, basis, alg, output, fixes, data)


def solve_explicit_dynamics_3D(grid, solids, basis, alg, output, fixes, data):
    """USL or MUSL explicit dynamics on a Grid3D (SolveExplicitSolidMechanics3D.jl:230, :14)."""
    return _solve(3, grid, solids, basis, alg, output, fixes, data)
