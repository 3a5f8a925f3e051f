"""Quadratic and cubic B-spline bases on the GPU against the oracle: USL in 2D
and 3D (FP64 within 1e-10, FP32 within a stated bound), with contact and
with the cell sort; MUSL in 2D (consistent mass, 25 / 49-entry stencil) and
3D (lumped); the solver entry point with a B-spline basis; grids too small
for the basis rejected."""
import ctypes as C
import math

import numpy as np
import pytest

from cases import descriptors, field_errors
from jump_gb300 import _capi, scenarios
from jump_gb300.engine import MPMContext

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
CG_TOL = 1e-9
TOUCH = ((0.3, 0.3), (0.3 + 0.4 / math.sqrt(2.0), 0.3 + 0.4 / math.sqrt(2.0)))


def pair(problem, steps, oracle_lib, **kw):
    grid, solids, alg, data = problem
    scenarios.apply_dirichlet(grid, data)
    tol = 0.0 if kw.get("algorithm") == "musl" else alg.tolerance
    okw = {k: v for k, v in kw.items() if k not in ("precision", "sort_interval")}
    dg = MPMContext(descriptors(grid, solids, tol, data.get("bodyforce"), data["dt"], **kw))
    do = oracle_lib.OracleContext(descriptors(grid, solids, tol, data.get("bodyforce"), data["dt"], **okw))
    dg.step(steps)
    do.step(steps)
    return dg, do


def worst(errs):
    return sorted(errs.items(), key=lambda kv: -kv[1])[:3]


@pytest.mark.parametrize("basis", ["quad", "cubic"])
@pytest.mark.parametrize("material", ["elastic", "neohookean", "j2"])
def test_usl_2d_vs_oracle(basis, material, oracle_lib):
    prob = scenarios.two_disks(nodes=21, centers=TOUCH, speed=0.3, material=material)
    dg, do = pair(prob, 100, oracle_lib, basis=basis)
    so = do.download_all()
    assert min(np.abs(b.strain).max() for b in so) > 1e-5
    errs = field_errors(dg.download_all(), so)
    assert max(errs.values()) <= FP64_TOL, worst(errs)


@pytest.mark.parametrize("basis", ["quad", "cubic"])
def test_usl_3d_taylor_vs_oracle(basis, oracle_lib):
    prob = scenarios.taylor_bar(h=1e-3, radius=2e-3, length=6e-3, width=8e-3, height=10e-3, speed=300.0)
    dg, do = pair(prob, 60, oracle_lib, basis=basis)
    so = do.download_all()
    assert so[0].alpha.max() > 0, "the bar must yield"
    errs = field_errors(dg.download_all(), so)
    assert max(errs.values()) <= FP64_TOL, worst(errs)


@pytest.mark.parametrize("basis", ["quad", "cubic"])
def test_usl_fp32_bound(basis, oracle_lib):
    prob = scenarios.two_disks(nodes=21, centers=TOUCH, speed=0.3)
    dg, do = pair(prob, 100, oracle_lib, basis=basis, precision="f32")
    errs = field_errors(dg.download_all(), do.download_all(), fields=("pos", "velocity", "stress", "F"))
    assert max(errs.values()) <= 1e-4, worst(errs)  # stated FP32 bound, B-spline two disks


def test_usl_cubic_with_sort_vs_oracle(oracle_lib):
    prob = scenarios.two_disks(nodes=31, centers=TOUCH, speed=0.3, material="neohookean")
    dg, do = pair(prob, 100, oracle_lib, basis="cubic", sort_interval=5)
    errs = field_errors(dg.download_all(), do.download_all())
    assert max(errs.values()) <= FP64_TOL, worst(errs)


@pytest.mark.parametrize("basis", ["quad", "cubic"])
def test_contact_3d_vs_oracle(basis, oracle_lib):
    grid, solids, alg, data = scenarios.sphere_plate(h=1e-3, gap=0.0, speed=100.0)
    scenarios.apply_dirichlet(grid, data)
    mk = lambda: descriptors(grid, solids, alg.tolerance, data.get("bodyforce"), data["dt"], contact=True,
                             basis=basis)
    dg, do = MPMContext(mk()), oracle_lib.OracleContext(mk())
    dg.step(40)
    do.step(40)
    so = do.download_all()
    assert np.abs(so[1].strain).max() > 1e-6
    errs = field_errors(dg.download_all(), so)
    assert max(errs.values()) <= CG_TOL, worst(errs)


@pytest.mark.parametrize("basis", ["quad", "cubic"])
@pytest.mark.parametrize("alpha", [1.0, 0.99])
def test_musl_2d_vs_oracle(basis, alpha, oracle_lib):
    prob = scenarios.two_disks(nodes=21, centers=TOUCH, speed=0.3, material="neohookean")
    dg, do = pair(prob, 80, oracle_lib, basis=basis, algorithm="musl", alpha=alpha)
    so = do.download_all()
    assert min(np.abs(b.strain).max() for b in so) > 1e-5
    errs = field_errors(dg.download_all(), so)
    assert max(errs.values()) <= CG_TOL, worst(errs)


@pytest.mark.parametrize("basis", ["quad", "cubic"])
def test_musl_3d_vs_oracle(basis, oracle_lib):
    prob = scenarios.taylor_bar(h=1e-3, radius=2e-3, length=6e-3, width=8e-3, height=10e-3, speed=300.0)
    dg, do = pair(prob, 60, oracle_lib, basis=basis, algorithm="musl", alpha=0.99)
    so = do.download_all()
    assert np.abs(so[0].strain).max() > 1e-4
    errs = field_errors(dg.download_all(), so)
    assert max(errs.values()) <= FP64_TOL, worst(errs)


def test_solver_entry_with_quadratic_basis(oracle_lib):
    """Main_TwoDisks.jl's setting: QuadBsplineBasis with USL."""
    from jump_gb300 import EmptyOutput, QuadBsplineBasis, solve_explicit_dynamics_2D
    from jump_gb300.problem import step_times
    grid, solids, alg, data = scenarios.two_disks(nodes=21, centers=TOUCH, speed=0.3)
    data["total_time"] = 0.05
    scenarios.apply_dirichlet(grid, data)
    o = oracle_lib.OracleContext(descriptors(grid, solids, alg.tolerance, data["bodyforce"], data["dt"],
                                             basis="quad"))
    o.step(len(step_times(data["time"], data["total_time"], data["dt"])))
    solve_explicit_dynamics_2D(grid, solids, QuadBsplineBasis(), alg, EmptyOutput(1000), [], data)
    for s, st in zip(solids, o.download_all()):
        assert np.max(np.abs(s.pos - st.pos)) <= 1e-12


def test_small_grid_rejected():
    grid, solids, alg, data = scenarios.two_disks(nodes=3, radius=0.1, centers=((0.3, 0.3), (0.7, 0.7)))
    scenarios.apply_dirichlet(grid, data)
    d = descriptors(grid, solids, alg.tolerance, data["bodyforce"], data["dt"], basis="cubic")
    L = _capi.lib()
    h = C.c_void_p()
    assert L.mpm_create(C.byref(d.grid), d.bodies, d.nbodies, C.byref(d.params), C.byref(h)) == _capi.MPM_ERR_ARG
