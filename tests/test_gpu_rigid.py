"""Rigid solids (RigidMaterial) on the GPU against the oracle: the grid-update
override of SolveExplicitSolidMechanics2D.jl:448-479 (nodal momenta m_I v_rigid
in the non-zero components, zero for a fixed body, later bodies last) and the
rigid advance of :539-551, with a rigid plate striking a disk that rests on a
fixed rigid base (2D and 3D), the quadratic B-spline basis, the cell sort, FP32
particles, two rigid bodies overriding one node, and the configurations that
reject rigid solids."""
import copy

import numpy as np
import pytest

from cases import descriptors, field_errors, rel_err
from jump_gb300 import _capi, scenarios
from jump_gb300.engine import MPMContext
from jump_gb300.material import ElasticMaterial, RigidMaterial
from jump_gb300.solid import Solid2D, buildParticleForRectangle

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10


def _pair(problem, oracle, steps, **kw):
    grid, solids, alg, data = problem
    scenarios.apply_dirichlet(grid, data)
    mk = lambda: descriptors(grid, solids, alg.tolerance, data["bodyforce"], data["dt"], **kw)
    g = MPMContext(mk())
    o = oracle.OracleContext(mk(), threads=4)
    g.step(steps)
    o.step(steps)
    return g, o, grid


@pytest.mark.parametrize("dim,steps,material", [(2, 200, "elastic"), (3, 210, "neohookean")])
def test_rigid_punch_vs_oracle(dim, steps, material, oracle_lib):
    kw = {} if dim == 2 else {"h": 0.05}
    prob = scenarios.rigid_punch(dim=dim, material=material, **kw)
    p0 = [s.pos.copy() for s in prob[1]]
    g, o, grid = _pair(prob, oracle_lib, steps)
    sg, so = g.download_all(), o.download_all()
    assert np.abs(so[0].strain).max() > 0.1, "the punch must load the disk"
    errs = field_errors(sg, so)
    assert max(errs.values()) <= FP64_TOL, sorted(errs.items(), key=lambda kv: -kv[1])[:4]
    # the punch moved by steps * dt * v exactly as the oracle adds it; the fixed base did not move
    assert np.array_equal(sg[1].pos, so[1].pos)
    assert np.array_equal(sg[2].pos, p0[2])
    dy = sg[1].pos[:, 1] - p0[1][:, 1]
    assert np.allclose(dy, -0.1 * steps * prob[3]["dt"], rtol=1e-12)
    # rigid particles keep their other fields
    assert np.all(sg[1].stress == 0.0) and np.all(sg[2].strain == 0.0)
    # the grid arrays of the last step carry the override
    for a, b in zip(g.download_grid(grid.nodeCount), o.download_grid(grid.nodeCount)):
        assert rel_err(a, b) <= 1e-12
    g.close()


def test_rigid_punch_quadratic_basis_and_sort(oracle_lib):
    """The override uses each rigid particle's linear cell whatever the basis;
    the cell sort moves rigid particles like any other."""
    prob = scenarios.rigid_punch(dim=2)
    g, o, _ = _pair(prob, oracle_lib, 150, basis="quad", sort_interval=4)
    errs = field_errors(g.download_all(), o.download_all())
    assert max(errs.values()) <= FP64_TOL, sorted(errs.items(), key=lambda kv: -kv[1])[:4]


def test_rigid_punch_fp32(oracle_lib):
    prob = scenarios.rigid_punch(dim=2)
    g, o, _ = _pair(prob, oracle_lib, 150, precision="f32")
    errs = field_errors(g.download_all(), o.download_all(), fields=("pos", "velocity", "F"))
    # stated FP32 bound of this case: 1e-4 relative per field
    assert max(errs.values()) <= 1e-4, errs


def _two_rigid_bodies():
    """A deformable block under two overlapping rigid bars: the first moves along
    +x only, the second along -y only, so nodes they share take x from the first
    and y from the second (each body sets only its non-zero components)."""
    from jump_gb300.algorithm import USL, ConstantBodyForce2D
    from jump_gb300.grid import Grid2D
    h = 0.05
    grid = Grid2D(0.0, 1.0, 0.0, 1.0, 21, 21)
    off = h / 2
    blk = Solid2D(buildParticleForRectangle([0.5, 0.4], 0.4, 0.3, off), ElasticMaterial(1000.0, 0.3, 1000.0, 1))
    a = Solid2D(buildParticleForRectangle([0.45, 0.6], 0.3, 0.1, off), RigidMaterial(0.05, 0.0, 2000.0))
    b = Solid2D(buildParticleForRectangle([0.55, 0.6], 0.3, 0.1, off), RigidMaterial(0.0, -0.05, 2000.0))
    for s in (blk, a, b):
        s.mass *= off * off
        s.volume[:] = off * off
        s.volumeInitial[:] = off * off
    data = {"dt": 1e-3, "bodyforce": ConstantBodyForce2D([0.0, 0.0]),
            "dirichlet_grid": [("bottom", (1, 1))]}
    return grid, [blk, a, b], USL(1e-9), data


def test_two_rigid_bodies_share_nodes(oracle_lib):
    g, o, grid = _pair(_two_rigid_bodies(), oracle_lib, 100)
    sg, so = g.download_all(), o.download_all()
    assert np.abs(so[0].strain).max() > 1e-3
    errs = field_errors(sg, so)
    assert max(errs.values()) <= FP64_TOL, sorted(errs.items(), key=lambda kv: -kv[1])[:4]
    m, p0, p, f = g.download_grid(grid.nodeCount)
    mo, p0o, po, fo = o.download_grid(grid.nodeCount)
    assert rel_err(p, po) <= 1e-12 and rel_err(p0, p0o) <= 1e-12
    # somewhere both rigid velocities were imposed on one node: v = (0.05, -0.05)
    live = m > 1e-9
    v = p[live] / m[live][:, None]
    assert np.any(np.all(np.isclose(v, [0.05, -0.05], rtol=0, atol=1e-12), axis=1))


def test_rigid_rejected_where_unsupported():
    grid, solids, alg, data = scenarios.rigid_punch(dim=2)
    scenarios.apply_dirichlet(grid, data)
    mk = lambda **kw: descriptors(grid, solids, alg.tolerance, data["bodyforce"], data["dt"], **kw)
    for kw in ({"contact": True}, {"algorithm": "musl", "alpha": 0.99}):
        with pytest.raises(_capi.MPMError) as e:
            MPMContext(mk(**kw))
        assert e.value.code == _capi.MPM_ERR_UNSUPPORTED
    many = [solids[0]] + [copy.deepcopy(solids[1]) for _ in range(_capi.MPM_MAX_RIGID_BODIES + 1)]
    with pytest.raises(_capi.MPMError) as e:
        MPMContext(descriptors(grid, many, alg.tolerance, data["bodyforce"], data["dt"]))
    assert e.value.code == _capi.MPM_ERR_ARG
    from jump_gb300.batch import Ensemble
    with pytest.raises(_capi.MPMError) as e:
        Ensemble([scenarios.rigid_punch(dim=2)], precision="f64")
    assert e.value.code == _capi.MPM_ERR_UNSUPPORTED
