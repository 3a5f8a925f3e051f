"""Edge cases of the step on the GPU against the oracle: an empty body among
others, a single-particle body, the smallest grid (two nodes per axis), a
particle that leaves the grid (frozen, MPM_ERR_OUT_OF_GRID), det F <= 0
(MPM_ERR_NEGATIVE_J, the state still advanced), a non-finite stress
(MPM_ERR_NONFINITE) and particles exactly on grid nodes (zero gradient
factors)."""
import numpy as np
import pytest

from cases import descriptors, field_errors
from jump_gb300 import _capi, scenarios
from jump_gb300.engine import MPMContext
from jump_gb300.grid import Grid2D
from jump_gb300.material import ElasticMaterial
from jump_gb300.solid import Solid2D

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10


def worst(errs):
    return sorted(errs.items(), key=lambda kv: -kv[1])[:3]


def particles(xs, vs, E=1e3, rho=1000.0, vol=1e-4):
    s = Solid2D(np.asarray(xs, dtype=np.float64).reshape(-1, 2), ElasticMaterial(E, 0.3, rho, max(1, len(xs))))
    s.mass[:] = rho * vol
    s.volume[:] = vol
    s.volumeInitial[:] = vol
    if len(xs):
        s.velocity[:] = np.asarray(vs, dtype=np.float64).reshape(-1, 2)
    return s


def close(sg, so, E=1e3):
    """Kinematic fields relative to their size; strain and stress against the
    material's scale (they are rounding noise around zero for a rigid motion)."""
    errs = field_errors(sg, so, fields=("pos", "velocity", "volume", "F"))
    assert max(errs.values()) <= FP64_TOL, worst(errs)
    for a, b in zip(sg, so):
        assert np.max(np.abs(a.strain - b.strain), initial=0.0) <= 1e-12
        assert np.max(np.abs(a.stress - b.stress), initial=0.0) <= 1e-12 * E


def run_pair(grid, solids, tol, dt, oracle_lib, steps):
    mk = lambda: descriptors(grid, solids, tol, None, dt)
    g, o = MPMContext(mk()), oracle_lib.OracleContext(mk())
    rg = g.step(steps, check=False)
    ro = o.step(steps, check=False)
    return g, o, rg, ro


def test_empty_body_among_others(oracle_lib):
    grid, solids, alg, data = scenarios.two_disks(nodes=21)
    scenarios.apply_dirichlet(grid, data)
    bodies = [solids[0], particles([], []), solids[1]]
    g, o, rg, ro = run_pair(grid, bodies, alg.tolerance, data["dt"], oracle_lib, 50)
    assert rg == ro == _capi.MPM_OK
    sg, so = g.download_all(), o.download_all()
    assert sg[1].pos.shape == (0, 2)
    errs = field_errors([sg[0], sg[2]], [so[0], so[2]])
    assert max(errs.values()) <= FP64_TOL, worst(errs)


def test_single_particle_body(oracle_lib):
    grid = Grid2D(0.0, 1.0, 0.0, 1.0, 11, 11)
    g, o, rg, ro = run_pair(grid, [particles([[0.43, 0.51]], [[0.2, -0.1]])], 0.0, 1e-3, oracle_lib, 40)
    assert rg == ro == _capi.MPM_OK
    close(g.download_all(), o.download_all())


def test_smallest_grid(oracle_lib):
    grid = Grid2D(0.0, 1.0, 0.0, 1.0, 2, 2)
    xs = [[0.25, 0.25], [0.75, 0.25], [0.25, 0.75], [0.75, 0.75]]
    vs = [[0.01, 0.0], [-0.01, 0.0], [0.0, 0.02], [0.0, -0.02]]
    g, o, rg, ro = run_pair(grid, [particles(xs, vs, vol=0.0625)], 0.0, 1e-3, oracle_lib, 30)
    assert rg == ro == _capi.MPM_OK
    sg, so = g.download_all(), o.download_all()
    assert np.abs(so[0].strain).max() > 1e-6  # the four particles squeeze the one cell
    close(sg, so)


def test_particle_leaving_the_grid_is_frozen(oracle_lib):
    grid = Grid2D(0.0, 1.0, 0.0, 1.0, 11, 11)
    xs = [[0.45, 0.5], [0.55, 0.5], [0.95, 0.5]]
    vs = [[0.0, 0.0], [0.0, 0.0], [60.0, 0.0]]  # the last one crosses x = 1 within a few steps
    g, o, rg, ro = run_pair(grid, [particles(xs, vs)], 0.0, 1e-3, oracle_lib, 20)
    assert rg == ro == _capi.MPM_ERR_OUT_OF_GRID
    sg, so = g.download_all(), o.download_all()
    assert sg[0].pos[2, 0] > 1.0 - 0.1  # it reached the last cell before it was frozen
    close(sg, so)
    before = sg[0].pos.copy()
    g.step(5, check=False)
    after = g.download_all()[0].pos
    np.testing.assert_array_equal(after[2], before[2])  # frozen: no further motion


def test_negative_jacobian_reported_and_state_advanced(oracle_lib):
    grid = Grid2D(0.0, 1.0, 0.0, 1.0, 11, 11)
    s = particles([[0.42, 0.51], [0.47, 0.53]], [[0.1, 0.0], [-0.1, 0.0]])  # one cell: they interact
    s.deformationGradient[0] = np.array([[-1.0, 0.0], [0.0, 1.0]])  # det F < 0
    g, o, rg, ro = run_pair(grid, [s], 0.0, 1e-3, oracle_lib, 10)
    assert rg == ro == _capi.MPM_ERR_NEGATIVE_J
    sg, so = g.download_all(), o.download_all()
    assert sg[0].volume[0] < 0 and np.any(sg[0].pos != s.pos) and np.abs(so[0].strain).max() > 1e-6
    close(sg, so)


def test_nonfinite_stress_reported():
    grid = Grid2D(0.0, 1.0, 0.0, 1.0, 11, 11)
    s = particles([[0.43, 0.51], [0.61, 0.47]], [[0.1, 0.0], [-0.1, 0.0]])
    s.stress[1] = np.array([[np.nan, 0.0], [0.0, 0.0]])  # symmetric, but not finite
    c = MPMContext(descriptors(grid, [s], 0.0, None, 1e-3))
    assert c.step(1, check=False) == _capi.MPM_ERR_NONFINITE
    # the NaN positions leave the grid on the next step: reported, not a fault
    with pytest.raises(_capi.MPMError) as e:
        c.step(1)
    assert e.value.code in (_capi.MPM_ERR_NONFINITE, _capi.MPM_ERR_OUT_OF_GRID)


@pytest.mark.parametrize("dim", [2, 3])
def test_particles_on_grid_nodes(dim, oracle_lib):
    """A lattice of particles on grid nodes, cell faces and cell midpoints (node
    spacing 0.25, particle spacing 0.125, exact in binary): x - x_lower == 0
    makes a gradient factor exactly zero, a case the step's hat (stored by P2G,
    reused by G2P with FP64 particles) must carry through; an expansion moves
    them off the nodes over the run."""
    from jump_gb300.grid import Grid3D
    from jump_gb300.solid import Solid3D
    ax = np.arange(0.25, 0.76, 0.125)
    if dim == 2:
        grid = Grid2D(0.0, 1.0, 0.0, 1.0, 5, 5)
        xs = np.array([[a, b] for a in ax for b in ax])
    else:
        grid = Grid3D(0.0, 1.0, 0.0, 1.0, 0.0, 1.0, 5, 5, 5)
        xs = np.array([[a, b, c] for a in ax for b in ax for c in ax])
    vol = 0.125 ** dim
    s = (Solid2D if dim == 2 else Solid3D)(xs, ElasticMaterial(1e3, 0.3, 1000.0, len(xs)))
    s.mass[:] = 1000.0 * vol
    s.volume[:] = vol
    s.volumeInitial[:] = vol
    s.velocity[:] = 0.01 * (xs - 0.5)
    g, o, rg, ro = run_pair(grid, [s], 0.0, 1e-3, oracle_lib, 10)
    assert rg == ro == _capi.MPM_OK
    sg, so = g.download_all(), o.download_all()
    assert np.abs(so[0].strain).max() > 1e-5
    close(sg, so)
