"""External pins of the CPU oracle: known answers that do not come from another
restatement of the reference.

* the hat basis (Basis.jl:219-251, 292-332): partition of unity, zero gradient
  sum, linear reproduction, and the sign(0) = 0 gradient of a point on a node
  line (Basis.jl:247-248), which makes that sum 1/h instead of 0;
* the B-spline bases (Basis.jl:374-820, Bsplines.jl): partition of unity and
  zero gradient sum, and the one place the reference's constant 0.6666666667
  (Bsplines.jl:167) breaks the former;
* constitutive updates of one material point against closed forms: linear
  elastic (Material.jl:68-81), neo-Hookean under uniaxial stretch (:119-122), J2
  radial return under monotonic shear with linear hardening (:174-275);
* the two-disk collision (Main_TwoDisks.jl) without boundary conditions: total
  mass on the grid equals the particles' mass, linear momentum is conserved,
  and KE + SE stays within a stated band (the reference plots it, :119-138);
* the standing-wave manufactured solution of Main_MMS_1D.jl: the displacement
  error falls at second order under refinement at fixed CFL.

The same checks run on the GPU in tests/test_gpu_pins.py."""
import math

import numpy as np
import pytest

import pins
from jump_gb300.engine import Descriptors
from jump_gb300.grid import Grid2D, Grid3D
from jump_gb300.material import ElasticMaterial, NeoHookeanMaterial


@pytest.fixture(scope="module")
def O(oracle_lib):
    return oracle_lib


def _desc(dim, nodes=9):
    g = Grid2D(0.0, 1.0, 0.0, 1.0, nodes, nodes) if dim == 2 else \
        Grid3D(0.0, 1.0, 0.0, 1.0, 0.0, 1.0, nodes, nodes, nodes)
    return g, Descriptors(g, [], dt=1e-3).grid


def _node_xyz(g, ids, dim):
    nx = g.nodeCountX
    ny = g.nodeCountY
    ix, iy = ids % nx, (ids // nx) % ny
    h = 1.0 / (nx - 1)
    out = [ix * h, iy * h]
    if dim == 3:
        out.append((ids // (nx * ny)) * h)
    return np.stack(out, axis=1)


@pytest.mark.parametrize("dim", [2, 3])
def test_hat_basis_properties(dim, O):
    g, gd = _desc(dim)
    h = 0.125  # 1/8: node coordinates are exact
    rng = np.random.default_rng(5)
    for _ in range(200):
        x = rng.uniform(0.01, 0.99, dim)
        ids, N, dN = O.shape(gd, 0, x)
        X = _node_xyz(g, ids, dim)
        # the hat values of the formula N_I = prod_a (1 - |x_a - X_a| / h)
        assert np.allclose(N, np.prod(1 - np.abs(x - X) / h, axis=1), rtol=0, atol=1e-15)
        assert abs(N.sum() - 1.0) <= 1e-15 and np.all(N >= 0)
        assert np.all(np.abs(dN.sum(axis=0)) <= 1e-13 / h)
        assert np.allclose((N[:, None] * X).sum(axis=0), x, rtol=0, atol=1e-15)  # linear reproduction
        # the gradient of a linear field: sum_I grad N_I X_I^T = identity
        assert np.allclose(dN.T @ X, np.eye(dim), rtol=0, atol=1e-13)


@pytest.mark.parametrize("dim", [2, 3])
def test_hat_gradient_on_a_node_line(dim, O):
    """x on the node line x = X_i: the lower node's x-factor is 1 with gradient
    -sign(0)/h = 0 and the upper node's is 0 with gradient +1/h, so the x-gradients
    sum to 1/h, not 0 (the reference's sign(0) = 0, Basis.jl:247-248)."""
    _, gd = _desc(dim)
    h = 0.125
    x = np.array([3 * h, 0.41, 0.29][:dim])
    ids, N, dN = O.shape(gd, 0, x)
    lower = (ids % 9) == 3
    assert np.all(dN[lower, 0] == 0.0)
    assert np.all(N[~lower] == 0.0)
    assert dN[:, 0].sum() == pytest.approx(1.0 / h, rel=1e-15)
    assert np.all(np.abs(dN[:, 1:].sum(axis=0)) <= 1e-13 / h)


@pytest.mark.parametrize("basis,dim", [(1, 2), (2, 2), (1, 3), (2, 3)])
def test_bspline_partition_of_unity(basis, dim, O):
    """Modified quadratic (basis 1) and cubic (2) B-splines sum to one with zero
    gradient sum everywhere on the grid, boundary cells included, except the cubic
    spline's cells next to a boundary where Bsplines.jl:167 writes 2/3 as
    0.6666666667: there the sum exceeds one by 3.3e-11 per axis."""
    g, gd = _desc(dim)
    h = 0.125
    rng = np.random.default_rng(7)
    worst_in, worst_edge = 0.0, 0.0
    for _ in range(400):
        x = rng.uniform(0.001, 0.999, dim)
        ids, N, dN = O.shape(gd, basis, x)
        dev = abs(N.sum() - 1.0)
        near_edge = np.any((x < 2 * h) | (x > 1 - 2 * h))
        if near_edge:
            worst_edge = max(worst_edge, dev)
        else:
            worst_in = max(worst_in, dev)
        assert np.all(np.abs(dN.sum(axis=0)) <= (1e-9 if basis == 2 and near_edge else 1e-12) / h)
    assert worst_in <= 1e-14
    if basis == 1:
        assert worst_edge <= 1e-14
    else:
        assert 1e-12 < worst_edge <= dim * 3.4e-11


# ---------------------------------------------------------------------------
# one material point


@pytest.mark.parametrize("dim", [2, 3])
def test_elastic_point_closed_form(dim, O):
    E, nu = 2e9, 0.3
    rng = np.random.default_rng(dim)
    a = rng.normal(scale=1e-3, size=(dim, dim))
    eps = 0.5 * (a + a.T)
    sig, *_ = pins.point_state(O.OracleContext, dim, ElasticMaterial(E, nu, 1000.0, 1), strain=eps)
    want = pins.elastic_closed_form(E, nu, eps)
    assert np.max(np.abs(sig - want)) <= 1e-12 * np.max(np.abs(want))


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("stretch", [0.8, 1.25])
def test_neohookean_uniaxial_closed_form(dim, stretch, O):
    E, nu = 1e6, 0.3
    F = np.eye(dim)
    F[0, 0] = stretch
    sig, *_ = pins.point_state(O.OracleContext, dim, NeoHookeanMaterial(E, nu, 1000.0, 1), F=F)
    want = pins.neohookean_uniaxial(E, nu, stretch, dim)
    assert np.max(np.abs(sig - want)) <= 1e-12 * np.max(np.abs(want))


@pytest.mark.parametrize("dim", [2, 3])
def test_j2_monotonic_shear_closed_form(dim, O):
    E, nu, fy, k1 = 117e9, 0.35, 400e6, 100e6
    _, mu = pins.lame(E, nu)
    onset = fy / (2 * mu * math.sqrt(2.0))
    eps = np.linspace(0.25, 6.0, 24) * onset
    hist = pins.j2_shear_history(O.OracleContext, dim, E, nu, 8930.0, fy, k1, eps)
    yielded = 0
    for e, (alpha, s12, sig) in zip(eps, hist):
        a_ex, s_ex = pins.j2_shear_closed_form(E, nu, fy, k1, e)
        assert abs(alpha - a_ex) <= 1e-12 * max(a_ex, onset), (e, alpha, a_ex)
        assert abs(s12 - s_ex) <= 1e-12 * abs(s_ex), (e, s12, s_ex)
        off = sig.copy()
        off[0, 1] = off[1, 0] = 0.0
        assert np.max(np.abs(off)) <= 1e-12 * abs(s_ex)  # pure shear stays pure shear
        yielded += alpha > 0
    assert 0 < yielded < len(eps)


# ---------------------------------------------------------------------------
# conservation


def test_two_disks_free_conservation(O):
    recs, mass, pscale, m_grid = pins.two_disks_free(O.OracleContext, pins.MOMENTUM_STEPS, 0.0, threads=1)
    assert abs(m_grid - mass) <= 1e-13 * mass  # partition of unity: all particle mass reaches the grid
    p = np.array([r[2] for r in recs])
    assert np.max(np.abs(p)) <= 1e-13 * pscale  # equal and opposite disks: momentum stays zero
    recs, *_ = pins.two_disks_free(O.OracleContext, 3001, pins.ENERGY_TOL, threads=1)
    e = np.array([r[0] + r[1] for r in recs])
    # stated band over the 3001 steps of the two-disk configuration: 8% of the initial
    # energy (the oracle's largest excursion, mid-collision, is 7.3%)
    assert np.max(np.abs(e - e[0])) <= 0.08 * e[0]
    assert np.min(np.array([r[1] for r in recs])) >= 0.0 and max(r[1] for r in recs) > 0.05 * e[0]


# ---------------------------------------------------------------------------
# manufactured solution


def test_mms_standing_wave_second_order(O):
    errs = [pins.mms_errors(O.OracleContext, n) for n in (8, 16, 32, 64)]
    eu = [e[0] for e in errs]
    orders = [math.log2(eu[k] / eu[k + 1]) for k in range(len(eu) - 1)]
    assert all(o >= 1.9 for o in orders), (eu, orders)
    assert eu[-1] <= 2.5e-4
