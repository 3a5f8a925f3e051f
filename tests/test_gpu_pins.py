"""The oracle's external pins (tests/test_oracle_pins.py) on the GPU path: closed
forms of one material point, the hat basis seen through the P2G of a single
particle, conservation on the free two-disk collision, and the second-order
convergence of the standing-wave manufactured solution."""
import math

import numpy as np
import pytest

import pins
from jump_gb300.algorithm import ConstantBodyForce2D, ConstantBodyForce3D
from jump_gb300.engine import Descriptors, MPMContext
from jump_gb300.grid import Grid2D, Grid3D
from jump_gb300.material import ElasticMaterial, NeoHookeanMaterial
from jump_gb300.solid import Solid2D, Solid3D

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("on_node", [False, True])
def test_single_particle_p2g_is_the_hat_basis(dim, on_node):
    """One particle of mass m, velocity v and stress sigma: after one step the grid
    holds m N_I, m N_I v and -V sigma grad N_I, with N_I = prod_a (1 - |x_a - X_a|/h)
    and the gradient of the hat formula (the sign(0) = 0 factor on a node line)."""
    h = 0.125
    g = Grid2D(0.0, 1.0, 0.0, 1.0, 9, 9) if dim == 2 else Grid3D(0.0, 1.0, 0.0, 1.0, 0.0, 1.0, 9, 9, 9)
    x = np.array([[3 * h if on_node else 0.4137, 0.5921, 0.2713][:dim]])
    s = (Solid2D if dim == 2 else Solid3D)(x, ElasticMaterial(1e3, 0.3, 1000.0, 1))
    m, V = 0.75, 2e-3
    s.mass[:] = m
    s.volume[:] = V
    s.volumeInitial[:] = V
    v = np.array([0.3, -0.2, 0.1][:dim])
    s.velocity[0] = v
    sig = np.array([[2.0, 0.5, -0.3], [0.5, -1.0, 0.7], [-0.3, 0.7, 1.5]])[:dim, :dim]
    s.stress[0] = sig
    bf = ConstantBodyForce2D([0.0, 0.0]) if dim == 2 else ConstantBodyForce3D([0.0, 0.0, 0.0])
    c = MPMContext(Descriptors(g, [s], tolerance=0.0, body_force=bf, dt=1e-6))
    c.step(1)
    mass, p0, _, f = c.download_grid(g.nodeCount)
    c.close()
    ids = np.nonzero(mass)[0] if not on_node else None
    # every node of the particle's cell, from the formula
    base = np.floor(x[0] / h).astype(int)
    nodes, Nf, dNf = [], [], []
    for k in range(1 << dim):
        off = np.array([(k >> a) & 1 for a in range(dim)])
        idx = base + off
        X = idx * h
        d = x[0] - X
        fac = 1 - np.abs(d) / h
        grad = -np.sign(d) / h
        nid = idx[0] + 9 * idx[1] + (81 * idx[2] if dim == 3 else 0)
        nodes.append(nid)
        Nf.append(np.prod(fac))
        dNf.append([grad[a] * np.prod(np.delete(fac, a)) for a in range(dim)])
    nodes, Nf, dNf = np.array(nodes), np.array(Nf), np.array(dNf)
    assert np.allclose(mass[nodes], m * Nf, rtol=0, atol=1e-15)
    assert abs(mass.sum() - m) <= 1e-15
    assert np.allclose(p0[nodes], m * Nf[:, None] * v[None, :], rtol=0, atol=1e-15)
    assert np.allclose(f[nodes], -V * dNf @ sig.T, rtol=0, atol=1e-14)
    if on_node:
        # the x-gradients sum to 1/h: the internal forces do not cancel
        assert np.allclose(f.sum(axis=0), -V * sig[:, 0] / h, rtol=1e-12, atol=1e-15)
    else:
        assert set(ids) == set(nodes[Nf > 0])
        assert np.all(np.abs(f.sum(axis=0)) <= 1e-13 * V * np.abs(sig).max() / h)


@pytest.mark.parametrize("dim", [2, 3])
def test_elastic_point_closed_form_gpu(dim):
    E, nu = 2e9, 0.3
    rng = np.random.default_rng(dim)
    a = rng.normal(scale=1e-3, size=(dim, dim))
    eps = 0.5 * (a + a.T)
    sig, *_ = pins.point_state(MPMContext, dim, ElasticMaterial(E, nu, 1000.0, 1), strain=eps)
    want = pins.elastic_closed_form(E, nu, eps)
    assert np.max(np.abs(sig - want)) <= 1e-12 * np.max(np.abs(want))


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("stretch", [0.8, 1.25])
def test_neohookean_uniaxial_closed_form_gpu(dim, stretch):
    E, nu = 1e6, 0.3
    F = np.eye(dim)
    F[0, 0] = stretch
    sig, *_ = pins.point_state(MPMContext, dim, NeoHookeanMaterial(E, nu, 1000.0, 1), F=F)
    want = pins.neohookean_uniaxial(E, nu, stretch, dim)
    assert np.max(np.abs(sig - want)) <= 1e-12 * np.max(np.abs(want))


@pytest.mark.parametrize("dim", [2, 3])
def test_j2_monotonic_shear_closed_form_gpu(dim):
    E, nu, fy, k1 = 117e9, 0.35, 400e6, 100e6
    _, mu = pins.lame(E, nu)
    onset = fy / (2 * mu * math.sqrt(2.0))
    eps = np.linspace(0.25, 6.0, 24) * onset
    hist = pins.j2_shear_history(MPMContext, dim, E, nu, 8930.0, fy, k1, eps)
    for e, (alpha, s12, _) in zip(eps, hist):
        a_ex, s_ex = pins.j2_shear_closed_form(E, nu, fy, k1, e)
        assert abs(alpha - a_ex) <= 1e-12 * max(a_ex, onset), (e, alpha, a_ex)
        assert abs(s12 - s_ex) <= 1e-12 * abs(s_ex), (e, s12, s_ex)


def test_two_disks_free_conservation_gpu():
    recs, mass, pscale, m_grid = pins.two_disks_free(MPMContext, pins.MOMENTUM_STEPS, 0.0)
    assert abs(m_grid - mass) <= 1e-13 * mass
    p = np.array([r[2] for r in recs])
    assert np.max(np.abs(p)) <= 1e-13 * pscale
    recs, *_ = pins.two_disks_free(MPMContext, 3001, pins.ENERGY_TOL)
    e = np.array([r[0] + r[1] for r in recs])
    assert np.max(np.abs(e - e[0])) <= 0.08 * e[0]


def test_mms_standing_wave_second_order_gpu():
    errs = [pins.mms_errors(MPMContext, n) for n in (8, 16, 32, 64, 128)]
    eu = [e[0] for e in errs]
    orders = [math.log2(eu[k] / eu[k + 1]) for k in range(len(eu) - 1)]
    assert all(o >= 1.9 for o in orders), (eu, orders)
