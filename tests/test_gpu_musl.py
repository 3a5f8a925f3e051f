"""MUSL on the GPU against the oracle: 2D with the blended consistent mass
matrix (conjugate-gradient solve on the device, banded Cholesky in the
oracle) and 3D with lumped mass, FLIP/PIC blends alpha = 1 and 0.99, elastic,
neo-Hookean and J2 bodies, with and without the cell sort; the solver entry
point with MUSL; rejected combinations."""
import math

import numpy as np
import pytest

from cases import descriptors, field_errors
from jump_gb300 import _capi, scenarios
from jump_gb300.algorithm import MUSL
from jump_gb300.engine import MPMContext

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10          # 3D lumped MUSL: same statements, summation order only
CG_TOL = 1e-9             # 2D: iterative (relative residual 1e-13) vs direct mass solve


def pair(problem, steps, oracle_lib, alpha, **kw):
    grid, solids, alg, data = problem
    scenarios.apply_dirichlet(grid, data)
    mk = lambda **k: descriptors(grid, solids, 0.0, data.get("bodyforce"), data["dt"], algorithm="musl",
                                 alpha=alpha, **k)
    dg, do = MPMContext(mk(**kw)), oracle_lib.OracleContext(mk())
    dg.step(steps)
    do.step(steps)
    return dg, do


def worst(errs):
    return sorted(errs.items(), key=lambda kv: -kv[1])[:3]


TOUCH = ((0.3, 0.3), (0.3 + 0.4 / math.sqrt(2.0), 0.3 + 0.4 / math.sqrt(2.0)))


@pytest.mark.parametrize("alpha", [1.0, 0.99])
@pytest.mark.parametrize("material", ["elastic", "neohookean", "j2"])
def test_musl_2d_consistent_mass_vs_oracle(alpha, material, oracle_lib):
    prob = scenarios.two_disks(nodes=21, centers=TOUCH, speed=0.3, material=material)
    dg, do = pair(prob, 100, oracle_lib, alpha)
    so = do.download_all()
    assert min(np.abs(b.strain).max() for b in so) > 1e-6, "the disks must deform"
    errs = field_errors(dg.download_all(), so)
    assert max(errs.values()) <= CG_TOL, worst(errs)
    ke_g, se_g, _ = dg.energies()
    ke_o, se_o, _ = do.energies()
    assert abs(ke_g - ke_o) <= 1e-9 * ke_o and abs(se_g - se_o) <= 1e-8 * se_o


def test_musl_2d_gravity_vs_oracle(oracle_lib):
    # body force enters the 2D MUSL P2G; its Dirichlet update is never read, so the beam falls
    prob = scenarios.cantilever(h=0.125, ppc=2, length=1.0, depth=0.25)
    prob[1][0].youngs = None
    dg, do = pair(prob, 200, oracle_lib, 1.0)
    # a free fall does not strain the beam: its strain and stress are rounding noise
    errs = field_errors(dg.download_all(), do.download_all(), fields=("pos", "velocity", "F", "volume"))
    assert max(errs.values()) <= CG_TOL, worst(errs)


def test_musl_3d_lumped_taylor_vs_oracle(oracle_lib):
    # alpha 0.99: with alpha 1 the 3D solver's FLIP increment (p - p0)/m is zero at the
    # fixed wall nodes and the bar passes the wall undeformed (reference behaviour)
    prob = scenarios.taylor_bar(h=1e-3, radius=2e-3, length=6e-3, width=8e-3, height=10e-3, speed=300.0)
    dg, do = pair(prob, 60, oracle_lib, 0.99)
    so = do.download_all()
    assert np.abs(so[0].alpha).max() > 0, "particles must yield"
    errs = field_errors(dg.download_all(), so)
    assert max(errs.values()) <= FP64_TOL, worst(errs)


@pytest.mark.parametrize("material", ["elastic", "neohookean"])
def test_musl_3d_spheres_one_field_alpha1_vs_oracle(material, oracle_lib):
    """Two spheres colliding in one velocity field (they stick and deform), pure FLIP."""
    from jump_gb300.algorithm import ConstantBodyForce3D
    from jump_gb300.grid import Grid3D
    from jump_gb300.material import ElasticMaterial, NeoHookeanMaterial
    from jump_gb300.solid import Solid3D, assign_velocity, buildParticleForSphere
    g = Grid3D(0.0, 1.0, 0.0, 1.0, 0.0, 1.0, 21, 21, 21)
    off = g.dx / 2
    mk = ElasticMaterial if material == "elastic" else NeoHookeanMaterial
    c1 = buildParticleForSphere([0.4, 0.4, 0.45], 0.15, off)
    c2 = buildParticleForSphere([0.6, 0.6, 0.55], 0.15, off)
    s1, s2 = Solid3D(c1, mk(1e3, 0.3, 1000.0, len(c1))), Solid3D(c2, mk(1e3, 0.3, 1000.0, len(c2)))
    for so in (s1, s2):
        so.mass *= off ** 3
        so.volume[:] = off ** 3
        so.volumeInitial[:] = off ** 3
    assign_velocity(s1, [0.3, 0.3, 0.2])
    assign_velocity(s2, [-0.3, -0.3, -0.2])
    data = {"dt": 1e-3, "bodyforce": ConstantBodyForce3D([0.0, 0.0, 0.0]),
            "dirichlet_grid": [("front", (0, 0, 1))]}
    dg, do = pair((g, [s1, s2], None, data), 150, oracle_lib, 1.0)
    so = do.download_all()
    assert min(np.abs(b.strain).max() for b in so) > 1e-4
    errs = field_errors(dg.download_all(), so)
    assert max(errs.values()) <= FP64_TOL, worst(errs)


def test_musl_3d_spheres_with_sort_vs_oracle(oracle_lib):
    prob = scenarios.sphere_plate(h=2e-3, gap=0.0, speed=20.0)
    prob[3]["contact"] = False
    dg, do = pair(prob, 80, oracle_lib, 0.99, sort_interval=7)
    so = do.download_all()
    assert np.abs(so[1].strain).max() > 1e-7
    errs = field_errors(dg.download_all(), so)
    assert max(errs.values()) <= FP64_TOL, worst(errs)


def test_musl_grid_download_vs_oracle(oracle_lib):
    prob = scenarios.two_disks(nodes=21, centers=TOUCH, speed=0.3)
    dg, do = pair(prob, 30, oracle_lib, 1.0)
    nn = prob[0].nodeCount
    for a, b in zip(dg.download_grid(nn), do.download_grid(nn)):
        assert np.max(np.abs(a - b)) <= 1e-12 * max(np.max(np.abs(b)), 1e-300)


def test_solver_entry_with_musl(oracle_lib):
    """solve_explicit_dynamics_2D(grid, solids, LinearBasis(), MUSL(alpha), ...) mutates the solids
    like the oracle run of the same steps."""
    from jump_gb300 import EmptyOutput, LinearBasis, solve_explicit_dynamics_2D
    from jump_gb300.problem import step_times
    grid, solids, alg, data = scenarios.two_disks(nodes=21, centers=TOUCH, speed=0.3)
    data["total_time"] = 0.05
    scenarios.apply_dirichlet(grid, data)
    o = oracle_lib.OracleContext(descriptors(grid, solids, 0.0, data["bodyforce"], data["dt"],
                                             algorithm="musl", alpha=0.99))
    o.step(len(step_times(data["time"], data["total_time"], data["dt"])))
    solve_explicit_dynamics_2D(grid, solids, LinearBasis(), MUSL(0.99), EmptyOutput(1000), [], data)
    for s, st in zip(solids, o.download_all()):
        assert np.max(np.abs(s.pos - st.pos)) <= 1e-12


def test_musl_rejects_fp32_and_contact():
    import ctypes as C
    grid, solids, alg, data = scenarios.two_disks(nodes=11)
    scenarios.apply_dirichlet(grid, data)
    L = _capi.lib()
    for kw in ({"precision": "f32"}, {"contact": True}):
        d = descriptors(grid, solids, 0.0, data["bodyforce"], data["dt"], algorithm="musl", alpha=1.0, **kw)
        h = C.c_void_p()
        rc = L.mpm_create(C.byref(d.grid), d.bodies, d.nbodies, C.byref(d.params), C.byref(h))
        assert rc == _capi.MPM_ERR_UNSUPPORTED, kw
