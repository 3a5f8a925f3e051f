"""Host mirror of the reference types (no GPU)."""
import numpy as np
import pytest

import jump_gb300 as J
from jump_gb300 import scenarios
from jump_gb300.output import jfloat
from jump_gb300.problem import step_times


def test_grid2d_matches_reference_constructor():
    g = J.Grid2D(0.0, 1.0, 0.0, 2.0, 5, 9)
    assert g.dx == 0.25 and g.dy == 0.25 and g.nodeCount == 45 and g.cellCount == 32
    # node I (1-based) = nx*(j-1) + i  -> position (xmin + (i-1)dx, ymin + (j-1)dy)
    assert tuple(g.pos[J.to_1D_index(3, 4, g) - 1]) == (0.5, 0.75)
    assert list(g.bottomNodes) == [0, 1, 2, 3, 4]
    assert list(g.leftNodes[:3]) == [0, 5, 10] and list(g.rightNodes[:2]) == [4, 9]
    assert g.fixedNodes.shape == (2, 45) and g.fixedNodes.flags["F_CONTIGUOUS"]


def test_grid3d_faces():
    g = J.Grid3D(0, 1, 0, 1, 0, 1, 3, 4, 5)
    assert g.nodeCount == 60 and g.nodeCountXY == 12
    assert np.all(g.pos[g.frontNodes, 2] == 0.0) and np.all(g.pos[g.backNodes, 2] == 1.0)
    assert np.all(g.pos[g.bottomNodes, 1] == 0.0) and np.all(g.pos[g.topNodes, 1] == 1.0)
    assert np.all(g.pos[g.leftNodes, 0] == 0.0) and np.all(g.pos[g.rightNodes, 0] == 1.0)


def test_dirichlet():
    g = J.Grid2D(0, 1, 0, 1, 4, 4)
    J.fix_Dirichlet_grid(g, {"dirichlet_grid": [("bottom", (0, 1)), ("left", (1, 1))]})
    assert g.fixedNodes[1, 1] == 1 and g.fixedNodes[0, 1] == 0
    assert g.fixedNodes[0, 4] == 1 and g.fixedNodes[1, 4] == 1
    with pytest.raises(ValueError):
        J.fix_Dirichlet_grid(g, {"dirichlet_grid": [("front", (1, 1))]})


def test_julia_range_lengths():
    assert len(J.julia_range(-0.1875, 0.025, 0.1875)) == 16
    r = J.julia_range(0.0, 0.1, 1.0)
    assert len(r) == 11 and r[3] == 0.30000000000000004 or r[3] == 0.3


def test_generator_counts_match_reference_configs():
    g, s, alg, data = scenarios.two_disks()
    assert [x.parCount for x in s] == [208, 208]
    g, s, alg, data = scenarios.cantilever()
    assert s[0].parCount == 16384


@pytest.mark.slow
def test_taylor_bar_count():
    g, s, alg, data = scenarios.taylor_bar()
    assert s[0].parCount == 511784 and g.nodeCount == 65 * 65 * 161


def test_step_count_matches_while_loop():
    # `while t < Tf; t += dt` runs one extra step for Tf = 3.0, dt = 1e-3
    assert len(step_times(0.0, 3.0, 1e-3)) == 3001
    assert len(step_times(0.0, 0.5, 5e-4)) == 1000


def test_jfloat_prints_like_julia():
    assert jfloat(1e-5) == "1.0e-5" and jfloat(0.25) == "0.25" and jfloat(3.0) == "3.0"
    assert jfloat(1.5e-7) == "1.5e-7" and jfloat(1e16) == "1.0e16"


def test_material_constants():
    m = J.ElasticMaterial(1000.0, 0.3, 1000.0, 0, 0, 3)
    assert m.lambda_ == 1000.0 * 0.3 / 1.3 / (1 - 0.6) and getattr(m, "lambda") == m.lambda_
    p = J.ElastoPlasticMaterial(117e9, 0.35, 8930, 400e6, 100e6, 2)
    assert p.kappa == p.lambda_ + p.mu


def test_johnson_cook_with_damage_descriptor():
    """JohnsonCookMaterialWithDamage(strength, damage) packs as material type 5 with
    the strength part's constants, chi, Cp, m and the damage constants, and passes
    its state arrays (damage_init, dam, damage_part.temp starting at Tr, vmStr)."""
    import ctypes as C
    from jump_gb300 import _capi
    from jump_gb300.engine import Descriptors
    g, s, alg, data = scenarios.taylor_bar(h=1e-3, radius=2e-3, length=6e-3, width=8e-3, height=10e-3)
    scenarios.apply_dirichlet(g, data)
    n = s[0].parCount
    st = J.JohnsonCookMaterial(200e9, 0.33, 7850.0, 490e6, 383e6, 0.0123, 0.45, 0.5, 0.94, 0.9, 452.0, 1e-3, n)
    s[0].mat = J.JohnsonCookMaterialWithDamage(st, J.JohnsonCookDamage(0.07, 1.7, -0.5, 0.015, 0.1, 0.5,
                                                                       293.0, 1800.0, n))
    assert s[0].mat.E == 200e9 and s[0].mat.alpha is st.alpha  # the strength part's constants and state
    assert np.all(s[0].mat.damage_part.temp == 293.0) and s[0].mat.damage_part.Tmr == 1800.0 - 293.0
    d = Descriptors(g, s, tolerance=alg.tolerance, dt=data["dt"])
    m = d.bodies[0].mat
    assert m.type == _capi.MPM_MAT_JOHNSON_COOK_DAMAGE == 5
    assert (m.E, m.nu, m.density, m.A, m.B, m.C, m.n, m.epsdot0) == (200e9, 0.33, 7850.0, 490e6, 383e6, 0.0123,
                                                                     0.45, 0.5)
    assert (m.m, m.chi, m.Cp) == (0.94, 0.9, 452.0)
    assert (m.d1, m.d2, m.d3, m.d4, m.d5, m.depsdot0, m.Tr, m.Tm) == (0.07, 1.7, -0.5, 0.015, 0.1, 0.5, 293.0, 1800.0)
    b = d.bodies[0]
    for k in ("damage_init", "damage", "temperature", "alpha", "alphadot", "vmstr"):
        assert C.cast(getattr(b, k), C.c_void_p).value is not None, k
    assert b.temperature[0] == 293.0
    assert not b.pstrain  # the damage state replaces J2's plastic strain
