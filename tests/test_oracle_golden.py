"""The CPU oracle reproduces the independent pure-Python restatement
(tests/golden/make_golden.py) bit for bit on every golden case."""
import numpy as np
import pytest

from cases import GOLDEN_CASES, descriptors, golden_expected, golden_kw, load_golden, rel_err


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_oracle_matches_golden_bitwise(name, oracle_lib):
    grid, solids, tol, bf, dt, nsteps, z = load_golden(name)
    desc = descriptors(grid, solids, tol, bf, dt, **golden_kw(z))
    ctx = oracle_lib.OracleContext(desc)
    t = ctx.step(nsteps, t=0.0)
    assert t > 0
    for b, st in enumerate(ctx.download_all()):
        exp = golden_expected(z, b)
        for k, v in exp.items():
            got = getattr(st, k).ravel()
            if k in ("alpha", "pstrain", "vmstr") and not np.any(v):
                # fields a material never writes stay as uploaded (zeros)
                assert not np.any(got), (name, b, k)
                continue
            np.testing.assert_array_equal(got, np.asarray(v).ravel(), err_msg=f"{name} body {b} {k}")
    m, p0, p, f = ctx.download_grid(grid.nodeCount)
    np.testing.assert_array_equal(m, z["grid_mass"])
    np.testing.assert_array_equal(p0, z["grid_momentum0"])
    np.testing.assert_array_equal(p, z["grid_momentum"])
    np.testing.assert_array_equal(f, z["grid_force"])


@pytest.mark.parametrize("name", ["two_disks_elastic_20", "taylor_mini_j2_6", "two_disks_quad_12",
                                  "spheres_nh_cubic_8"])
def test_oracle_threads_agree(name, oracle_lib):
    """Slab-coloured parallel P2G re-associates node sums only (differences at rounding level);
    slabs are as wide as a particle's support (2, 3 or 4 nodes)."""
    grid, solids, tol, bf, dt, nsteps, z = load_golden(name)
    a = oracle_lib.OracleContext(descriptors(grid, solids, tol, bf, dt, **golden_kw(z)), threads=1)
    b = oracle_lib.OracleContext(descriptors(grid, solids, tol, bf, dt, **golden_kw(z)), threads=4)
    a.step(nsteps)
    b.step(nsteps)
    for sa, sb in zip(a.download_all(), b.download_all()):
        for k in ("pos", "velocity", "stress", "F", "alpha"):
            assert rel_err(getattr(sb, k), getattr(sa, k)) <= 1e-10, k
