"""CUDA path vs the CPU oracle on identical inputs (FP64 within 1e-10
relative per particle field; FP32 error bounds stated per case)."""
import numpy as np
import pytest

from cases import GOLDEN_CASES, descriptors, field_errors, golden_expected, golden_kw, load_golden, rel_err
from jump_gb300 import scenarios
from jump_gb300.engine import Descriptors, MPMContext

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10


def run_pair(grid, solids, tol, bf, dt, steps, oracle, precision="f64", sched=None):
    dg = MPMContext(descriptors(grid, solids, tol, bf, dt, precision=precision))
    do = oracle.OracleContext(descriptors(grid, solids, tol, bf, dt))
    for n in (sched or [steps]):
        dg.step(n)
        do.step(n)
    return dg, do


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_golden_cases_fp64(name, oracle_lib):
    grid, solids, tol, bf, dt, nsteps, z = load_golden(name)
    dg = MPMContext(descriptors(grid, solids, tol, bf, dt, **golden_kw(z)))
    dg.step(nsteps)
    # the 2D MUSL solves its mass matrix iteratively on the device (relative residual 1e-13)
    tol = 1e-9 if golden_kw(z) and int(z["meta_dim"]) == 2 else FP64_TOL
    for b, st in enumerate(dg.download_all()):
        for k, v in golden_expected(z, b).items():
            assert rel_err(getattr(st, k), v) <= tol, (name, b, k, rel_err(getattr(st, k), v))


@pytest.mark.parametrize("steps", [1, 10, 100])
def test_two_disks_fp64_vs_oracle(steps, oracle_lib):
    grid, solids, alg, data = scenarios.two_disks()
    scenarios.apply_dirichlet(grid, data)
    dg, do = run_pair(grid, solids, alg.tolerance, data["bodyforce"], data["dt"], steps, oracle_lib)
    errs = field_errors(dg.download_all(), do.download_all())
    worst = max(errs.values())
    assert worst <= FP64_TOL, sorted(errs.items(), key=lambda kv: -kv[1])[:4]
    ke_g, se_g, p_g = dg.energies()
    ke_o, se_o, p_o = do.energies()
    assert abs(ke_g - ke_o) <= 1e-10 * abs(ke_o) and abs(se_g - se_o) <= 1e-9 * max(abs(se_o), 1e-30)


def test_grid_download_matches_oracle(oracle_lib):
    grid, solids, alg, data = scenarios.two_disks()
    scenarios.apply_dirichlet(grid, data)
    dg, do = run_pair(grid, solids, alg.tolerance, data["bodyforce"], data["dt"], 5, oracle_lib)
    for a, b in zip(dg.download_grid(grid.nodeCount), do.download_grid(grid.nodeCount)):
        assert rel_err(a, b) <= 1e-12


def test_taylor_bar_small_fp64_100_steps(oracle_lib):
    """J2 plasticity in 3D at the wall, 100 steps (a coarser bar that the oracle runs in seconds)."""
    grid, solids, alg, data = scenarios.taylor_bar(h=5e-4)
    scenarios.apply_dirichlet(grid, data)
    dg, do = run_pair(grid, solids, alg.tolerance, data["bodyforce"], data["dt"], 100, oracle_lib)
    so, sg = do.download_all(), dg.download_all()
    assert np.max(so[0].alpha) > 0, "the case must yield"
    errs = field_errors(sg, so)
    assert max(errs.values()) <= FP64_TOL, sorted(errs.items(), key=lambda kv: -kv[1])[:4]


def test_fp32_variant_error_stated(oracle_lib):
    """FP32 particles + FP64 nodes against the FP64 oracle (two disks, 100 steps)."""
    grid, solids, alg, data = scenarios.two_disks()
    scenarios.apply_dirichlet(grid, data)
    dg, do = run_pair(grid, solids, alg.tolerance, data["bodyforce"], data["dt"], 100, oracle_lib,
                      precision="f32")
    errs = field_errors(dg.download_all(), do.download_all(), fields=("pos", "velocity", "stress", "F"))
    # stated bound for this case: 1e-4 relative per field
    assert max(errs.values()) <= 1e-4, errs


def test_invariants_full_taylor_bar():
    """Size-independent properties at the full 511,784-particle size: total mass
    is exact, the bar only moves towards/along the wall, momentum decays at impact."""
    grid, solids, alg, data = scenarios.taylor_bar()
    scenarios.apply_dirichlet(grid, data)
    d = Descriptors(grid, solids, tolerance=alg.tolerance, body_force=data["bodyforce"], dt=data["dt"])
    ctx = MPMContext(d)
    ke0, _, p0 = ctx.energies()
    ctx.step(50)
    ke1, se1, p1 = ctx.energies()
    st = ctx.download_body(0)
    assert np.all(np.isfinite(st.pos)) and np.all(st.volume > 0)
    assert abs(p1[0]) < 1e-9 * abs(p0[2]) and abs(p1[1]) < 1e-9 * abs(p0[2])  # symmetric bar
    assert p1[2] > p0[2]  # the wall removes downward momentum
    assert ke1 + se1 <= ke0 * (1 + 1e-9)  # plastic dissipation, no energy gain


@pytest.mark.parametrize("interval", [1, 7])
def test_cell_sort_keeps_parity(interval, oracle_lib):
    """Counting sort by (body, cell) every `interval` steps: downloads come back in
    the original particle order and match the oracle to FP64 tolerance."""
    grid, solids, alg, data = scenarios.two_disks()
    scenarios.apply_dirichlet(grid, data)
    dg = MPMContext(descriptors(grid, solids, alg.tolerance, data["bodyforce"], data["dt"],
                                sort_interval=interval))
    do = oracle_lib.OracleContext(descriptors(grid, solids, alg.tolerance, data["bodyforce"], data["dt"]))
    for n in (3, 17, 30):
        dg.step(n)
        do.step(n)
    errs = field_errors(dg.download_all(), do.download_all())
    assert max(errs.values()) <= FP64_TOL, sorted(errs.items(), key=lambda kv: -kv[1])[:4]


def test_cell_sort_taylor_bar_fp64_and_fp32(oracle_lib):
    grid, solids, alg, data = scenarios.taylor_bar(h=5e-4)
    scenarios.apply_dirichlet(grid, data)
    mk = lambda **kw: descriptors(grid, solids, alg.tolerance, data["bodyforce"], data["dt"], **kw)
    do = oracle_lib.OracleContext(mk())
    d64 = MPMContext(mk(sort_interval=5))
    d32 = MPMContext(mk(sort_interval=5, precision="f32"))
    for c in (do, d64, d32):
        c.step(40)
    so = do.download_all()
    e64 = field_errors(d64.download_all(), so)
    assert max(e64.values()) <= FP64_TOL, sorted(e64.items(), key=lambda kv: -kv[1])[:4]
    e32 = field_errors(d32.download_all(), so, fields=("pos", "velocity", "stress", "F"))
    # stated FP32 bound for this case: 1e-3 relative per field (stress near the yield surface)
    assert max(e32.values()) <= 1e-3, e32


def test_save_load_roundtrip_with_sort():
    grid, solids, alg, data = scenarios.two_disks()
    scenarios.apply_dirichlet(grid, data)
    mk = lambda: descriptors(grid, solids, alg.tolerance, data["bodyforce"], data["dt"], sort_interval=3)
    a = MPMContext(mk())
    a.step(8)
    snap = a.save()
    a.step(11)
    b = MPMContext(mk())
    b.load(snap)
    b.step(11)
    for x, y in zip(a.download_all(), b.download_all()):
        assert rel_err(x.pos, y.pos) <= 1e-12 and rel_err(x.stress, y.stress) <= 1e-10


@pytest.mark.parametrize("friction", [0.0, 0.3])
def test_contact_two_disks_vs_oracle(friction, oracle_lib):
    """Multi-body contact (one velocity field per body, FEMP correction), 2D, 60 steps;
    the disks meet off-axis so the Coulomb branch sees tangential slip."""
    grid, solids, alg, data = scenarios.two_disks(speed=0.3, centers=((0.3, 0.3), (0.6, 0.68)))
    scenarios.apply_dirichlet(grid, data)
    mk = lambda: descriptors(grid, solids, alg.tolerance, data["bodyforce"], data["dt"], contact=True,
                             friction=friction)
    dg, do = MPMContext(mk()), oracle_lib.OracleContext(mk())
    for c in (dg, do):
        c.step(200)  # the disks meet after ~100 steps
    assert max(np.abs(s.strain).max() for s in do.download_all()) > 1e-4, "the disks must be in contact"
    errs = field_errors(dg.download_all(), do.download_all())
    # contact-mode bound: 1e-9 relative per field after 200 steps, ~100 of them in
    # contact at strains up to 0.6 (rounding differences grow with the deformation;
    # the single-field path keeps 1e-10 after 100 steps)
    assert max(errs.values()) <= 1e-9, sorted(errs.items(), key=lambda kv: -kv[1])[:4]
    m_g, *_ = dg.download_grid(grid.nodeCount)
    m_o, *_ = do.download_grid(grid.nodeCount)
    assert rel_err(m_g, m_o) <= 1e-9


def test_contact_sphere_plate_3d_vs_oracle(oracle_lib):
    """3D frictionless contact: an elastic sphere striking a neo-Hookean plate."""
    grid, solids, alg, data = scenarios.sphere_plate(h=1e-3, gap=0.0, speed=100.0)
    scenarios.apply_dirichlet(grid, data)
    mk = lambda: descriptors(grid, solids, alg.tolerance, data.get("bodyforce"), data["dt"], contact=True)
    dg, do = MPMContext(mk()), oracle_lib.OracleContext(mk())
    for c in (dg, do):
        c.step(60)
    assert np.abs(do.download_body(1).strain).max() > 1e-6, "the sphere must load the plate"
    errs = field_errors(dg.download_all(), do.download_all())
    assert max(errs.values()) <= FP64_TOL, sorted(errs.items(), key=lambda kv: -kv[1])[:4]


def _ensemble_problems(n, seed=0):
    # disks start with touching rims so every problem deforms within the test steps
    return [scenarios.ensemble_member(i, seed=seed, gap=0.0) for i in range(n)]


def test_batch_matches_single_contexts_and_oracle(oracle_lib):
    """Persistent batched launch == one context per problem (FP64, 60 steps),
    and problem 0 matches the oracle."""
    from jump_gb300.batch import Ensemble
    probs = _ensemble_problems(12)
    ens = Ensemble(probs, precision="f64")
    ens.step(60)
    assert all(s == 0 for s in ens.status())
    E = ens.energies()
    for i, (grid, solids, alg, data) in enumerate(probs):
        ctx = MPMContext(descriptors(grid, solids, alg.tolerance, data["bodyforce"], data["dt"]))
        ctx.step(60)
        errs = field_errors(ens.download(i), ctx.download_all())
        assert max(errs.values()) <= FP64_TOL, (i, sorted(errs.items(), key=lambda kv: -kv[1])[:3])
        ke, se, _ = ctx.energies()
        assert abs(E[i, 0] - ke) <= 1e-10 * ke and abs(E[i, 1] - se) <= 1e-9 * max(se, 1e-300)
        if i == 0:
            o = oracle_lib.OracleContext(descriptors(grid, solids, alg.tolerance, data["bodyforce"], data["dt"]))
            o.step(60)
            errs = field_errors(ens.download(0), o.download_all())
            assert max(errs.values()) <= FP64_TOL
        ctx.close()


def test_batch_tune_and_fp32():
    from jump_gb300.batch import Ensemble
    probs = _ensemble_problems(16, seed=3)
    e64 = Ensemble(probs, precision="f64")
    e32 = Ensemble(probs, precision="f32")
    res = e32.tune(probe_steps=3, use_cache=False)
    assert res["threads"] % 32 == 0 and res["ms_per_step"] > 0
    e64.step(40)
    e32.step(40)
    for i in range(len(probs)):
        errs = field_errors(e32.download(i), e64.download(i), fields=("pos", "velocity", "stress", "F"))
        assert max(errs.values()) <= 1e-4, (i, errs)  # stated FP32 bound for the ensemble
