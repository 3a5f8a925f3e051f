"""The WIDE batch strategy (one launch per stage for all problems): contact
problems of the seeded sphere-on-plate impact ensemble against one contact
context per problem and against the oracle; the two-disk ensemble under both
strategies; problems mixing material models; strategy switches mid-run; the
autotuner leaving the state untouched; the FP32 variant's stated bound."""
import numpy as np
import pytest

from cases import descriptors, field_errors
from jump_gb300 import _capi, scenarios
from jump_gb300.batch import Ensemble
from jump_gb300.engine import MPMContext

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
CONTACT_TOL = 1e-9   # as the single-context contact parity bound


def impact_problems(n, h=2e-3, seed=0):
    probs = [scenarios.impact_member(i, seed=seed, h=h) for i in range(n)]
    for g, s, alg, data in probs:
        scenarios.apply_dirichlet(g, data)
    return probs


def single(problem, steps, precision="f64"):
    grid, solids, alg, data = problem
    ctx = MPMContext(descriptors(grid, solids, alg.tolerance, data.get("bodyforce"), data["dt"],
                                 precision=precision, contact=bool(data.get("contact")),
                                 friction=float(data.get("friction", 0.0))))
    ctx.step(steps)
    return ctx


def worst(errs):
    return sorted(errs.items(), key=lambda kv: -kv[1])[:3]


def test_contact_batch_matches_single_contexts_and_oracle(oracle_lib):
    probs = impact_problems(5)
    ens = Ensemble(probs, precision="f64")
    assert ens.strategy == "wide"
    with pytest.raises(_capi.MPMError, match="persistent"):
        ens.set_strategy("persistent")
    ens.step(40)
    assert all(s == 0 for s in ens.status())
    E = ens.energies()
    for i, p in enumerate(probs):
        ctx = single(p, 40)
        st = ens.download(i)
        assert np.abs(st[1].strain).max() > 1e-7, "the sphere must load the plate"
        errs = field_errors(st, ctx.download_all())
        assert max(errs.values()) <= CONTACT_TOL, (i, worst(errs))
        ke, se, _ = ctx.energies()
        assert abs(E[i, 0] - ke) <= 1e-9 * ke and abs(E[i, 1] - se) <= 1e-8 * max(se, 1e-300)
        ctx.close()
    grid, solids, alg, data = probs[2]
    o = oracle_lib.OracleContext(descriptors(grid, solids, alg.tolerance, data.get("bodyforce"), data["dt"],
                                             contact=True))
    o.step(40)
    errs = field_errors(ens.download(2), o.download_all())
    assert max(errs.values()) <= CONTACT_TOL, worst(errs)
    ens.close()


def test_wide_equals_persistent_on_two_disk_ensemble():
    probs = [scenarios.ensemble_member(i, gap=0.0) for i in range(10)]
    a, b = Ensemble(probs), Ensemble(probs)
    assert a.strategy == "persistent"
    b.set_strategy("wide")
    a.step(50)
    b.step(50)
    for i in range(len(probs)):
        errs = field_errors(b.download(i), a.download(i))
        assert max(errs.values()) <= FP64_TOL, (i, worst(errs))


def test_strategy_switches_mid_run():
    """persistent -> wide -> persistent: the wide step must drop the node data
    the persistent kernel left behind."""
    probs = [scenarios.ensemble_member(i, gap=0.0) for i in range(6)]
    ens = Ensemble(probs)
    for strat in ("persistent", "wide", "persistent", "wide"):
        ens.set_strategy(strat)
        ens.step(15)
    for i, p in enumerate(probs):
        ctx = single(p, 60)
        errs = field_errors(ens.download(i), ctx.download_all())
        assert max(errs.values()) <= FP64_TOL, (i, worst(errs))
        ctx.close()


def test_mixed_materials_run_wide():
    # disks of radius 0.2 with touching rims, so both bodies of every problem
    # are strained within the test steps (fields at rounding level would make
    # the relative comparison meaningless)
    touch = ((0.3, 0.3), (0.3 + 0.4 / np.sqrt(2.0), 0.3 + 0.4 / np.sqrt(2.0)))
    p_el = scenarios.two_disks(nodes=21, centers=touch)
    p_nh = scenarios.two_disks(nodes=31, material="neohookean", centers=touch)
    p_j2 = scenarios.two_disks(nodes=26, material="j2", centers=touch)
    probs = [p_el, p_nh, p_j2]
    for g, s, alg, data in probs:
        scenarios.apply_dirichlet(g, data)
    ens = Ensemble(probs)
    assert ens.strategy == "wide"
    ens.step(80)
    for i, p in enumerate(probs):
        ctx = single(p, 80)
        st = ens.download(i)
        assert min(np.abs(b.strain).max() for b in st) > 1e-6, "both disks must be strained"
        errs = field_errors(st, ctx.download_all())
        assert max(errs.values()) <= FP64_TOL, (i, worst(errs))
        ctx.close()


def test_tune_keeps_state_and_picks_a_strategy():
    probs = impact_problems(3)
    a, b = Ensemble(probs), Ensemble(probs)
    res = a.tune(probe_steps=4, use_cache=False)
    assert res["strategy"] == "wide" and res["ms_per_step"] > 0
    a.step(20)
    b.step(20)
    for i in range(len(probs)):
        errs = field_errors(a.download(i), b.download(i))
        assert max(errs.values()) <= CONTACT_TOL, (i, worst(errs))
    small = [scenarios.ensemble_member(i, gap=0.0) for i in range(8)]
    c = Ensemble(small)
    res = c.tune(probe_steps=4, use_cache=False)
    assert res["strategy"] in ("persistent", "wide")
    c.step(10)
    ref = Ensemble(small)
    ref.step(10)
    for i in range(len(small)):
        errs = field_errors(c.download(i), ref.download(i))
        assert max(errs.values()) <= FP64_TOL, (i, worst(errs))


def test_contact_batch_fp32_bound(oracle_lib):
    probs = impact_problems(3, seed=5)
    e32 = Ensemble(probs, precision="f32")
    e64 = Ensemble(probs, precision="f64")
    e32.step(40)
    e64.step(40)
    for i in range(len(probs)):
        errs = field_errors(e32.download(i), e64.download(i), fields=("pos", "velocity", "stress", "F"))
        assert max(errs.values()) <= 1e-3, (i, worst(errs))  # stated FP32 bound, impact ensemble
