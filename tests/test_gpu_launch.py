"""Launch configuration and its tuner: the P2G strategies (per-lane atomics,
warp sums over __match_any_sync groups, and both staged in shared-memory node
tiles, with the per-particle fallback of a CTA whose box exceeds the tile; and
for small problems every stage of every step in one cooperative launch), CTA sizes and
cell-sort intervals change only the
summation order of node sums, so every combination matches the oracle; the
sort can be switched on at run time; mpm_tune keeps the fastest combination
and leaves the simulation where it was."""
import numpy as np
import pytest

from cases import descriptors, field_errors
from jump_gb300 import _capi, scenarios
from jump_gb300.engine import MPMContext

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
TOUCH = ((0.3, 0.3), (0.3 + 0.4 / np.sqrt(2.0), 0.3 + 0.4 / np.sqrt(2.0)))


def worst(errs):
    return sorted(errs.items(), key=lambda kv: -kv[1])[:3]


def disks():
    prob = scenarios.two_disks(nodes=21, centers=TOUCH, speed=0.3, material="j2")
    scenarios.apply_dirichlet(prob[0], prob[3])
    return prob


def bar():
    prob = scenarios.taylor_bar(h=1e-3, radius=2e-3, length=6e-3, width=8e-3, height=10e-3, speed=300.0)
    scenarios.apply_dirichlet(prob[0], prob[3])
    return prob


def mk(prob, **kw):
    g, s, alg, data = prob
    return descriptors(g, s, alg.tolerance, data.get("bodyforce"), data["dt"], **kw)


@pytest.mark.parametrize("case", ["disks", "bar"])
@pytest.mark.parametrize("p2g,threads", [("atomic", 256), ("warp", 256), ("warp", 64), ("atomic", 128),
                                         ("tile", 256), ("tile", 64), ("tile_warp", 128), ("tile_warp", 32)])
def test_launch_settings_vs_oracle(case, p2g, threads, oracle_lib):
    prob = disks() if case == "disks" else bar()
    c, o = MPMContext(mk(prob)), oracle_lib.OracleContext(mk(prob))
    c.set_launch(p2g=p2g, threads=threads)
    assert c.launch() == {"p2g": p2g, "threads": threads, "sort_interval": 0}
    c.step(60)
    o.step(60)
    so = o.download_all()
    assert max(np.abs(b.strain).max() for b in so) > 1e-5
    errs = field_errors(c.download_all(), so)
    assert max(errs.values()) <= FP64_TOL, worst(errs)


def shuffled(prob, seed=5):
    """The same problem with every body's particles in a random order, so that a
    CTA's particles spread over the whole body (the tile strategies fall back to
    per-particle atomics until a cell sort gathers them)."""
    g, solids, alg, data = prob
    rng = np.random.default_rng(seed)
    for s in solids:
        n = s.parCount
        perm = rng.permutation(n)
        for obj in (s, s.mat):
            for k, v in vars(obj).items():
                if isinstance(v, np.ndarray) and v.ndim >= 1 and v.shape[0] == n:
                    setattr(obj, k, v[perm].copy())
    return prob


@pytest.mark.parametrize("p2g", ["tile", "tile_warp"])
@pytest.mark.parametrize("sort_interval", [0, 5])
@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_tiles_on_scattered_particles(p2g, sort_interval, precision, oracle_lib):
    prob = shuffled(bar())
    o = oracle_lib.OracleContext(mk(prob))
    o.step(40)
    so = o.download_all()
    assert max(np.abs(b.strain).max() for b in so) > 1e-5

    def err(strategy):
        c = MPMContext(mk(prob, precision=precision))
        c.set_launch(p2g=strategy, threads=256, sort_interval=sort_interval)
        c.step(40)
        fields = ("pos", "velocity", "stress", "F") if precision == "f32" else None
        return field_errors(c.download_all(), so, **({"fields": fields} if fields else {}))

    errs = err(p2g)
    if precision == "f64":
        assert max(errs.values()) <= FP64_TOL, worst(errs)
    else:
        # FP32 particles: no less accurate than per-lane atomics on the same case
        # (this bar at 300 m/s reaches ~2e-3 in stress near the yield surface)
        ref = max(err("atomic").values())
        assert max(errs.values()) <= 2 * ref, (worst(errs), ref)


def test_sort_switched_on_at_run_time(oracle_lib):
    prob = bar()
    c, o = MPMContext(mk(prob)), oracle_lib.OracleContext(mk(prob))
    c.step(10)
    c.set_launch(sort_interval=3, p2g="warp")
    c.step(40)
    c.set_launch(sort_interval=0)
    c.step(10)
    o.step(60)
    errs = field_errors(c.download_all(), o.download_all())
    assert max(errs.values()) <= FP64_TOL, worst(errs)


@pytest.mark.parametrize("p2g", ["warp", "tile", "tile_warp"])
def test_contact_with_warp_sums_and_tiles(p2g, oracle_lib):
    g, s, alg, data = scenarios.sphere_plate(h=1e-3, gap=0.0, speed=100.0)
    scenarios.apply_dirichlet(g, data)
    d = lambda: descriptors(g, s, alg.tolerance, data.get("bodyforce"), data["dt"], contact=True)
    c, o = MPMContext(d()), oracle_lib.OracleContext(d())
    c.set_launch(p2g=p2g, sort_interval=4)
    c.step(40)
    o.step(40)
    errs = field_errors(c.download_all(), o.download_all())
    assert max(errs.values()) <= 1e-9, worst(errs)


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_tune_keeps_the_state(precision):
    prob = bar()
    a, b = MPMContext(mk(prob, precision=precision)), MPMContext(mk(prob, precision=precision))
    a.step(10)
    before = a.download_all()
    res = a.tune(3)
    assert res["p2g"] in ("atomic", "warp", "tile", "tile_warp", "fused") and res["threads"] in (64, 128, 256)
    # the fused candidate where it applies (FP64 problems of at most 2048 particles)
    assert len(res["probes"]) == (49 if precision == "f64" else 48)
    assert res["sort_interval"] in (0, 1, 4, 16) and res["ms_per_step"] > 0
    errs = field_errors(a.download_all(), before)
    assert max(errs.values()) == 0.0, worst(errs)  # tuning does not advance the simulation
    a.step(20)
    b.step(30)
    errs = field_errors(a.download_all(), b.download_all(), fields=("pos", "velocity", "stress", "F"))
    assert max(errs.values()) <= (FP64_TOL if precision == "f64" else 1e-4), worst(errs)


def test_set_launch_rejects_bad_arguments():
    c = MPMContext(mk(disks()))
    before = c.launch()
    assert before == {"p2g": "fused", "threads": 64, "sort_interval": 0}  # 416 particles: the fused default
    L = _capi.lib()
    assert L.mpm_set_launch(c.h, 7, -1, -1) == _capi.MPM_ERR_ARG
    assert L.mpm_set_launch(c.h, -1, 100, -1) == _capi.MPM_ERR_ARG
    assert L.mpm_set_launch(c.h, -1, 512, -1) == _capi.MPM_ERR_ARG
    assert c.launch() == before


def test_fused_strategy_default_and_vs_oracle(oracle_lib):
    """A small FP64 problem defaults to the fused strategy (every stage of
    every step in one cooperative launch); it matches the oracle, and the per-stage
    launches on the same problem to summation order."""
    prob = disks()
    c, a, o = MPMContext(mk(prob)), MPMContext(mk(prob)), oracle_lib.OracleContext(mk(prob))
    assert c.launch()["p2g"] == "fused"
    a.set_launch(p2g="atomic")
    for ctx in (c, a, o):
        ctx.step(60)
    so = o.download_all()
    errs = field_errors(c.download_all(), so)
    assert max(errs.values()) <= FP64_TOL, worst(errs)
    errs = field_errors(c.download_all(), a.download_all())
    assert max(errs.values()) <= 1e-12, worst(errs)
    # the grid arrays after a fused step equal those after per-stage steps
    ng = prob[0].nodeCount
    for x, y in zip(c.download_grid(ng), a.download_grid(ng)):
        assert np.max(np.abs(x - y)) <= 1e-12 * max(np.max(np.abs(y)), 1e-300)


def test_fused_then_per_stage_steps(oracle_lib):
    """Steps alternating between the fused strategy and per-stage launches
    (the dense reset of the fused steps leaves the per-stage block list stale;
    the next per-stage step clears every node first) match the oracle."""
    prob = disks()
    c, o = MPMContext(mk(prob)), oracle_lib.OracleContext(mk(prob))
    for k, p2g in enumerate(("fused", "atomic", "fused", "warp", "fused", "tile")):
        c.set_launch(p2g=p2g)
        c.step(10 + k)
        o.step(10 + k)
    errs = field_errors(c.download_all(), o.download_all())
    assert max(errs.values()) <= FP64_TOL, worst(errs)


def test_fused_rules():
    """The fused strategy is refused where it does not apply; a sort
    switched on under it moves the context to per-stage launches."""
    f32 = MPMContext(mk(bar(), precision="f32"))  # FP32 particles: per-stage launches only
    assert f32.launch()["p2g"] != "fused"
    with pytest.raises(_capi.MPMError):
        f32.set_launch(p2g="fused")
    small = MPMContext(mk(disks()))
    small.set_launch(sort_interval=3)
    assert small.launch() == {"p2g": "atomic", "threads": small.launch()["threads"], "sort_interval": 3}
    with pytest.raises(_capi.MPMError):
        small.set_launch(p2g="fused")
    small.step(5)
