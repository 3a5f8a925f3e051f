"""Launch configuration and its tuner: the P2G strategies (per-lane atomics,
warp-segmented sums, and both staged in shared-memory node tiles, with the
per-particle fallback of a CTA whose box exceeds the tile), CTA sizes and
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
    assert res["p2g"] in ("atomic", "warp", "tile", "tile_warp") and res["threads"] in (64, 128, 256)
    assert len(res["probes"]) == 48
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
    assert before == {"p2g": "atomic", "threads": 64, "sort_interval": 0}  # 416 particles: small CTAs
    L = _capi.lib()
    assert L.mpm_set_launch(c.h, 7, -1, -1) == _capi.MPM_ERR_ARG
    assert L.mpm_set_launch(c.h, -1, 100, -1) == _capi.MPM_ERR_ARG
    assert L.mpm_set_launch(c.h, -1, 512, -1) == _capi.MPM_ERR_ARG
    assert c.launch() == before
