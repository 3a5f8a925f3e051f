"""EnergiesFix sums taken inside a multi-step call (mpm_step_energies) against
the same sums taken between single steps and against the oracle, and the
solver's hook schedule (counter % interval == 0) when no hook reads particle
arrays."""
import numpy as np
import pytest

from cases import descriptors, field_errors
from jump_gb300 import EmptyOutput, EnergiesFix, LinearBasis, scenarios, solve_explicit_dynamics_2D
from jump_gb300.engine import MPMContext
from jump_gb300.problem import step_times

pytestmark = pytest.mark.gpu


def disks():
    grid, solids, alg, data = scenarios.two_disks(nodes=21)
    scenarios.apply_dirichlet(grid, data)
    return grid, solids, alg, data


@pytest.mark.parametrize("every,first", [(1, 0), (3, 1), (5, 4)])
def test_step_energies_matches_step_then_energies(every, first):
    grid, solids, alg, data = disks()
    mk = lambda: descriptors(grid, solids, alg.tolerance, data["bodyforce"], data["dt"])
    a, b = MPMContext(mk()), MPMContext(mk())
    n = 25
    recs, t = a.step_energies(n, every, first, t=0.5)
    assert t == pytest.approx(0.5 + n * data["dt"], abs=1e-15)
    want = []
    for k in range(n):
        b.step(1)
        if k >= first and (k - first) % every == 0:
            ke, se, mom = b.energies()
            want.append([ke, se, *mom])
    want = np.array(want)
    assert recs.shape == want.shape == ((n - 1 - first) // every + 1, 4)
    assert np.max(np.abs(recs - want)) <= 1e-12 * np.max(np.abs(want))
    errs = field_errors(a.download_all(), b.download_all())
    assert max(errs.values()) <= 1e-12, errs


@pytest.mark.parametrize("precision,sort,threads", [("f64", 0, 128), ("f32", 3, 32), ("f64", 2, 256)])
def test_step_energies_taylor_bar_captured(precision, sort, threads):
    """The 3D J2 bar, whose recording steps run as one captured graph each (the
    step, then the EnergiesFix sums through the device record cursor): records
    of two calls (the second needs more record slots than the first) against
    mpm_energies after single steps, FP64 and FP32, with the cell sort
    switching buffers (two captured graphs) and at several CTA sizes."""
    grid, solids, alg, data = scenarios.taylor_bar(h=1e-3)
    scenarios.apply_dirichlet(grid, data)
    mk = lambda: descriptors(grid, solids, alg.tolerance, data.get("bodyforce"), data["dt"], precision=precision)
    a, b = MPMContext(mk()), MPMContext(mk())
    for c in (a, b):
        c.set_launch(threads=threads, sort_interval=sort)
    calls = [(7, 1, 0), (20, 2, 1)]
    got = [a.step_energies(n, e, f)[0] for n, e, f in calls]
    want = []
    for n, e, f in calls:
        w = []
        for k in range(n):
            b.step(1)
            if k >= f and (k - f) % e == 0:
                ke, se, mom = b.energies()
                w.append([ke, se, *mom])
        want.append(np.array(w))
    for g, w in zip(got, want):
        assert g.shape == w.shape
        scale = np.max(np.abs(w), axis=0)
        scale[2:] = scale[2:].max()  # momentum components against the momentum's size
        # FP32: two runs of the same FP32 problem differ at FP32's resolution
        # (summation order of the FP32 warp sums); FP64: at FP64's
        tol = 2e-6 if precision == "f32" else 1e-11
        assert np.all(np.abs(g - w) <= tol * scale), (g, w)
    a.close()
    b.close()


def test_step_energies_without_records():
    grid, solids, alg, data = disks()
    c = MPMContext(descriptors(grid, solids, alg.tolerance, data["bodyforce"], data["dt"]))
    recs, _ = c.step_energies(3, 2, 5)
    assert recs.shape == (0, 4)


@pytest.mark.parametrize("interval", [1, 7])
def test_solver_energies_fix_vs_oracle(interval, oracle_lib, tmp_path):
    grid, solids, alg, data = disks()
    data["total_time"] = 0.06
    o = oracle_lib.OracleContext(descriptors(grid, solids, alg.tolerance, data["bodyforce"], data["dt"]))
    times = step_times(data["time"], data["total_time"], data["dt"])
    want_t, want = [], []
    for c in range(len(times)):
        o.step(1)
        if c % interval == 0:
            ke, se, _ = o.energies()
            want_t.append(times[c])
            want.append((ke, se))
    fix = EnergiesFix(solids, str(tmp_path / "energies.txt"))
    solve_explicit_dynamics_2D(grid, solids, LinearBasis(), alg, EmptyOutput(interval), [fix], data)
    assert fix.recordTime == want_t
    got = np.array([fix.kinEnergy, fix.strEnergy]).T
    want = np.array(want)
    assert np.max(np.abs(got - want)) <= 1e-10 * np.max(np.abs(want))
    lines = open(tmp_path / "energies.txt").read().splitlines()
    assert len(lines) == len(want_t)
    assert float(lines[-1].split()[0]) == want_t[-1]
    for s, st in zip(solids, o.download_all()):
        assert np.max(np.abs(s.pos - st.pos)) <= 1e-12


def test_solver_dumps_and_fixes_vs_oracle(oracle_lib, tmp_path):
    """solve_explicit_dynamics_2D with OvitoOutput, DisplacementFix and EnergiesFix:
    the LAMMPS dump of every hook step (counter % 10 == 0) holds the oracle's
    particle state after that step, the displacement file the tracked
    particle's displacement, the energies file the sums of the downloaded state."""
    from jump_gb300 import DisplacementFix, OvitoOutput
    grid, solids, alg, data = disks()
    data["total_time"] = 0.025
    o = oracle_lib.OracleContext(descriptors(grid, solids, alg.tolerance, data["bodyforce"], data["dt"]))
    times = step_times(data["time"], data["total_time"], data["dt"])
    want = {}
    for c in range(len(times)):
        o.step(1)
        if c % 10 == 0:
            want[c] = o.download_all()
    track = solids[1].pos[5].copy()
    out = OvitoOutput(10, str(tmp_path) + "/", ["sigmaxx", "sigmayy", "vx", "vy"])
    disp = DisplacementFix(solids, track, str(tmp_path) + "/")
    en = EnergiesFix(solids, str(tmp_path / "energies.txt"))
    solve_explicit_dynamics_2D(grid, solids, LinearBasis(), alg, out, [disp, en], data)
    for c, st in want.items():
        rows = [r.split() for r in open(tmp_path / f"dump_p.{c}.LAMMPS").read().splitlines()[9:]]
        vals = np.array([[float(v) for v in r] for r in rows])
        x = np.concatenate([b.pos for b in st])
        v = np.concatenate([b.velocity for b in st])
        sxx = np.concatenate([b.stress.reshape(-1, 2, 2)[:, 0, 0] for b in st])
        assert vals.shape == (len(x), 9) and np.array_equal(vals[:, 0], np.arange(1, len(x) + 1))
        assert np.max(np.abs(vals[:, 2:4] - x)) <= 1e-10 * np.max(np.abs(x))
        assert np.max(np.abs(vals[:, 7:9] - v)) <= 1e-10 * np.max(np.abs(v))
        assert np.max(np.abs(vals[:, 5] - sxx)) <= 1e-10 * max(np.max(np.abs(sxx)), 1.0)  # noise before contact
    dlines = open(tmp_path / "recorded-position.txt").read().splitlines()
    assert [float(l.split()[0]) for l in dlines] == [times[c] for c in sorted(want)]
    last = np.array([float(t) for t in dlines[-1].split()[1:]])
    ref = want[max(want)][1].pos[5] - track
    assert np.max(np.abs(last - ref)) <= 1e-10 * max(np.max(np.abs(ref)), 1e-300)
    assert len(open(tmp_path / "energies.txt").read().splitlines()) == len(want)
