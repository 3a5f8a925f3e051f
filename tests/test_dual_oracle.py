"""The dual-number gradient oracle (oracle/mpm_dual.cpp) on the CPU.

Its restatement of the USL step, templated on the scalar type, run with plain
doubles reproduces the main oracle bit for bit (so the two restatements cannot
disagree about the step), and its forward-mode derivatives agree with central
differences of the main oracle to the differences' own accuracy.  The GPU
adjoint is checked against it in tests/test_gpu_adjoint.py."""
import copy

import numpy as np
import pytest

from jump_gb300 import scenarios
from jump_gb300.engine import Descriptors


def _desc(problem, E=None, v0=None):
    grid, solids, alg, data = problem
    solids = copy.deepcopy(solids)
    off = 0
    for s in solids:
        n = s.parCount
        if E is not None:
            s.youngs = np.asarray(E[off:off + n], dtype=np.float64).copy()
        if v0 is not None:
            s.velocity = np.asarray(v0[off:off + n], dtype=np.float64).reshape(n, s.dim).copy()
        off += n
    scenarios.apply_dirichlet(grid, data)
    return Descriptors(grid, solids, tolerance=alg.tolerance, body_force=data.get("bodyforce"), dt=data["dt"])


def _params(problem):
    solids = problem[1]
    E = np.concatenate([s.youngs if getattr(s, "youngs", None) is not None else np.full(s.parCount, s.mat.E)
                        for s in solids])
    v0 = np.concatenate([s.velocity for s in solids])
    return E, v0


CASES = {
    "cantilever_nh_gravity": (lambda: scenarios.cantilever(h=0.25), 400),
    "two_disks_elastic": (lambda: scenarios.two_disks(), 60),
    "two_disks_j2": (lambda: scenarios.two_disks(material="j2"), 40),
    "block_3d_nh": (lambda: scenarios.block_3d(h=0.125), 200),
    "taylor_bar_3d_j2": (lambda: scenarios.taylor_bar(h=1e-3), 30),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_dual_restatement_matches_oracle_bit_for_bit(name, oracle_lib):
    make, steps = CASES[name]
    prob = make()
    E, v0 = _params(prob)
    o = oracle_lib.OracleContext(_desc(prob, E, v0), threads=1)
    o.step(steps)
    so = o.download_all()
    o.close()
    pos, sig = oracle_lib.dual_values(_desc(prob, E, v0), steps)
    assert np.array_equal(np.concatenate([s.pos for s in so]), pos)
    assert np.array_equal(np.concatenate([s.stress for s in so]), sig)


def _loss_fd(oracle_lib, prob, E, v0, steps, xbar, kind, q, h):
    vals = []
    for sg in (1.0, -1.0):
        if kind == "E":
            Ep, vp = E.copy(), v0
            Ep[q] *= 1 + sg * h
        else:
            Ep, vp = E, v0.copy().ravel()
            vp[q] += sg * h
            vp = vp.reshape(v0.shape)
        o = oracle_lib.OracleContext(_desc(prob, Ep, vp), threads=1)
        o.step(steps)
        vals.append(float(np.sum(np.concatenate([s.pos for s in o.download_all()]) * xbar)))
        o.close()
    return (vals[0] - vals[1]) / (2 * h * (E[q] if kind == "E" else 1.0))


@pytest.mark.parametrize("name", ["cantilever_nh_gravity", "two_disks_j2", "block_3d_nh"])
def test_dual_gradient_vs_central_differences(name, oracle_lib):
    make, steps = CASES[name]
    prob = make()
    E, v0 = _params(prob)
    n, d = v0.shape
    rng = np.random.default_rng(1)
    xbar = rng.normal(size=(n, d))
    ids = rng.choice(n, 8, replace=False)
    g = oracle_lib.dual_gradient(_desc(prob, E, v0), steps, "E", ids, xbar)
    fd = np.array([_loss_fd(oracle_lib, prob, E, v0, steps, xbar, "E", int(q), 1e-4) for q in ids])
    # central differences with a 1e-4 relative step carry ~1e-5 of their own error
    assert np.max(np.abs(g - fd)) <= 2e-4 * np.max(np.abs(fd)), (g, fd)
    vid = rng.choice(n * d, 8, replace=False)
    gv = oracle_lib.dual_gradient(_desc(prob, E, v0), steps, "v0", vid, xbar)
    fdv = np.array([_loss_fd(oracle_lib, prob, E, v0, steps, xbar, "v0", int(q), 1e-6) for q in vid])
    assert np.max(np.abs(gv - fdv)) <= 2e-4 * np.max(np.abs(fdv)), (gv, fdv)
