"""Reverse mode: gradients of a loss on the final positions with respect to
per-particle Young's modulus and initial velocity, from the adjoint kernels on
the GPU, against

* forward-mode dual numbers through the templated restatement of the step
  (oracle/mpm_dual.cpp) for neo-Hookean, linear elastic and J2 bodies in 2D and
  3D (bound 1e-8, norm-relative), and
* central finite differences of the deterministic CPU oracle on a 2D
  neo-Hookean cantilever and a 3D neo-Hookean block (400 steps, long enough
  for the clamp to be felt at the tip);

and the inverse problems the gradients serve: recovering a stiffness field and
an initial velocity field from final positions."""
import copy

import numpy as np
import pytest

from jump_gb300 import scenarios
from jump_gb300.adjoint import final_positions, make_context, rollout_grad
from jump_gb300.engine import Descriptors

pytestmark = pytest.mark.gpu

NSTEPS, EVERY = 400, 50


def oracle_final(oracle_lib, problem, E, v0):
    grid, solids, alg, data = problem
    solids = copy.deepcopy(solids)
    off = 0
    for s in solids:
        n = s.parCount
        s.youngs = np.asarray(E[off:off + n], dtype=np.float64).copy()
        s.velocity = np.asarray(v0[off:off + n]).reshape(n, s.dim).copy()
        off += n
    o = oracle_lib.OracleContext(Descriptors(grid, solids, tolerance=alg.tolerance,
                                             body_force=data.get("bodyforce"), dt=data["dt"]))
    o.step(NSTEPS)
    x = np.concatenate([st.pos for st in o.download_all()])
    o.close()
    return x


def setup_case(dim):
    if dim == 2:
        problem = scenarios.cantilever(h=0.0625, ppc=2, length=1.0, depth=0.25)
    else:
        problem = scenarios.block_3d()
    grid, solids, alg, data = problem
    scenarios.apply_dirichlet(grid, data)
    E = np.concatenate([s.youngs for s in solids])
    v0 = np.concatenate([s.velocity for s in solids])
    x_all = np.concatenate([s.pos for s in solids])
    tip = x_all[:, 0] > np.quantile(x_all[:, 0], 0.9)
    return problem, E, v0, tip


@pytest.mark.parametrize("dim", [2, 3])
def test_adjoint_matches_finite_differences(dim, oracle_lib):
    problem, E, v0, tip = setup_case(dim)
    rng = np.random.default_rng(7)
    # target: the tip of a stiffer beam, so the loss and its gradient are non-zero
    target = oracle_final(oracle_lib, problem, 1.3 * E, v0)[tip]

    def loss(x):
        return float(np.sum((x[tip] - target) ** 2))

    def loss_grad(x):
        g = np.zeros_like(x)
        g[tip] = 2.0 * (x[tip] - target)
        return g

    x_gpu, g = rollout_grad(problem, E, v0, NSTEPS, EVERY, loss_grad)
    x_cpu = oracle_final(oracle_lib, problem, E, v0)
    assert np.max(np.abs(x_gpu - x_cpu)) <= 1e-10 * np.max(np.abs(x_cpu))

    # dL/dE on random particles (central differences, relative step 1e-4)
    ids = rng.choice(len(E), 16, replace=False)
    fd = []
    for p in ids:
        h = 1e-4 * E[p]
        Ep, Em = E.copy(), E.copy()
        Ep[p] += h
        Em[p] -= h
        fd.append((loss(oracle_final(oracle_lib, problem, Ep, v0)) -
                   loss(oracle_final(oracle_lib, problem, Em, v0))) / (2 * h))
    fd = np.array(fd)
    ad = g["E"][ids]
    assert np.linalg.norm(ad - fd) <= 1e-5 * np.linalg.norm(fd), (ad, fd)

    # dL/dv0 on random (particle, component) pairs
    pairs = [(int(rng.integers(len(E))), int(rng.integers(dim))) for _ in range(8)]
    fd_v, ad_v = [], []
    for p, a in pairs:
        h = 1e-5
        vp, vm = v0.copy(), v0.copy()
        vp[p, a] += h
        vm[p, a] -= h
        fd_v.append((loss(oracle_final(oracle_lib, problem, E, vp)) -
                     loss(oracle_final(oracle_lib, problem, E, vm))) / (2 * h))
        ad_v.append(g["v0"][p, a])
    fd_v, ad_v = np.array(fd_v), np.array(ad_v)
    assert np.linalg.norm(ad_v - fd_v) <= 1e-5 * np.linalg.norm(fd_v), (ad_v, fd_v)


def _desc_for(problem, E, v0):
    grid, solids, alg, data = problem
    solids = copy.deepcopy(solids)
    off = 0
    for s in solids:
        n = s.parCount
        s.youngs = np.asarray(E[off:off + n], dtype=np.float64).copy()
        s.velocity = np.asarray(v0[off:off + n]).reshape(n, s.dim).copy()
        off += n
    scenarios.apply_dirichlet(grid, data)
    return Descriptors(grid, solids, tolerance=alg.tolerance, body_force=data.get("bodyforce"), dt=data["dt"])


DUAL_CASES = {
    # name: (problem, steps, checkpoint interval)
    "cantilever_nh_2d": (lambda: scenarios.cantilever(h=0.0625, ppc=2, length=1.0, depth=0.25), 400, 50),
    "disks_elastic_2d": (lambda: scenarios.two_disks(centers=((0.3, 0.3), (0.585, 0.585))), 150, 25),
    "disks_j2_2d": (lambda: scenarios.two_disks(material="j2", centers=((0.3, 0.3), (0.585, 0.585))), 150, 25),
    "block_nh_3d": (lambda: scenarios.block_3d(), 200, 50),
    "taylor_j2_3d": (lambda: scenarios.taylor_bar(h=1e-3), 30, 10),
}


@pytest.mark.parametrize("name", sorted(DUAL_CASES))
def test_adjoint_matches_dual_numbers(name, oracle_lib):
    """dL/dE and dL/dv0 of L = xbar . x_final: the GPU adjoint against forward-mode
    dual numbers through the restatement, on the same seeded inputs."""
    make, nsteps, every = DUAL_CASES[name]
    problem = make()
    scenarios.apply_dirichlet(problem[0], problem[3])
    solids = problem[1]
    rng = np.random.default_rng(3)
    E = np.concatenate([np.full(s.parCount, s.mat.E) if getattr(s, "youngs", None) is None else s.youngs
                        for s in solids])
    E = E * np.exp(rng.uniform(-0.2, 0.2, len(E)))  # per-particle moduli
    v0 = np.concatenate([s.velocity for s in solids])
    n, d = v0.shape
    xbar = rng.normal(size=(n, d))
    ctx = make_context(problem, E, v0)
    ctx.fwd_checkpointed(nsteps, every)
    g = ctx.bwd(xbar)
    ctx.close()
    o = oracle_lib.OracleContext(_desc_for(problem, E, v0))
    o.step(nsteps)
    st = o.download_all()
    o.close()
    if name.startswith(("disks_j2", "taylor_j2")):
        assert max(float(np.max(s.alpha)) for s in st) > 0, "the J2 case must yield"
    # half the checked particles among the most strained (where E matters), half at random
    strain = np.concatenate([np.abs(s.strain.reshape(s.n, -1)).max(axis=1) for s in st])
    ids = np.unique(np.concatenate([np.argsort(strain)[-8:], rng.choice(n, 8, replace=False)]))
    dual = oracle_lib.dual_gradient(_desc_for(problem, E, v0), nsteps, "E", ids, xbar)
    ad = g["E"][ids]
    assert np.linalg.norm(ad - dual) <= 1e-8 * np.linalg.norm(dual), (ad, dual)
    vid = rng.choice(n * d, 16, replace=False)
    dual_v = oracle_lib.dual_gradient(_desc_for(problem, E, v0), nsteps, "v0", vid, xbar)
    ad_v = g["v0"].ravel()[vid]
    assert np.linalg.norm(ad_v - dual_v) <= 1e-8 * np.linalg.norm(dual_v), (ad_v, dual_v)


def test_checkpointed_forward_is_the_forward():
    problem, E, v0, tip = setup_case(2)
    a = make_context(problem, E, v0)
    a.fwd_checkpointed(NSTEPS, EVERY)
    b = make_context(problem, E, v0)
    b.step(NSTEPS)
    xa, xb = final_positions(a), final_positions(b)
    assert np.max(np.abs(xa - xb)) <= 1e-12 * np.max(np.abs(xb))
    a.bwd(np.ones_like(xa))
    assert np.max(np.abs(final_positions(a) - xa)) == 0.0  # context left at the final state


def _segments_case():
    problem, _, v0, _ = setup_case(2)
    x0 = np.concatenate([s.pos for s in problem[1]])
    xs = x0[:, 0] / x0[:, 0].max()
    return problem, v0, xs


def test_inverse_problem_recovers_stiffness_segments():
    """Recover the Young's moduli of four segments of the cantilever (the
    particles' E piecewise constant along x) from the final positions of all
    particles: L-BFGS on the log moduli, each gradient the sum of the adjoint's
    per-particle dL/dE over a segment.  From a uniform start 30-60% off, every
    segment's modulus comes back within the stated tolerance."""
    opt = pytest.importorskip("scipy.optimize")
    problem, v0, xs = _segments_case()
    nseg = 4
    seg = np.minimum((xs * nseg).astype(int), nseg - 1)
    E_true_seg = 1e6 * np.array([1.6, 0.7, 1.3, 0.9])
    ctx = make_context(problem, E_true_seg[seg], v0)
    ctx.step(NSTEPS)
    target = final_positions(ctx)
    ctx.close()
    scale = 1e6

    def f(a):
        E = np.exp(a)[seg]
        x, g = rollout_grad(problem, E, v0, NSTEPS, EVERY, lambda x: 2.0 * (x - target))
        L = float(np.sum((x - target) ** 2))
        ga = np.array([np.sum(g["E"][seg == k] * E[seg == k]) for k in range(nseg)])
        return L * scale, ga * scale

    a0 = np.full(nseg, np.log(1e6))
    L0 = f(a0)[0]
    res = opt.minimize(f, a0, jac=True, method="L-BFGS-B", options={"maxiter": 60, "ftol": 1e-16, "gtol": 1e-14})
    err = np.abs(np.exp(res.x) / E_true_seg - 1)
    print("\nstiffness segments", np.exp(res.x) / E_true_seg, "misfit", L0, "->", res.fun, "iterations", res.nit)
    assert res.fun <= 1e-6 * L0, (L0, res.fun)
    assert np.max(err) <= 0.01, err


def test_inverse_problem_per_particle_stiffness_error_falls():
    """Per-particle Young's modulus (a smooth field along x) from the final
    positions of all particles, by scaled gradient steps on log E with a
    backtracking step length: the misfit falls 100x and the RMS error of log E
    falls by a quarter (the field is only partly identifiable: particles near
    the free end carry little stress)."""
    problem, v0, xs = _segments_case()
    E_true = 1e6 * np.exp(0.4 * np.sin(2 * np.pi * xs))
    ctx = make_context(problem, E_true, v0)
    ctx.step(NSTEPS)
    target = final_positions(ctx)
    ctx.close()

    def misfit(E):
        c = make_context(problem, E, v0)
        c.step(NSTEPS)
        x = final_positions(c)
        c.close()
        return float(np.sum((x - target) ** 2))

    la = np.full(len(xs), np.log(1e6))
    err0 = float(np.sqrt(np.mean((la - np.log(E_true)) ** 2)))
    t, losses = None, []
    for _ in range(30):
        E = np.exp(la)
        x, g = rollout_grad(problem, E, v0, NSTEPS, EVERY, lambda x: 2.0 * (x - target))
        L0 = float(np.sum((x - target) ** 2))
        losses.append(L0)
        gl = g["E"] * E  # dL/d log E
        if t is None:
            t = 0.1 / np.max(np.abs(gl))
        for _ in range(30):
            if misfit(np.exp(la - t * gl)) < L0:
                break
            t *= 0.5
        la = la - t * gl
        t *= 2.0
    err1 = float(np.sqrt(np.mean((la - np.log(E_true)) ** 2)))
    print("\nper-particle log-E error", err0, "->", err1, "misfit", losses[0], "->", losses[-1])
    assert losses[-1] < 0.01 * losses[0], losses
    assert err1 < 0.75 * err0, (err0, err1)


def test_store_every_step_matches_checkpointing():
    """checkpoint_every = 1 (every state and node buffer kept, no recompute)
    gives the gradients of the checkpointed sweep."""
    problem, E, v0, tip = setup_case(2)
    x_a, ga = rollout_grad(problem, E, v0, NSTEPS, EVERY, lambda x: np.where(tip[:, None], x, 0.0))
    x_b, gb = rollout_grad(problem, E, v0, NSTEPS, 1, lambda x: np.where(tip[:, None], x, 0.0))
    assert np.max(np.abs(x_a - x_b)) <= 1e-12 * np.max(np.abs(x_a))
    for k in ("E", "v0"):
        assert np.max(np.abs(ga[k] - gb[k])) <= 1e-9 * np.max(np.abs(ga[k])), k


def test_inverse_problem_recovers_initial_velocity():
    """Recover a smooth initial velocity field of the cantilever from the final
    positions of all its particles: adjoint gradient steps from rest, with a
    backtracking step length (each trial one GPU forward rollout), cut the
    misfit by 100x and the velocity error by 3x."""
    problem, E, v_rest, tip = setup_case(2)
    x0 = np.concatenate([s.pos for s in problem[1]])
    v_true = np.zeros_like(v_rest)
    v_true[:, 1] = 0.05 * np.sin(0.5 * np.pi * x0[:, 0] / x0[:, 0].max())
    ctx = make_context(problem, E, v_true)
    ctx.step(NSTEPS)
    target = final_positions(ctx)
    ctx.close()

    def misfit(v):
        c = make_context(problem, E, v)
        c.step(NSTEPS)
        x = final_positions(c)
        c.close()
        return float(np.sum((x - target) ** 2))

    v = np.zeros_like(v_true)
    t = None
    losses = []
    for _ in range(8):
        x, g = rollout_grad(problem, E, v, NSTEPS, EVERY, lambda x: 2.0 * (x - target))
        L0 = float(np.sum((x - target) ** 2))
        losses.append(L0)
        gv = np.asarray(g["v0"]).reshape(v.shape)
        if t is None:
            t = 0.01 / np.max(np.abs(gv))  # first trial: a 1 cm/s change where the gradient is largest
        for _ in range(20):  # backtracking: halve until the misfit drops
            if misfit(v - t * gv) < L0:
                break
            t *= 0.5
        v = v - t * gv
        t *= 2.0
    losses.append(misfit(v))
    err0, err1 = np.linalg.norm(v_true), np.linalg.norm(v - v_true)
    assert losses[-1] < 0.01 * losses[0], losses
    assert err1 < err0 / 3.0, (err1, err0)


def test_adjoint_full_size_cantilever_32_parameters():
    """The differentiable-solve configuration at its full size: the neo-Hookean
    cantilever of 16,384 particles with per-particle E, 2000 steps, checkpoints
    every 50.  dL/dE of the squared tip-displacement error on 32 random
    particles against central differences (relative step 1e-4) of GPU forward
    runs, to 1e-5 norm-relative.  The loss difference is formed from the
    position difference, sum((x+ - x-)(x+ + x- - 2 t)) over the tip, so that two
    nearly equal losses are never subtracted."""
    problem = scenarios.cantilever()
    grid, solids, alg, data = problem
    scenarios.apply_dirichlet(grid, data)
    E = np.concatenate([s.youngs for s in solids])
    v0 = np.concatenate([s.velocity for s in solids])
    assert len(E) == 16384
    nsteps, every = 2000, 50
    x0 = np.concatenate([s.pos for s in solids])
    tip = x0[:, 0] > np.quantile(x0[:, 0], 0.95)
    c = make_context(problem, 1.3 * E, v0)
    c.step(nsteps)
    target = final_positions(c)[tip]
    c.close()

    def loss_grad(x):
        g = np.zeros_like(x)
        g[tip] = 2.0 * (x[tip] - target)
        return g

    x, g = rollout_grad(problem, E, v0, nsteps, every, loss_grad)

    def run(Ep):
        cc = make_context(problem, Ep, v0)
        cc.step(nsteps)
        xx = final_positions(cc)[tip]
        cc.close()
        return xx

    rng = np.random.default_rng(11)
    ids = rng.choice(len(E), 32, replace=False)
    fd = []
    for p in ids:
        h = 1e-4 * E[p]
        Ep, Em = E.copy(), E.copy()
        Ep[p] += h
        Em[p] -= h
        xp, xm = run(Ep), run(Em)
        fd.append(float(np.sum((xp - xm) * (xp + xm - 2.0 * target))) / (2 * h))
    fd = np.array(fd)
    ad = g["E"][ids]
    err = np.linalg.norm(ad - fd) / np.linalg.norm(fd)
    print("\nfull-size cantilever dL/dE vs central differences (32 parameters):", err)
    assert err <= 1e-5, (err, ad, fd)


@pytest.mark.parametrize("name", ["disks_j2_2d", "block_nh_3d", "taylor_j2_3d"])
def test_tiled_adjoint_scatter_matches_per_particle(name):
    """A context whose P2G strategy is a tile one scatters the G2P adjoint's node
    adjoints through a shared-memory node tile; its gradients equal those of the
    per-particle scatter up to summation order (the forward and its recomputes
    use the tile P2G too, so the bound is that of two summation orders)."""
    make, nsteps, every = DUAL_CASES[name]
    problem = make()
    grid, solids, alg, data = problem
    scenarios.apply_dirichlet(grid, data)
    E = np.concatenate([s.youngs if getattr(s, "youngs", None) is not None else np.full(s.parCount, s.mat.E)
                        for s in solids])
    v0 = np.concatenate([s.velocity for s in solids])
    xbar = np.random.default_rng(5).normal(size=v0.shape)
    grads = {}
    for strategy in ("atomic", "tile"):
        c = make_context(problem, E, v0)
        c.set_launch(p2g=strategy)
        c.fwd_checkpointed(nsteps, every)
        grads[strategy] = c.bwd(xbar)
        c.close()
    for k in ("E", "v0", "x0"):
        a, b = grads["atomic"][k], grads["tile"][k]
        assert np.max(np.abs(a - b)) <= 1e-9 * np.max(np.abs(a)), k
