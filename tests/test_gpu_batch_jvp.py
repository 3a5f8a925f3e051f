"""Forward-mode derivatives of batched problems (mpm_batch_jvp): d(loss)/dE of
each problem against central finite differences of FP64 batch runs with every
problem's modulus perturbed at once (problems are independent, so one pair of
runs gives every problem's difference quotient).  Cases: the sphere-on-plate
impact ensemble (two velocity fields, frictionless contact; d(plate
deflection)/d(plate E)), two elastic disks (one modulus for both bodies),
and a neo-Hookean beam under gravity."""
import copy

import numpy as np
import pytest

from cases import field_errors
from jump_gb300 import scenarios
from jump_gb300.batch import Ensemble

pytestmark = pytest.mark.gpu

REL_STEP = 1e-6


def perturbed(probs, bodies, factor):
    out = []
    for g, s, alg, data in probs:
        s = copy.deepcopy(s)
        for k in bodies:
            s[k].mat.E *= factor
        out.append((g, s, alg, data))
    return out


def check_jvp(probs, bodies, steps, loss_w, tol):
    """loss_w(i, states) -> (loss, weights on x); returns the relative errors."""
    ens = Ensemble(probs)
    seeds = [[1.0 if k in bodies else 0.0 for k in range(len(p[1]))] for p in probs]
    # scale: derivative with respect to s = E / E0 (dE/ds = E0 of each problem)
    for i, p in enumerate(probs):
        seeds[i] = [p[1][k].mat.E if k in bodies else 0.0 for k in range(len(p[1]))]
    xd = ens.jvp(steps, seeds)
    states = [ens.download(i) for i in range(len(probs))]
    ref = Ensemble(probs)
    ref.step(steps)
    for i in range(len(probs)):
        errs = field_errors(states[i], ref.download(i))
        assert max(errs.values()) <= 1e-10, ("jvp must advance the state like step", i, errs)
    ep, em = Ensemble(perturbed(probs, bodies, 1 + REL_STEP)), Ensemble(perturbed(probs, bodies, 1 - REL_STEP))
    ep.step(steps)
    em.step(steps)
    rel = []
    for i in range(len(probs)):
        _, w = loss_w(i, states[i])
        ad = float(np.sum(w * xd[i]))
        lp, _ = loss_w(i, ep.download(i))
        lm, _ = loss_w(i, em.download(i))
        fd = (lp - lm) / (2 * REL_STEP)
        assert abs(fd) > 0, "the loss must depend on the modulus"
        rel.append(abs(ad - fd) / abs(fd))
    assert max(rel) <= tol, rel
    return rel


def test_jvp_impact_ensemble_plate_modulus():
    probs = [scenarios.impact_member(i, h=2e-3) for i in range(4)]
    for g, s, alg, data in probs:
        scenarios.apply_dirichlet(g, data)
    ns = probs[0][1][0].parCount

    def loss(i, st):
        # plate deflection: mean z of the plate particles
        z = st[1].pos[:, 2]
        w = np.zeros((ns + len(z), 3))
        w[ns:, 2] = 1.0 / len(z)
        return float(np.mean(z)), w

    check_jvp(probs, bodies=(1,), steps=60, loss_w=loss, tol=1e-5)


def test_jvp_two_disks_common_modulus():
    touch = ((0.3, 0.3), (0.3 + 0.4 / np.sqrt(2.0), 0.3 + 0.4 / np.sqrt(2.0)))
    probs = []
    for nodes, E in ((21, 1000.0), (31, 2500.0)):
        p = scenarios.two_disks(nodes=nodes, E=E, centers=touch)
        # one material object per disk so that each can be perturbed
        g, s, alg, data = p
        s[1].mat = copy.deepcopy(s[1].mat)
        scenarios.apply_dirichlet(g, data)
        probs.append(p)

    def loss(i, st):
        x = np.concatenate([b.pos for b in st])
        return float(np.sum(x[:, 0] ** 2)), np.stack([2 * x[:, 0], np.zeros(len(x))], axis=1)

    check_jvp(probs, bodies=(0, 1), steps=150, loss_w=loss, tol=1e-5)


def test_jvp_neohookean_beam_gravity():
    g, s, alg, data = scenarios.cantilever(h=0.125, ppc=2, length=1.0, depth=0.25)
    s[0].youngs = None
    scenarios.apply_dirichlet(g, data)
    probs = [(g, s, alg, data)]

    def loss(i, st):
        y = st[0].pos[:, 1]
        w = np.zeros((len(y), 2))
        w[:, 1] = 1.0 / len(y)
        return float(np.mean(y)), w

    check_jvp(probs, bodies=(0,), steps=300, loss_w=loss, tol=1e-5)
