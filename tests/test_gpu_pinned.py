"""Page-locked host arrays (asynchronous copies, no per-field synchronisation)
give the results of pageable arrays, bit for bit, including the symmetry
check of the inputs and the J2 von Mises download."""
import copy

import numpy as np
import pytest

from cases import descriptors
from jump_gb300 import _capi, scenarios
from jump_gb300.engine import BodyState, MPMContext

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

SOLID = ("pos", "velocity", "mass", "volume", "volumeInitial", "deformationGradient", "strain", "stress")


def pinned_like(a):
    t = torch.empty_strided(a.shape, tuple(x // a.itemsize for x in a.strides), dtype=torch.float64,
                            pin_memory=True)
    out = t.numpy()
    np.copyto(out, a)
    return out


def pin(solids):
    solids = copy.deepcopy(solids)
    for s in solids:
        for k in SOLID:
            setattr(s, k, pinned_like(getattr(s, k)))
        for k in ("alpha", "pstrain_3D", "vmStr"):
            if getattr(s.mat, k, None) is not None:
                setattr(s.mat, k, pinned_like(getattr(s.mat, k)))
    return solids


def pinned_state(n, d):
    st = BodyState(n, d)
    for k in st.FIELDS:
        setattr(st, k, pinned_like(getattr(st, k)))
    return st


def bar():
    g, s, alg, data = scenarios.taylor_bar(h=1e-3, radius=2e-3, length=6e-3, width=8e-3, height=10e-3, speed=300.0)
    scenarios.apply_dirichlet(g, data)
    return g, s, alg, data


def test_pinned_upload_and_download_match_pageable():
    g, s, alg, data = bar()
    mk = lambda sols: descriptors(g, sols, alg.tolerance, data.get("bodyforce"), data["dt"])
    sp = pin(s)
    assert _capi.lib() is not None
    a, b = MPMContext(mk(s)), MPMContext(mk(sp))
    for steps in (0, 20):
        a.step(steps)
        b.step(steps)
        pa = a.download_all()  # pageable destination
        pa2 = a.download_all([pinned_state(x.parCount, 3) for x in s])  # page-locked destination
        pb = b.download_all()
        for x, y, z in zip(pa, pa2, pb):
            for k in BodyState.FIELDS:
                np.testing.assert_array_equal(getattr(x, k), getattr(y, k), err_msg=k)
                if steps == 0:  # the same input through both upload paths
                    np.testing.assert_array_equal(getattr(x, k), getattr(z, k), err_msg=k)
                else:
                    ref = np.max(np.abs(getattr(x, k))) or 1.0
                    assert np.max(np.abs(getattr(x, k) - getattr(z, k))) <= 1e-10 * ref, k
    assert pa[0].alpha.max() > 0 and pa[0].vmstr.max() > 0


def test_pinned_asymmetric_stress_rejected():
    g, s, alg, data = bar()
    sp = pin(s)
    sp[0].stress[0, 0, 1] = 1.0  # sigma_xy != sigma_yx
    d = descriptors(g, sp, alg.tolerance, data.get("bodyforce"), data["dt"])
    with pytest.raises(_capi.MPMError) as e:
        MPMContext(d)
    assert e.value.code == _capi.MPM_ERR_ARG
