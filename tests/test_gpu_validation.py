"""Input validation that runs on the device: the upload kernels compare the
mirrored entries of every strain, stress and (3D) plastic-strain matrix and
mpm_create / mpm_batch_create reject asymmetric ones with MPM_ERR_ARG, as
the symmetric storage would otherwise drop half of the matrix."""
import ctypes as C

import numpy as np
import pytest

from jump_gb300 import _capi, scenarios
from jump_gb300.batch import Ensemble
from jump_gb300.engine import Descriptors, MPMContext

pytestmark = pytest.mark.gpu


def create_rc(grid, solids, alg, data):
    L = _capi.lib()
    d = Descriptors(grid, solids, tolerance=alg.tolerance, body_force=data.get("bodyforce"), dt=data["dt"])
    h = C.c_void_p()
    rc = L.mpm_create(C.byref(d.grid), d.bodies, d.nbodies, C.byref(d.params), C.byref(h))
    if rc == _capi.MPM_OK:
        L.mpm_destroy(h)
    return rc, L.mpm_last_error()


def test_asymmetric_stress_rejected():
    g, s, alg, data = scenarios.two_disks(nodes=6)
    s[1].stress[s[1].parCount - 1] = np.array([[1.0, 2.0], [3.0, 4.0]])
    rc, msg = create_rc(g, s, alg, data)
    assert rc == _capi.MPM_ERR_ARG and b"symmetric" in msg


def test_asymmetric_strain_rejected():
    g, s, alg, data = scenarios.two_disks(nodes=6)
    s[0].strain[3] = np.array([[0.0, 1e-9], [0.0, 0.0]])
    rc, msg = create_rc(g, s, alg, data)
    assert rc == _capi.MPM_ERR_ARG and b"strain and stress" in msg


def test_asymmetric_pstrain_3d_rejected():
    g, s, alg, data = scenarios.taylor_bar(h=1e-3)
    scenarios.apply_dirichlet(g, data)
    s[0].mat.pstrain_3D[7] = np.array([[0.0, 0.0, 1.0], [0.0, 0.0, 0.0], [0.0, 0.0, 0.0]])
    rc, msg = create_rc(g, s, alg, data)
    assert rc == _capi.MPM_ERR_ARG and b"pstrain" in msg


def test_symmetric_inputs_accepted_and_status_clear():
    """A symmetric non-zero stress passes, and the upload check leaves no bit
    behind for the first step's status."""
    g, s, alg, data = scenarios.two_disks(nodes=6)
    s[0].stress[:] = np.array([[1.0, 2.0], [2.0, 4.0]])
    ctx = MPMContext(Descriptors(g, s, tolerance=alg.tolerance, body_force=data["bodyforce"], dt=data["dt"]))
    assert ctx.step(1) == _capi.MPM_OK
    st = ctx.download_body(0)
    sig = st.matrices()[2]
    assert np.allclose(sig[:, 0, 1], sig[:, 1, 0])
    ctx.close()


def test_batch_rejects_asymmetric_stress():
    probs = [scenarios.ensemble_member(i, gap=0.0) for i in range(3)]
    probs[2][1][0].stress[0] = np.array([[1.0, 2.0], [3.0, 4.0]])
    with pytest.raises(_capi.MPMError, match="symmetric"):
        Ensemble(probs)
