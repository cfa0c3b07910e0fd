"""The in-place update (W3G_UPDATE_SWAP, w3g_set_update_mode): WARP3D's
update (src/update.f:73-94) copies the converged n+1 history, strains and
stresses into n; the swap mode exchanges the arrays instead and copies
back only the history of crystal-plasticity blocks, whose local solve
starts from history1. Newton runs in both modes must be bitwise equal --
displacements, iteration counts and the state at n after every step -- on
a model of bilinear (mm01) and UMAT blocks of all three element types and
on a polycrystal of mm10 bricks."""
import numpy as np
import pytest

from tests.test_gpu_umat import _model
from warp3d_gb300 import abi
from warp3d_gb300.model import Crystal, Model, cube_mesh, random_orientations
from warp3d_gb300.newton import NewtonDriver, uniaxial_bcs

pytestmark = pytest.mark.gpu


def _run(model, nxyz, origins, mode, steps, strain, **kw):
    from warp3d_gb300.engine import Engine
    eng = Engine(model)
    eng.set_update_mode(mode)
    fixed, topz = uniaxial_bcs(model, nxyz, origins=origins)
    drv = NewtonDriver(model, eng, fixed, tol=1e-8, **kw)
    states = []
    for s in range(1, steps + 1):
        imp = np.zeros(model.nodof)
        imp[topz] = strain * nxyz[2]
        drv.step(s, imp)
        st = model.new_state()
        eng.download(st, names=("history", "urcs_n", "eps_n"))
        states.append(st)
    eng.close()
    return drv, states


def _same(a, b):
    assert [h[1] for h in a[0].history] == [h[1] for h in b[0].history]
    assert np.array_equal(a[0].u, b[0].u)
    for sa, sb in zip(a[1], b[1]):
        for name in ("history", "urcs_n", "eps_n"):
            for x, y in zip(getattr(sa, name), getattr(sb, name)):
                assert np.array_equal(x, y), name


def test_swap_update_equals_copy_update_mm01_and_umat():
    model, origins = _model(True, seed=29, types=(abi.ETYPE_L3DISOP, abi.ETYPE_Q3DISOP))
    runs = [_run(model, (3, 2, 3), origins, mode, 3, 0.0015, maxit=40) for mode in (abi.UPDATE_COPY, abi.UPDATE_SWAP)]
    _same(*runs)


def test_swap_update_equals_copy_update_crystal():
    n = 2
    coords, incid = cube_mesh(n, jitter=0.05)
    model = Model(coords, incid, materials=[Crystal()], angles=random_orientations(n ** 3, 7), dt=1.0)
    runs = [_run(model, (n, n, n), None, mode, 3, 0.0005, maxit=60, extrapolate=True)
            for mode in (abi.UPDATE_COPY, abi.UPDATE_SWAP)]
    _same(*runs)


def test_update_mode_rejects_unknown_values():
    from warp3d_gb300.engine import Engine
    model, _ = _model(True, seed=3, types=(abi.ETYPE_L3DISOP,))
    eng = Engine(model)
    with pytest.raises(abi.W3GError):
        eng.set_update_mode(7)
    eng.close()
