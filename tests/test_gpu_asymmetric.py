"""Asymmetric assembly ("assembly asymmetric on"): full column-major
element matrices (totdof², span) for 8-node bricks (gptns1.f bdbt_asym,
kg1.f's asymmetric branch, tanstf.f:223-225) and mm10 tangents left
unsymmetrized (mm10_a.f:1165-1166); 20-node bricks and tetrahedra (mm01)
through their packed items and an expansion. The CUDA engine against the
oracle at the plain path's 1e-12 (FP32: 1e-5); the tensor-core forms and
the symmetric-only device solver are refused."""
import numpy as np
import pytest

import oracle
from tests.conftest import rel_err
from tests.helpers import loaded_state, make_model
from warp3d_gb300 import abi
from warp3d_gb300.model import Crystal, Model, cube_mesh, random_orientations
from warp3d_gb300.newton import NewtonDriver, uniaxial_bcs

pytestmark = pytest.mark.gpu


def _engine(model):
    from warp3d_gb300.engine import Engine
    return Engine(model)


def _pair(model, state, step, it, extrap, u, du):
    eng = _engine(model)
    eng.upload(state)
    ora = oracle.Oracle(model, state=state.copy())
    fo, fg = np.zeros(model.nodof), np.zeros(model.nodof)
    assert ora.recover(step, it, extrap, model.c, u, du, fo)[0] == 0
    assert eng.recover(step, it, extrap, model.c, u, du, fg)[0] == 0
    got = model.new_state()
    eng.download(got)
    errs = {n: rel_err(got.concat(n), ora.state.concat(n)) for n in ("urcs_n1", "history1", "einfvec")}
    errs["ifv"] = float(np.max(np.abs(fg - fo)) / np.max(np.abs(ora.state.concat("einfvec"))))
    ko, kg = model.estiff_blocks(), model.estiff_blocks()
    ora.tanstf(step, it, model.c, u, du, ko)
    eng.tanstf(step, it, model.c, u, du, kg)
    errs["ke"] = max(rel_err(g, o, axis=1) for g, o in zip(kg, ko))
    return eng, ora, errs, ko


@pytest.mark.parametrize("opts", [dict(), dict(bbar=True), dict(geonl=False, bbar=True)])
def test_bilinear_full_matrices(opts):
    model, nxyz = make_model(n=4, jitter=0.1, spans=[40, 24], asymmetric=True, **opts)
    assert model.estiff_blocks()[0].shape == (40, 576)
    ora, drv, du = loaded_state(model, nxyz, oracle.Oracle, steps=2, strain_per_step=0.0015, shear_per_step=0.001)
    eng, o2, errs, ko = _pair(model, ora.state, 3, 1, False, drv.u, du)
    print(opts, {k: f"{v:.1e}" for k, v in errs.items()})
    assert max(errs.values()) <= 1e-12, errs
    K = ko[0][5].reshape(24, 24).T
    assert rel_err(K, K.T) < 1e-13          # a symmetric material gives a symmetric matrix
    eng.set_precision(abi.TANGENT_FP32)
    kg = model.estiff_blocks()
    eng.tanstf(3, 1, model.c, drv.u, du, kg)
    assert max(rel_err(g, o, axis=1) for g, o in zip(kg, ko)) <= 1e-5
    with pytest.raises(abi.W3GError):
        eng.set_precision(abi.TANGENT_TF32)


def test_crystal_full_unsymmetric_matrices():
    coords, incid = cube_mesh(3, jitter=0.05)
    model = Model(coords, incid, materials=[Crystal()], angles=random_orientations(27, 7), block_spans=[20, 7],
                  asymmetric=True)
    nxyz = (3, 3, 3)
    ora = oracle.Oracle(model)
    fixed, topz = uniaxial_bcs(model, nxyz)
    drv = NewtonDriver(model, ora, fixed, tol=1e-8, maxit=60, extrapolate=True)
    for s in range(1, 3):
        imp = np.zeros(model.nodof)
        imp[topz] = 0.0005 * nxyz[2]
        drv.step(s, imp)
    du = drv.du_prev.copy()
    eng, o2, errs, ko = _pair(model, ora.state, 3, 1, False, drv.u, du)
    print({k: f"{v:.1e}" for k, v in errs.items()})
    assert max(errs.values()) <= 1e-12, errs
    asym = max(rel_err(k.reshape(24, 24).T, k.reshape(24, 24)) for blk in ko for k in blk)
    assert asym > 1e-8


@pytest.mark.parametrize("etype,spans", [(abi.ETYPE_Q3DISOP, [5, 3]), (abi.ETYPE_TET10, [30, 18])])
def test_other_types_full_matrices(etype, spans):
    # 20-node bricks and tetrahedra (mm01): packed work items, expanded
    model, nxyz = make_model(n=2, jitter=0.08, spans=spans, etype=etype, asymmetric=True)
    tot = model.totdof
    assert model.estiff_blocks()[0].shape == (spans[0], tot * tot)
    ora, drv, du = loaded_state(model, nxyz, oracle.Oracle, steps=2, strain_per_step=0.0015)
    eng, o2, errs, ko = _pair(model, ora.state, 3, 1, False, drv.u, du)
    print(etype, {k: f"{v:.1e}" for k, v in errs.items()})
    assert max(errs.values()) <= 1e-12, errs
    eng.set_precision(abi.TANGENT_FP32)
    kg = model.estiff_blocks()
    eng.tanstf(3, 1, model.c, drv.u, du, kg)
    assert max(rel_err(g, o, axis=1) for g, o in zip(kg, ko)) <= 1e-5


def test_mixed_types_full_matrices():
    from warp3d_gb300.model import Bilinear, Part, cube_mesh_hex20
    c8, i8 = cube_mesh(2, jitter=0.05)
    c20, i20 = cube_mesh_hex20(2, jitter=0.05)
    # two disconnected parts: bricks, then 20-node bricks shifted aside
    off = c8.shape[0]
    coords = np.vstack([c8, c20 + np.array([5.0, 0.0, 0.0])])
    mat = Bilinear.from_hprime(200000.0, 0.3, 400.0, 2000.0)
    model = Model(coords, parts=[Part(abi.ETYPE_L3DISOP, i8, [8], [mat]),
                                 Part(abi.ETYPE_Q3DISOP, i20 + off, [8], [mat])], asymmetric=True)
    du = np.random.default_rng(4).normal(0.0, 1e-4, model.nodof)
    state = model.new_state()
    eng, o2, errs, ko = _pair(model, state, 1, 1, False, np.zeros(model.nodof), du)
    assert max(errs.values()) <= 1e-12, errs


def test_refusals():
    coords, incid = cube_mesh(2)
    from warp3d_gb300.solver import DeviceCsr
    with pytest.raises(abi.W3GError):
        DeviceCsr(_engine(Model(coords, incid, asymmetric=True)))
