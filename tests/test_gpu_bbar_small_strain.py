"""Parity of the CUDA engine with the oracle for the b-bar bricks (WARP3D's
default l3disop formulation: vol_terms, vol_avg, bmod, kgstiff with the
averaged derivatives) and for small-displacement blocks (rstgp2).

The GPU evaluates b-bar as B + beta m (v - g)^T: in the recovery as the
element-mean dilatation rate added to each point's normal rates and the
element-mean pressure replacing each point's in the internal forces; in
the tangent as D* B-bar = D* B + (D* m) h^T with h = beta (v - g). The
oracle follows bmod's literal update of [B]. Same bars as the plain path:
1e-12 relative for the FP64 form (states, forces, Ke per element), the
precision forms' own tolerances for the FP32 and tensor-core tangents.
"""
import numpy as np
import pytest

import oracle
from tests.conftest import rel_err
from tests.helpers import loaded_state, make_model
from warp3d_gb300 import abi
from warp3d_gb300.model import Crystal, Model, cube_mesh, random_orientations
from warp3d_gb300.newton import NewtonDriver, uniaxial_bcs

pytestmark = pytest.mark.gpu

TOL = 1e-12
TOL_TC = {abi.TANGENT_TF32: 2e-3, abi.TANGENT_BF16: 2e-2, abi.TANGENT_TF32X3: 1e-5, abi.TANGENT_BF16X3: 2e-4}

OPTIONS = {
    "bbar": dict(bbar=True),
    "bbar_stabilized": dict(bbar=True, eps_bbar=0.1),
    "small": dict(geonl=False),
    "small_bbar": dict(geonl=False, bbar=True),
}


def _engine(model, **kw):
    from warp3d_gb300.engine import Engine
    return Engine(model, **kw)


def _recover_both(model, state, step, it, u, du, sched=None):
    eng = _engine(model)
    if sched:
        eng.set_schedule(**sched)
    eng.upload(state)
    ora = oracle.Oracle(model, state=state.copy())
    ifv_o, ifv_g = np.zeros(model.nodof), np.zeros(model.nodof)
    st_o, info_o = ora.recover(step, it, False, model.c, u, du, ifv_o)
    st_g, info_g = eng.recover(step, it, False, model.c, u, du, ifv_g)
    assert st_o == st_g == 0
    got = model.new_state()
    eng.download(got)
    o = ora.state
    errs = {name: rel_err(got.concat(name), o.concat(name))
            for name in ("urcs_n1", "eps_n1", "cep", "einfvec", "element_vol", "rot_n1")}
    if it > 0 and any(model.block_crystal):
        errs["history1"] = rel_err(got.concat("history1"), o.concat("history1"))
    elif it > 0:
        keep = [k for k in range(11) if k != 3]
        errs["history1"] = rel_err(got.concat("history1")[:, :, keep], o.concat("history1")[:, :, keep])
    errs["ifv"] = float(np.max(np.abs(ifv_g - ifv_o)) / np.max(np.abs(o.concat("einfvec"))))
    errs["energy"] = abs(info_g.internal_energy - info_o.internal_energy) / max(abs(info_o.internal_energy), 1e-300)
    return eng, ora, errs


def _tangent_err(model, eng, ora, step, it, u, du):
    est_o, est_g = model.estiff_blocks(), model.estiff_blocks()
    ora.tanstf(step, it, model.c, u, du, est_o)
    eng.tanstf(step, it, model.c, u, du, est_g)
    assert all(np.all(np.isfinite(g)) for g in est_g)
    return max(rel_err(g, o, axis=1) for g, o in zip(est_g, est_o))


@pytest.fixture(scope="module", params=list(OPTIONS))
def case(request):
    opts = OPTIONS[request.param]
    model, nxyz = make_model(n=5, jitter=0.1, spans=[64, 61], **opts)
    ora, drv, du = loaded_state(model, nxyz, oracle.Oracle, steps=3, strain_per_step=0.0015,
                                shear_per_step=0.001)
    return request.param, model, ora.state, drv.u.copy(), du


def test_recover_and_tangent_parity(case):
    name, model, state, u, du = case
    eng, ora, errs = _recover_both(model, state, 4, 1, u, du)
    errs["ke"] = _tangent_err(model, eng, ora, 4, 1, u, du)
    print(name, {k: f"{v:.1e}" for k, v in errs.items()})
    assert max(errs.values()) <= TOL, errs


def test_iteration_zero(case):
    name, model, state, u, du = case
    eng, ora, errs = _recover_both(model, state, 4, 0, u, du)
    errs["ke"] = _tangent_err(model, eng, ora, 4, 0, u, du)
    print(name, {k: f"{v:.1e}" for k, v in errs.items()})
    assert max(errs.values()) <= TOL, errs


def test_persistent_schedule(case):
    name, model, state, u, du = case
    eng, ora, errs = _recover_both(model, state, 4, 2, u, du,
                                   sched=dict(mode=abi.SCHED_PERSISTENT, order=abi.ORDER_HEAVY_FIRST))
    errs["ke"] = _tangent_err(model, eng, ora, 4, 2, u, du)
    assert max(errs.values()) <= TOL, errs


def test_fp32_and_tensor_core_tangents(case):
    name, model, state, u, du = case
    eng, ora, _ = _recover_both(model, state, 4, 1, u, du)
    errs = {}
    for prec, tol in [(abi.TANGENT_FP32, 1e-5), *TOL_TC.items()]:
        eng.set_precision(prec)
        errs[prec] = _tangent_err(model, eng, ora, 4, 1, u, du)
        assert errs[prec] <= tol, (prec, errs[prec])
    print(name, {k: f"{v:.1e}" for k, v in errs.items()})


@pytest.mark.parametrize("etype", [abi.ETYPE_Q3DISOP, abi.ETYPE_TET10])
def test_small_displacement_other_types(etype):
    model, nxyz = make_model(n=2, jitter=0.08, spans=[5, 3] if etype == abi.ETYPE_Q3DISOP else [30, 18],
                             etype=etype, geonl=False)
    ora, drv, du = loaded_state(model, nxyz, oracle.Oracle, steps=3, strain_per_step=0.0015)
    eng, o2, errs = _recover_both(model, ora.state, 4, 1, drv.u, du)
    errs["ke"] = _tangent_err(model, eng, o2, 4, 1, drv.u, du)
    print(etype, {k: f"{v:.1e}" for k, v in errs.items()})
    assert max(errs.values()) <= TOL, errs


def test_blocks_with_and_without_bbar():
    # ragged blocks (40, 23, 1), the middle one a displacement brick: the
    # b-bar instantiations handle both kinds of block in one launch
    model, nxyz = make_model(n=4, jitter=0.1, spans=[40, 23, 1], bbar=True)
    model.lprops[40:63, 18] = 0
    ora, drv, du = loaded_state(model, nxyz, oracle.Oracle, steps=2, strain_per_step=0.0015)
    for sched in (None, dict(mode=abi.SCHED_PERSISTENT, order=abi.ORDER_HEAVY_FIRST)):
        eng, o2, errs = _recover_both(model, ora.state, 3, 1, drv.u, du, sched=sched)
        errs["ke"] = _tangent_err(model, eng, o2, 3, 1, drv.u, du)
        assert max(errs.values()) <= TOL, (sched, errs)
        for prec, tol in [(abi.TANGENT_FP32, 1e-5), *TOL_TC.items()]:
            eng.set_precision(prec)
            err = _tangent_err(model, eng, o2, 3, 1, drv.u, du)
            assert err <= tol, (sched, prec, err)


@pytest.mark.parametrize("opts", [dict(bbar=True), dict(geonl=False, bbar=True)])
def test_newton_engine_matches_oracle(opts):
    # residual floor of the finite-strain kinematics: ~5e-10 relative (the
    # polar decomposition near F = I), so the geonl run stops at 1e-8
    tol = 1e-8 if opts.get("geonl", True) else 1e-10
    model, nxyz = make_model(n=3, jitter=0.1, **opts)
    fixed, topz = uniaxial_bcs(model, nxyz)
    runs = {}
    for nm, eng in (("oracle", oracle.Oracle(model)), ("gpu", _engine(model))):
        drv = NewtonDriver(model, eng, fixed, tol=tol)
        its = []
        for s in range(1, 5):
            imp = np.zeros(model.nodof)
            imp[topz] = 0.0015 * nxyz[2]
            its.append(len(drv.step(s, imp)))
        runs[nm] = (drv.u.copy(), its)
    assert runs["gpu"][1] == runs["oracle"][1]
    assert rel_err(runs["gpu"][0], runs["oracle"][0]) < 10 * tol


@pytest.mark.parametrize("bbar", [False, True])
def test_crystal_small_displacement_parity(bbar):
    from warp3d_gb300.model import Crystal, Model, cube_mesh, random_orientations
    coords, incid = cube_mesh(3, jitter=0.05)
    model = Model(coords, incid, materials=[Crystal()], angles=random_orientations(27, 5), block_spans=[20, 7],
                  geonl=False, bbar=bbar)
    nxyz = (3, 3, 3)
    ora = oracle.Oracle(model)
    fixed, topz = uniaxial_bcs(model, nxyz)
    drv = NewtonDriver(model, ora, fixed, tol=1e-8, maxit=60, extrapolate=True)
    for s in range(1, 3):
        imp = np.zeros(model.nodof)
        imp[topz] = 0.0005 * nxyz[2]
        drv.step(s, imp)
    eng, o2, errs = _recover_both(model, ora.state, 3, 1, drv.u, drv.du_prev.copy())
    errs["ke"] = _tangent_err(model, eng, o2, 3, 1, drv.u, drv.du_prev.copy())
    print("mm10 small", bbar, {k: f"{v:.1e}" for k, v in errs.items()})
    assert max(errs.values()) <= TOL, errs
