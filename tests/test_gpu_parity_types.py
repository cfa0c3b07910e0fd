"""Parity of the CUDA engine with the oracle for the 20-node brick
(q3disop, 27 Gauss points), the 10-node tetrahedron (4 Gauss points) and
a model that mixes all three element types in blocks of uneven size.

Same bar as the 8-node cases: every output array of recovery and tangent
within 1e-12 of the oracle (max |gpu - oracle| / max |oracle| per array,
per element for Ke); the FP32 tangent within 1e-5.
"""
import numpy as np
import pytest

import oracle
from tests.conftest import rel_err
from tests.helpers import loaded_state, make_model
from warp3d_gb300 import abi
from warp3d_gb300.model import Bilinear, Model, Part, mixed_mesh, random_spans

pytestmark = pytest.mark.gpu

TOL = 1e-12
TOL_FP32 = 1e-5


def _engine(model, **kw):
    from warp3d_gb300.engine import Engine
    return Engine(model, **kw)


def _flat(blocks):
    return np.concatenate([b.reshape(-1) for b in blocks])


def _state_word(h):
    return h[..., 3].copy().view(np.int64) & 0xFFFFFFFF


def _recover_both(model, state, step, it, extrap, u, du):
    eng = _engine(model)
    eng.upload(state)
    ora = oracle.Oracle(model, state=state.copy())
    ifv_o = np.zeros(model.nodof)
    ifv_g = np.zeros(model.nodof)
    st_o, info_o = ora.recover(step, it, extrap, model.c, u, du, ifv_o)
    st_g, info_g = eng.recover(step, it, extrap, model.c, u, du, ifv_g)
    assert st_o == st_g == 0
    got = model.new_state()
    eng.download(got)
    o = ora.state
    errs = {}
    for name in ("urcs_n1", "eps_n1", "cep", "einfvec", "element_vol"):
        errs[name] = rel_err(_flat(getattr(got, name)), _flat(getattr(o, name)))
    if it > 0:
        errs["rot_n1"] = rel_err(_flat(got.rot_n1), _flat(o.rot_n1))
        keep = [k for k in range(11) if k != 3]
        errs["history1"] = rel_err(_flat([h[..., keep] for h in got.history1]),
                                   _flat([h[..., keep] for h in o.history1]))
        for hg, ho in zip(got.history1, o.history1):
            assert np.array_equal(_state_word(hg), _state_word(ho))
    errs["ifv"] = float(np.max(np.abs(ifv_g - ifv_o)) / np.max(np.abs(_flat(o.einfvec))))
    errs["energy"] = abs(info_g.internal_energy - info_o.internal_energy) / max(abs(info_o.internal_energy), 1e-300)
    if info_o.plastic_work != 0.0:
        errs["plastic_work"] = abs(info_g.plastic_work - info_o.plastic_work) / abs(info_o.plastic_work)
    errs["sum_ifv"] = abs(info_g.sum_ifv - info_o.sum_ifv) / info_o.sum_ifv
    assert info_g.num_term_ifv == info_o.num_term_ifv
    print("recover parity", {k: f"{v:.2e}" for k, v in errs.items()})
    for k, v in errs.items():
        assert v <= TOL, (k, v)
    return eng, ora


def _tangent_both(model, eng, ora, step, it, u, du, tol=TOL):
    est_o = model.estiff_blocks()
    est_g = model.estiff_blocks()
    ora.tanstf(step, it, model.c, u, du, est_o)
    eng.tanstf(step, it, model.c, u, du, est_g)
    err = max(rel_err(g, o, axis=1) for g, o in zip(est_g, est_o))
    print(f"tangent parity {err:.2e}")
    assert err <= tol


@pytest.fixture(scope="module", params=[abi.ETYPE_Q3DISOP, abi.ETYPE_TET10], ids=["hex20", "tet10"])
def typed_case(request):
    etype = request.param
    spans = [20, 7] if etype == abi.ETYPE_Q3DISOP else [100, 1, 61]
    model, nxyz = make_model(n=3, jitter=0.08, spans=spans, etype=etype)
    ora, drv, du = loaded_state(model, nxyz, oracle.Oracle, steps=3, strain_per_step=0.0015,
                                shear_per_step=0.001)
    return model, ora.state, drv.u.copy(), du


def test_typed_recover_and_tangent_parity(typed_case):
    model, state, u, du = typed_case
    eng, ora = _recover_both(model, state, 4, 1, False, u, du)
    _tangent_both(model, eng, ora, 4, 1, u, du)


def test_typed_iteration_zero(typed_case):
    model, state, u, du = typed_case
    eng, ora = _recover_both(model, state, 4, 0, False, u, du)
    _tangent_both(model, eng, ora, 4, 0, u, du)
    _recover_both(model, state, 4, 0, True, u, du)


def test_typed_first_step():
    for etype in (abi.ETYPE_Q3DISOP, abi.ETYPE_TET10):
        model, nxyz = make_model(n=2, jitter=0.08, spans=None, etype=etype)
        state = model.new_state()
        rng = np.random.default_rng(5)
        du = rng.normal(0.0, 2e-3, model.nodof)
        u = np.zeros(model.nodof)
        eng, ora = _recover_both(model, state, 1, 1, False, u, du)
        _tangent_both(model, eng, ora, 1, 1, u, du)
        _recover_both(model, state, 1, 0, False, u, du)


def test_typed_fp32_tangent(typed_case):
    model, state, u, du = typed_case
    eng, ora = _recover_both(model, state, 4, 1, False, u, du)
    eng.set_precision(abi.TANGENT_FP32)
    _tangent_both(model, eng, ora, 4, 1, u, du, tol=TOL_FP32)


def _mixed_model(seed=11):
    rng = np.random.Generator(np.random.PCG64(seed))
    coords, parts, origins = mixed_mesh(
        [(abi.ETYPE_L3DISOP, 3), (abi.ETYPE_Q3DISOP, 2), (abi.ETYPE_TET10, 2)], ny=2, nz=3, jitter=0.05, seed=seed)
    plist = []
    for etype, inc in parts:
        spans = random_spans(inc.shape[0], rng, 1, 20)
        mats = [Bilinear.from_hprime(200000.0, 0.3, float(rng.uniform(250.0, 550.0)), 2000.0) for _ in spans]
        plist.append(Part(etype, inc, spans, mats))
    return Model(coords, parts=plist), origins


def test_mixed_types_uneven_blocks():
    model, origins = _mixed_model()
    assert not model.uniform and model.nelblk > 6
    # pure tension: with per-block yields down to 250 MPa an added shear
    # makes the oracle's Newton iterations on the tetrahedra diverge (their
    # geometric stiffness carries the unscaled weights, as in the reference)
    ora, drv, du = loaded_state(model, (3, 2, 3), oracle.Oracle, steps=3, strain_per_step=0.0015,
                                origins=origins)
    eng, o2 = _recover_both(model, ora.state, 4, 1, False, drv.u, du)
    _tangent_both(model, eng, o2, 4, 1, drv.u, du)
    eng.set_precision(abi.TANGENT_FP32)
    _tangent_both(model, eng, o2, 4, 1, drv.u, du, tol=TOL_FP32)
    # hex8, hex20 and tet10 element kernels: one launch each
    assert eng.last_launch_count() == 3
