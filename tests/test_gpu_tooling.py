"""Timers, output checks, failure statuses and the autotuning cache.

Failures are made on the host (inputs), never on the device: an inverted
element is covered by test_gpu_parity.py; here a NaN in the increment, and
a crystal whose local Newton limit (miter = 1) cannot be met. WARP3D lets a
NaN input through its element routines without a step cut, as the engine
does; w3g_check_finite reports it. The local-solve failure returns
W3G_LOCAL_FAIL (WARP3D's material_cut_step) on both the engine and the
oracle.
"""
import json

import numpy as np
import pytest

import oracle
from tests.helpers import make_model
from warp3d_gb300 import abi
from warp3d_gb300.model import Crystal, Model, cube_mesh, random_orientations

pytestmark = pytest.mark.gpu


def _engine(model, **kw):
    from warp3d_gb300.engine import Engine
    return Engine(model, **kw)


def test_timers_accumulate_per_entry_point():
    model, _ = make_model(n=3, jitter=0.1, spans=[20, 7])
    eng = _engine(model)
    u = np.zeros(model.nodof)
    du = np.random.default_rng(1).normal(0.0, 1e-3, model.nodof)
    ifv = np.zeros(model.nodof)
    for _ in range(2):
        eng.recover(1, 1, False, model.c, u, du, ifv)
        eng.tanstf(1, 1, model.c, u, du, model.estiff_blocks())
    eng.update()
    t = eng.timers()
    assert (t["recover_calls"], t["tangent_calls"], t["update_calls"]) == (2, 2, 1)
    assert t["recover_s"] > 0.0 and t["tangent_s"] > 0.0 and t["update_s"] > 0.0
    eng.reset_timers()
    assert eng.timers()["recover_calls"] == 0


def test_check_finite_reports_a_poisoned_increment():
    model, _ = make_model(n=3, jitter=0.1, spans=[27])
    eng = _engine(model)
    u = np.zeros(model.nodof)
    du = np.random.default_rng(2).normal(0.0, 1e-3, model.nodof)
    ifv = np.zeros(model.nodof)
    st, _ = eng.recover(1, 1, False, model.c, u, du, ifv)
    eng.tanstf(1, 1, model.c, u, du, None)
    assert st == 0 and eng.check_finite() == 0
    du[3 * 13 + 1] = np.nan                       # one dof of an interior node
    eng.recover(1, 1, False, model.c, u, du, ifv)
    eng.tanstf(1, 1, model.c, u, du, None)
    bad = eng.check_finite()
    print("non-finite values after a NaN increment:", bad)
    assert bad > 0
    assert np.isnan(ifv).any()


def test_local_newton_failure_returns_local_fail():
    coords, incid = cube_mesh(2, jitter=0.05)
    model = Model(coords, incid, materials=[Crystal(miter=1)], angles=random_orientations(8, 3))
    u = np.zeros(model.nodof)
    du = np.zeros(model.nodof)
    top = np.where(np.isclose(model.coords[:, 2], 2.0))[0]
    du[3 * top + 2] = 0.02                        # 1% axial strain in one increment: plastic
    ifv = np.zeros(model.nodof)
    st_o, info_o = oracle.Oracle(model).recover(1, 1, False, model.c, u, du, ifv.copy())
    st_g, info_g = _engine(model).recover(1, 1, False, model.c, u, du, ifv)
    assert st_o == st_g == abi.LOCAL_FAIL
    assert info_g.material_cut_step == abi.LOCAL_FAIL


def test_autotune_cache_is_written_and_reused(tmp_path):
    torch = pytest.importorskip("torch")
    model, _ = make_model(n=4, jitter=0.1, spans=[40, 24])
    eng = _engine(model)
    dev = torch.device("cuda", 0)
    c = torch.from_numpy(model.c).to(dev)
    u = torch.zeros(model.nodof, dtype=torch.float64, device=dev)
    du = torch.from_numpy(np.random.default_rng(3).normal(0.0, 1e-3, model.nodof)).to(dev)
    ifv = torch.zeros_like(u)
    cache = str(tmp_path / "tune.json")
    sc1, ms1 = eng.autotune(1, 1, False, c.data_ptr(), u.data_ptr(), du.data_ptr(), ifv.data_ptr(), cache=cache)
    data = json.load(open(cache))
    key = eng.tuning_key()
    assert key in data and data[key]["schedule"] == sc1
    assert "hex8" not in key and "p0" in key
    eng2 = _engine(model)
    sc2, ms2 = eng2.autotune(1, 1, False, c.data_ptr(), u.data_ptr(), du.data_ptr(), ifv.data_ptr(), cache=cache)
    assert sc2 == sc1 and ms2 == ms1
    assert eng2.schedule() == sc1
