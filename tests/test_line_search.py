"""The Newton line search (mnralg_ls, src/mnralg.f:758-914) restated in
warp3d_gb300.newton.line_search, with WARP3D's defaults (rho 0.7, slack
tolerance 0.5, step lengths 0.01 .. 1, indypm.f:1278-1283): the search
rules on synthetic s(alpha), and a Newton run it rescues -- a small
tetrahedral bar of the example UMAT (linear kinematic hardening, two yield
stresses) whose second step's full Newton steps never converge."""
import numpy as np
import pytest

import oracle
from tests.conftest import rel_err
from tests.helpers import MESHES
from warp3d_gb300 import abi
from warp3d_gb300.model import Model, Part, Umat
from warp3d_gb300.newton import NewtonDriver, line_search, uniaxial_bcs


def _record(sfun):
    calls = []

    def trial(alpha):
        calls.append(alpha)
        return sfun(alpha)
    return trial, calls


def test_full_step_accepted_when_the_ratio_is_below_the_slack_tolerance():
    trial, calls = _record(lambda a: -0.1)
    assert line_search(-1.0, trial) == (1.0, 1)
    assert calls == [1.0]


def test_backtracks_by_rho_until_the_ratio_falls_below_one_half():
    # s(alpha) = s0 (1 - alpha / 0.45): |s / s0| < 0.5 first at alpha = 0.7^2
    trial, calls = _record(lambda a: -1.0 * (1.0 - a / 0.45))
    alpha, n = line_search(-1.0, trial)
    assert np.isclose(alpha, 0.49) and n == 3
    assert np.allclose(calls, [1.0, 0.7, 0.49])


def test_ratio_not_decreasing_takes_the_full_step():
    # |s / s0| = 0.95, 0.94, ...: not 10% smaller -> recompute at alpha = 1
    trial, calls = _record(lambda a: {1.0: -0.95, 0.7: -0.94}[round(a, 9)])
    alpha, _ = line_search(-1.0, trial)
    assert alpha == 1.0 and calls == [1.0, 0.7, 1.0]


def test_below_the_minimum_step_length_takes_the_full_step():
    # the ratio falls by 20% per trial but never below 0.5 before alpha < 0.01
    # (|s / s0| = 20 * 0.8^k at the k-th trial, alpha = 0.7^k)
    trial, calls = _record(lambda a: -20.0 * 0.8 ** round(np.log(a) / np.log(0.7)))
    alpha, _ = line_search(-1.0, trial)
    assert alpha == 1.0 and calls[-1] == 1.0 and min(calls) >= 0.01 and calls[-2] < 0.015


def _bar():
    etype, nxyz = abi.ETYPE_TET10, (1, 1, 2)
    coords, incid = MESHES[etype](1, jitter=0.08, seed=37, n_xyz=nxyz)
    mats = [Umat((200000.0, 0.3, 400.0 + 25.0 * b, 2000.0, 0.0)) for b in range(2)]
    return Model(coords, parts=[Part(etype, incid, [7, 5], mats)], geonl=False), nxyz


def run_bar(engine_cls, line_search_on, steps=4, device=False):
    model, nxyz = _bar()
    eng = engine_cls(model)
    fixed, topz = uniaxial_bcs(model, nxyz)
    if device:
        from warp3d_gb300.solver import DeviceNewtonDriver
        drv = DeviceNewtonDriver(model, eng, fixed, tol=1e-8, maxit=40, line_search=line_search_on)
    else:
        drv = NewtonDriver(model, eng, fixed, tol=1e-8, maxit=40, line_search=line_search_on)
    for s in range(1, steps + 1):
        imp = np.zeros(model.nodof)
        imp[topz] = 0.0015 * nxyz[2]
        drv.step(s, imp)
    return drv


def test_line_search_rescues_a_stalled_newton_run():
    try:
        run_bar(oracle.Oracle, False, steps=2)
        raise AssertionError("expected the full-step run to stall")
    except RuntimeError as exc:
        assert "no convergence" in str(exc)
    drv = run_bar(oracle.Oracle, True)
    assert [h[1] for h in drv.history] == [1, 6, 6, 6]
    # the search shortens the second iteration of every plastic step
    assert all(al[1] < 0.6 for _, al in drv.alphas[1:])


@pytest.mark.gpu
def test_device_newton_with_line_search_matches_the_host_driver():
    """The device Newton loop (solver.DeviceNewtonDriver: device recovery,
    assembly, PCG and one device s-value reduction per trial length) with
    the line search on, against the host driver on the oracle: the same
    iteration counts, the same accepted step lengths, displacements equal
    to the Newton tolerance."""
    from warp3d_gb300.engine import Engine
    from warp3d_gb300.solver import DeviceNewtonDriver
    host = run_bar(oracle.Oracle, True)
    model, nxyz = _bar()
    fixed, topz = uniaxial_bcs(model, nxyz)
    dev = DeviceNewtonDriver(model, Engine(model), fixed, tol=1e-8, maxit=40, lin_rtol=1e-12, line_search=True)
    for s in range(1, 5):
        imp = np.zeros(model.nodof)
        imp[topz] = 0.0015 * nxyz[2]
        dev.step(s, imp)
    its = [[h[1] for h in d.history] for d in (host, dev)]
    print("iterations host / device", its, "alphas", dev.alphas)
    assert its[0] == its[1]
    for (_, a), (_, b) in zip(host.alphas, dev.alphas):
        assert np.allclose(a, b, rtol=1e-12, atol=0.0), (a, b)
    assert rel_err(dev.u, host.u) < 1e-7
