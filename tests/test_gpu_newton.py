"""End-to-end Newton solutions driven through the CUDA engine.

The 8x8x8 uniaxial bilinear cube of the plain method (512 hex8, 10 steps
to 1% strain): the GPU engine reproduces the closed-form stress-strain
response and the oracle-driven solution; with the FP32 (precision form)
tangent the same converged displacements are reached to the 1e-8
relative global residual, at the cost of extra Newton iterations.
"""
import numpy as np
import pytest

import oracle
from tests.conftest import rel_err
from warp3d_gb300 import abi
from warp3d_gb300.model import Model, cube_mesh
from warp3d_gb300.newton import NewtonDriver, uniaxial_bcs

pytestmark = pytest.mark.gpu


def _run(engine_factory, n=8, nsteps=10, jitter=0.0, tol=1e-8):
    coords, incid = cube_mesh(n, jitter=jitter)
    model = Model(coords, incid)
    eng = engine_factory(model)
    fixed, topz = uniaxial_bcs(model, (n, n, n))
    drv = NewtonDriver(model, eng, fixed, tol=tol)
    for s in range(1, nsteps + 1):
        imp = np.zeros(model.nodof)
        imp[topz] = 0.01 * n / nsteps
        drv.step(s, imp)
    return model, eng, drv


def _gpu(precision=abi.TANGENT_FP64):
    from warp3d_gb300.engine import Engine
    return lambda m: Engine(m, precision=precision)


def test_plain_gpu_newton_matches_oracle_and_closed_form():
    m_o, ora, d_o = _run(oracle.Oracle)
    m_g, eng, d_g = _run(_gpu())
    assert rel_err(d_g.u, d_o.u) < 1e-9
    st = m_g.new_state()
    eng.download(st)
    szz = np.concatenate(st.urcs_n)[:, :, 2]
    ezz = np.concatenate(st.eps_n)[:, :, 2].mean()
    p = m_g.props[0]
    E, sy, H = float(p[6]), float(p[22]), float(p[14])
    ref = sy + E * H / (E + H) * (ezz - sy / E)
    assert abs(szz.mean() - ref) < 1e-11 * ref
    assert [h[1] for h in d_g.history] == [h[1] for h in d_o.history]


def test_mixed_precision_tangent_reaches_same_solution():
    m_p, e_p, d_p = _run(_gpu(), jitter=0.1)
    m_m, e_m, d_m = _run(_gpu(abi.TANGENT_FP32), jitter=0.1)
    its_p = [h[1] for h in d_p.history]
    its_m = [h[1] for h in d_m.history]
    print("newton iterations per step: fp64", its_p, "fp32 tangent", its_m)
    assert rel_err(d_m.u, d_p.u) < 1e-7
    assert max(h[2][-1] for h in d_m.history) <= 1e-8
