"""Known answers for the oracle's UMAT path (material model 8 with the
reference's example UMAT: Mises plasticity with linear kinematic
hardening, src/user_routines_umat.f:77-330, driven as drive_umat_update
does, src/rstgp1.f:3476).

- uniaxial stress of a small-displacement bar, loaded in tension then
  reversed: the closed form of linear kinematic hardening (elastic slope E,
  plastic slope E H/(E + H), reverse yielding after a stress drop of twice
  the yield stress -- the Bauschinger shift), for 8-node bricks, 20-node
  bricks and tetrahedra;
- the symmetrised [D] against central differences of the stress update;
- below yield: the isotropic elastic [D] and no state change;
- the kiter = 0 path: [D] and the stress of the increment, no history.
"""
import numpy as np
import pytest

import oracle
from tests.conftest import rel_err
from tests.helpers import MESHES
from warp3d_gb300 import abi
from warp3d_gb300.model import Model, Umat
from warp3d_gb300.newton import NewtonDriver, uniaxial_bcs

E, NU, SY, H = 200000.0, 0.3, 400.0, 2000.0
PROPS = (E, NU, SY, H, 0.0)


def _elastic_D():
    lam = E * NU / ((1 + NU) * (1 - 2 * NU))
    G = E / (2 * (1 + NU))
    D = np.zeros((6, 6))
    D[:3, :3] = lam
    D[np.arange(3), np.arange(3)] += 2 * G
    D[3, 3] = D[4, 4] = D[5, 5] = G
    return D


@pytest.mark.parametrize("etype", [abi.ETYPE_L3DISOP, abi.ETYPE_Q3DISOP, abi.ETYPE_TET10])
def test_umat_uniaxial_tension_and_reversal_closed_form(etype):
    n = 3 if etype == abi.ETYPE_L3DISOP else 2
    coords, incid = MESHES[etype](n, jitter=0.0, n_xyz=(n, n, n))
    model = Model(coords, incid, etype=etype, geonl=False, materials=[Umat(PROPS)])
    ora = oracle.Oracle(model)
    fixed, topz = uniaxial_bcs(model, (n, n, n))
    drv = NewtonDriver(model, ora, fixed, tol=1e-10)
    Et = E * H / (E + H)
    # strain path: 8 steps to 1%, then 12 steps back to -0.5%
    path = list(np.linspace(0.00125, 0.01, 8)) + list(np.linspace(0.01 - 0.00125, -0.005, 12))
    e_prev, s_max = 0.0, None
    for s, e in enumerate(path, start=1):
        imp = np.zeros(model.nodof)
        imp[topz] = (e - e_prev) * n
        drv.step(s, imp)
        e_prev = e
        st = ora.state
        ezz = np.concatenate([a.reshape(-1, 6) for a in st.eps_n])[:, 2]
        szz = np.concatenate([a.reshape(-1, 9) for a in st.urcs_n])[:, 2]
        assert rel_err(ezz, np.full_like(ezz, e)) < 1e-8
        if s <= 8:   # monotonic tension
            ref = E * e if E * e <= SY else SY + Et * (e - SY / E)
            s_max = ref
        else:        # reversal: elastic until s_max - 2 SY, then the plastic slope
            e_max = 0.01
            se = s_max - E * (e_max - e)
            ref = se if se >= s_max - 2 * SY else (s_max - 2 * SY) + Et * (e - (e_max - 2 * SY / E))
        assert rel_err(szz, np.full_like(szz, ref)) < 1e-8, (s, e, szz[0], ref)


def test_umat_tangent_is_the_derivative_of_the_stress_update():
    rng = np.random.default_rng(4)
    # a plastic state at n: one update beyond yield, then a further increment
    d0 = np.array([0.004, -0.001, -0.0012, 0.0008, 0.0005, -0.0003])
    st, un, hn, _ = oracle.umat_point(PROPS, 1, 1, False, np.zeros(9), np.zeros(6), d0, np.zeros(20))
    assert st == 0 and hn[19] == 1.0
    d1 = rng.normal(0.0, 1e-3, 6)
    _, s1, _, D = oracle.umat_point(PROPS, 2, 1, False, un, d0, d1, hn)
    Dfd = np.zeros((6, 6))
    h = 1e-7
    for k in range(6):
        dp, dm = d1.copy(), d1.copy()
        dp[k] += h
        dm[k] -= h
        sp = oracle.umat_point(PROPS, 2, 1, False, un, d0, dp, hn)[1][:6]
        sm = oracle.umat_point(PROPS, 2, 1, False, un, d0, dm, hn)[1][:6]
        Dfd[:, k] = (sp - sm) / (2 * h)
    # the UMAT's [D] is the consistent tangent of the radial return, and
    # symmetric already, so its symmetrised store equals it
    assert rel_err(D, Dfd) < 1e-6


def test_umat_elastic_state_and_iteration_zero():
    d = np.array([1e-4, -3e-5, -3e-5, 2e-5, 0.0, 1e-5])
    st, un1, h1, D = oracle.umat_point(PROPS, 1, 1, False, np.zeros(9), np.zeros(6), d, np.zeros(20))
    assert st == 0
    assert rel_err(D, _elastic_D()) < 1e-14
    assert rel_err(un1[:6], _elastic_D() @ d) < 1e-14
    assert h1[18] == 0.0 and h1[19] == 0.0
    # total work: the trapezoid rule, plastic work zero
    assert abs(un1[6] - 0.5 * un1[:6] @ d) < 1e-14 * abs(un1[6])
    assert un1[7] == 0.0
    # kiter = 0, no extrapolation: [D] and the stress of the imposed
    # increment at the state n; history untouched (not written)
    h0 = np.full(20, -7.0)
    st, un1, h1, D = oracle.umat_point(PROPS, 1, 0, False, np.zeros(9), np.zeros(6), d, h0)
    assert st == 0 and np.all(h1 == 0.0)
    assert rel_err(un1[:6], _elastic_D() @ d) < 1e-14
