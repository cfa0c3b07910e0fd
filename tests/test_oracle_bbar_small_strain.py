"""Known answers for two options of the 8-node brick path in the oracle:
the mean-dilatation b-bar (vol_terms, vol_avg, bmod, kgstiff's averaged
derivatives; WARP3D's default for l3disop elements, inelem.f:192) and the
small-displacement recovery (rstgp2, rknstr_sm_displ, rstgp1_b itype 2).

- The b-bar stiffness of a single brick against a textbook mean-dilatation
  brick written here in numpy (B-bar = B + beta m (v - g)^T with
  m = (1,1,1,0,0,0), beta = (1 - eps_bbar)/3, v the volume-averaged
  derivatives), with and without the stabilization factor.
- b-bar leaves homogeneous deformations untouched (patch test, uniaxial
  response) and changes inhomogeneous ones.
- The small-displacement tangent at a deformed state is the textbook
  stiffness of the undeformed brick; the small-displacement uniaxial
  response is the bilinear closed form in the engineering strain.
"""
import numpy as np
import pytest

import oracle
from tests.conftest import rel_err
from tests.helpers import make_model
from warp3d_gb300 import abi
from warp3d_gb300.model import HEX8_NODES, Bilinear, Crystal, Model, cube_mesh, random_orientations
from warp3d_gb300.newton import NewtonDriver, uniaxial_bcs


def _elastic_D(E, nu):
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    mu = E / (2 * (1 + nu))
    D = np.zeros((6, 6))
    D[:3, :3] = lam
    D[np.arange(3), np.arange(3)] += 2 * mu
    D[3, 3] = D[4, 4] = D[5, 5] = mu
    return D


def _brick_gradients(X):
    g = 1 / np.sqrt(3.0)
    out = []
    for sx in (-1, 1):
        for sy in (-1, 1):
            for sz in (-1, 1):
                p = np.array([sx, sy, sz]) * g
                dN = np.zeros((3, 8))
                for a, s in enumerate(HEX8_NODES):
                    f = 1 + s * p
                    dN[:, a] = [s[0] * f[1] * f[2], f[0] * s[1] * f[2], f[0] * f[1] * s[2]]
                dN /= 8
                J = dN @ X
                out.append((np.linalg.solve(J, dN), np.linalg.det(J)))
    return out


def _textbook_brick_K(X, D, bbar=False, eps=0.0):
    """Small-strain brick stiffness, 2x2x2 Gauss (dofs u1..u8, v1..v8,
    w1..w8; strains xx, yy, zz, gxy, gyz, gxz), optionally mean-dilatation."""
    gps = _brick_gradients(X)
    v = sum(G * dj for G, dj in gps) / sum(dj for _, dj in gps)
    beta = (1.0 - eps) / 3.0
    K = np.zeros((24, 24))
    for G, dj in gps:
        B = np.zeros((6, 24))
        B[0, 0:8] = G[0]; B[1, 8:16] = G[1]; B[2, 16:24] = G[2]
        B[3, 0:8] = G[1]; B[3, 8:16] = G[0]
        B[4, 8:16] = G[2]; B[4, 16:24] = G[1]
        B[5, 0:8] = G[2]; B[5, 16:24] = G[0]
        if bbar:
            h = beta * (v - G)                       # (3, 8)
            for d in range(3):
                B[0:3, 8 * d:8 * (d + 1)] += h[d]
        K += B.T @ D @ B * dj
    return K


def _unpack(ke, n=24):
    K = np.zeros((n, n))
    iu = np.triu_indices(n)
    order = np.lexsort((iu[0], iu[1]))            # column-packed upper triangle
    K[iu[0][order], iu[1][order]] = ke
    return K + np.triu(K, 1).T


def _run(model, du, step=1, it=1, u=None):
    ora = oracle.Oracle(model)
    u = np.zeros(model.nodof) if u is None else u
    ifv = np.zeros(model.nodof)
    st, info = ora.recover(step, it, False, model.c, u, du, ifv)
    return ora, st, ifv


@pytest.mark.parametrize("geonl", [True, False])
@pytest.mark.parametrize("jitter,eps", [(0.0, 0.0), (0.25, 0.0), (0.25, 0.3)])
def test_bbar_brick_stiffness_matches_textbook(geonl, jitter, eps):
    coords, incid = cube_mesh(1, h=2.0)
    if jitter:
        coords = coords + np.random.default_rng(3).uniform(-jitter, jitter, coords.shape)
    model = Model(coords, incid, geonl=geonl, bbar=True, eps_bbar=eps)
    ora, st, _ = _run(model, np.zeros(model.nodof), it=0)
    assert st == 0
    est = model.estiff_blocks()
    ora.tanstf(1, 0, model.c, np.zeros(model.nodof), np.zeros(model.nodof), est)
    p = model.props[0]
    D = _elastic_D(float(p[6]), float(p[7]))
    K = _unpack(est[0][0])
    X = coords[incid[0]]
    assert rel_err(K, _textbook_brick_K(X, D, bbar=True, eps=eps)) < 1e-13
    # and differs from the displacement brick by the volumetric correction
    assert rel_err(K, _textbook_brick_K(X, D)) > 1e-3


@pytest.mark.parametrize("geonl", [True, False])
def test_bbar_uniform_strain_matches_plain_brick(geonl):
    n = 3
    A = np.array([[1.0, 0.3, -0.2], [0.1, -0.5, 0.4], [0.25, 0.2, 0.7]]) * 1e-4
    out = {}
    for bbar in (False, True):
        model, _ = make_model(n=n, jitter=0.12, seed=11, geonl=geonl, bbar=bbar)
        du = (A @ model.coords.T).T.ravel()
        ora, st, ifv = _run(model, du)
        assert st == 0
        s = ora.state
        out[bbar] = (np.concatenate(s.eps_n1), np.concatenate(s.urcs_n1), ifv)
    for k in range(3):
        assert rel_err(out[True][k], out[False][k]) < 1e-12


def test_bbar_changes_an_inhomogeneous_increment():
    # small displacement: eps = B-bar du with no rotation, so the
    # volumetric strain is the element's mean dilatation at every point
    out = {}
    for bbar in (False, True):
        model, _ = make_model(n=2, jitter=0.1, seed=4, bbar=bbar, geonl=False)
        du = np.random.default_rng(8).normal(0.0, 1e-4, model.nodof)
        ora, st, ifv = _run(model, du)
        assert st == 0
        eps = np.concatenate(ora.state.eps_n1)
        out[bbar] = eps
        if bbar:   # mean dilatation: one volumetric strain per element
            tr = eps[..., 0] + eps[..., 1] + eps[..., 2]
            assert rel_err(tr, np.broadcast_to(tr.mean(axis=1, keepdims=True), tr.shape)) < 1e-12
    assert rel_err(out[True], out[False]) > 1e-2


def test_small_strain_tangent_is_the_undeformed_brick():
    coords, incid = cube_mesh(1, h=2.0)
    coords = coords + np.random.default_rng(5).uniform(-0.2, 0.2, coords.shape)
    X = coords[incid[0]]
    du = np.random.default_rng(6).normal(0.0, 2e-5, 24)      # elastic
    for bbar in (False, True):
        model = Model(coords, incid, geonl=False, bbar=bbar)
        ora, st, _ = _run(model, du)
        assert st == 0
        est = model.estiff_blocks()
        ora.tanstf(1, 1, model.c, np.zeros(model.nodof), du, est)
        p = model.props[0]
        K = _unpack(est[0][0])
        assert rel_err(K, _textbook_brick_K(X, _elastic_D(float(p[6]), float(p[7])), bbar=bbar)) < 1e-13
        # small displacement: no rotation is stored (rplstr writes R only
        # for geonl blocks)
        assert np.array_equal(np.concatenate(ora.state.rot_n1), np.concatenate(model.new_state().rot_n1))


@pytest.mark.parametrize("etype", [abi.ETYPE_L3DISOP, abi.ETYPE_Q3DISOP, abi.ETYPE_TET10])
def test_small_strain_uniaxial_closed_form(etype):
    n = 3 if etype == abi.ETYPE_L3DISOP else 2
    mat = Bilinear.from_hprime(200000.0, 0.3, 400.0, 2000.0, beta=1.0)
    model, nxyz = make_model(n=n, jitter=0.0, materials=[mat], etype=etype, geonl=False,
                             bbar=etype == abi.ETYPE_L3DISOP)
    ora = oracle.Oracle(model)
    fixed, topz = uniaxial_bcs(model, nxyz)
    drv = NewtonDriver(model, ora, fixed, tol=1e-9)
    p = model.props[0]
    E = float(p[6]); sy = float(p[22]); H = float(p[14])
    Et = E * H / (E + H)
    nsteps = 8
    for s in range(1, nsteps + 1):
        imp = np.zeros(model.nodof)
        imp[topz] = 0.01 * n / nsteps
        drv.step(s, imp)
        st = ora.state
        e = 0.01 * s / nsteps
        ezz = np.concatenate(st.eps_n)[:, :, 2]
        szz = np.concatenate(st.urcs_n)[:, :, 2]
        assert rel_err(ezz, np.full_like(ezz, e)) < 1e-8
        ref = E * e if E * e <= sy else sy + Et * (e - sy / E)
        assert rel_err(szz, np.full_like(szz, ref)) < 1e-8
        assert np.max(np.abs(np.concatenate(st.urcs_n)[:, :, [0, 1, 3, 4, 5]])) < 1e-7 * sy


@pytest.mark.parametrize("bbar", [False, True])
def test_crystal_small_displacement_elastic_limit(bbar):
    # mm10 on small-displacement blocks: identity rotations
    # (drive_10_update, rstgp1.f:4415-4432), the increment B du; a small
    # elastic increment gives sigma = C eps with the stored tangent C
    coords, incid = cube_mesh(2, jitter=0.05)
    model = Model(coords, incid, materials=[Crystal()], angles=random_orientations(8, 3), geonl=False, bbar=bbar)
    ora = oracle.Oracle(model)
    du = np.random.default_rng(5).normal(0.0, 1e-7, model.nodof)
    st, _ = ora.recover(1, 1, False, model.c, np.zeros(model.nodof), du, np.zeros(model.nodof))
    assert st == 0
    s1 = ora.state
    eps = np.concatenate(s1.eps_n1).reshape(-1, 6)
    sig = np.concatenate(s1.urcs_n1)[..., :6].reshape(-1, 6)
    C = np.concatenate(s1.history1)[..., :36].reshape(-1, 6, 6)   # column-major -> C^T
    pred = np.einsum("gji,gj->gi", C, eps)
    assert rel_err(sig, pred) < 1e-6
    assert np.array_equal(np.concatenate(s1.rot_n1), np.concatenate(model.new_state().rot_n1))


def test_crystal_bbar_brick_runs_and_keeps_rigid_modes():
    # mm10 blocks with b-bar: the b-bar strain increment, forces and
    # tangent (WARP3D's F-bar scaling of F is read by UMATs only)
    coords, incid = cube_mesh(2, jitter=0.05)
    model = Model(coords, incid, materials=[Crystal()], angles=random_orientations(8, 3), bbar=True)
    ora = oracle.Oracle(model)
    du = np.random.default_rng(2).normal(0.0, 1e-4, model.nodof)
    st, _ = ora.recover(1, 1, False, model.c, np.zeros(model.nodof), du, np.zeros(model.nodof))
    assert st == 0
    est = model.estiff_blocks()
    assert ora.tanstf(1, 1, model.c, np.zeros(model.nodof), du, est) == 0
    for e in range(model.noelem):
        K = _unpack(est[0][e])
        for d in range(3):
            r = np.zeros((3, 8)); r[d] = 1.0
            assert np.max(np.abs(K @ r.ravel())) < 1e-10 * np.max(np.abs(K))


# ---- asymmetric assembly ("assembly asymmetric on") -----------------------
def _full(v, n):
    return v.reshape(n, n).T      # column-major (totdof**2) -> K[row, col]


@pytest.mark.parametrize("etype", [abi.ETYPE_L3DISOP, abi.ETYPE_Q3DISOP, abi.ETYPE_TET10])
def test_asymmetric_assembly_of_a_symmetric_material_is_the_full_symmetric_matrix(etype):
    out = {}
    for asym in (False, True):
        model, nxyz = make_model(n=2, jitter=0.1, etype=etype, asymmetric=asym, bbar=etype == abi.ETYPE_L3DISOP)
        du = np.random.default_rng(3).normal(0.0, 1e-3, model.nodof)
        ora, st, _ = _run(model, du)
        assert st == 0
        est = model.estiff_blocks()
        assert ora.tanstf(1, 1, model.c, np.zeros(model.nodof), du, est) == 0
        out[asym] = (model, est[0])
    (m0, packed), (m1, full) = out[False], out[True]
    n = m0.totdof
    assert full.shape == (m1.noelem, n * n)
    for e in range(m0.noelem):
        K = _full(full[e], n)
        assert rel_err(K, _unpack(packed[e], n)) < 1e-14


def test_asymmetric_assembly_keeps_the_crystal_tangent_unsymmetric():
    coords, incid = cube_mesh(2, jitter=0.05)
    res = {}
    for asym in (False, True):
        model = Model(coords, incid, materials=[Crystal()], angles=random_orientations(8, 3), asymmetric=asym)
        ora = oracle.Oracle(model)
        du = np.zeros(model.nodof)
        top = np.isclose(model.coords[:, 2], 2.0)
        du[3 * np.nonzero(top)[0] + 2] = 0.004                 # plastic in one increment
        st, _ = ora.recover(1, 1, True, model.c, np.zeros(model.nodof), du, np.zeros(model.nodof))
        assert st == 0
        est = model.estiff_blocks()
        assert ora.tanstf(1, 1, model.c, np.zeros(model.nodof), du, est) == 0
        res[asym] = (ora.state, est[0], model)
    (s0, k0, m0), (s1, k1, m1) = res[False], res[True]
    # the update is the same; only the stored tangent (history 1-36) differs
    assert np.array_equal(np.concatenate(s0.urcs_n1), np.concatenate(s1.urcs_n1))
    h0, h1 = np.concatenate(s0.history1), np.concatenate(s1.history1)
    assert np.array_equal(h0[..., 36:], h1[..., 36:])
    D1 = h1[..., :36].reshape(-1, 6, 6)
    assert np.max(np.abs(D1 - np.swapaxes(D1, 1, 2))) > 1e-8 * np.max(np.abs(D1))
    assert np.allclose(0.5 * (D1 + np.swapaxes(D1, 1, 2)), h0[..., :36].reshape(-1, 6, 6), rtol=0, atol=1e-9 * np.max(np.abs(D1)))
    asym = []
    for e in range(m1.noelem):
        K = _full(k1[e], 24)
        asym.append(np.max(np.abs(K - K.T)) / np.max(np.abs(K)))
        for d in range(3):                                   # rigid translations, both sides
            r = np.zeros((3, 8)); r[d] = 1.0
            assert np.max(np.abs(K @ r.ravel())) < 1e-10 * np.max(np.abs(K))
            assert np.max(np.abs(r.ravel() @ K)) < 1e-10 * np.max(np.abs(K))
    assert max(asym) > 1e-8            # the plastic points' tangents are not symmetric
