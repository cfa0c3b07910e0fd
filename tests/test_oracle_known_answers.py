"""Pins the oracle (CPU restatement of the reference path) to closed-form
known answers. WARP3D's own tests are end-to-end input decks without
element-level vectors, so these checks stand in for golden vectors:
element library identities, the textbook elastic brick stiffness, rigid
body modes, incremental objectivity under finite rotation, the uniform
strain patch test, the analytic bilinear uniaxial response and the
consistent tangent against finite differences of the stress update.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from warp3d_gb300 import abi
from warp3d_gb300.model import HEX8_NODES, Bilinear, Model, cube_mesh, cube_mesh_hex20, cube_mesh_tet10

MESHES = {abi.ETYPE_L3DISOP: cube_mesh, abi.ETYPE_Q3DISOP: cube_mesh_hex20, abi.ETYPE_TET10: cube_mesh_tet10}
ETYPES = [abi.ETYPE_L3DISOP, abi.ETYPE_Q3DISOP, abi.ETYPE_TET10]


def _mesh_model(etype, n, jitter=0.0, seed=12345, **kw):
    coords, incid = MESHES[etype](n, jitter=jitter, seed=seed)
    return Model(coords, incid, etype=etype, **kw), coords, incid
from warp3d_gb300.newton import NewtonDriver, uniaxial_bcs
from tests.conftest import rel_err


def _gp_and_derivs():
    lib = oracle.load()
    out = []
    for g in range(1, 9):
        xyzw = np.zeros(4)
        assert lib.w3o_gauss_point(abi.ETYPE_L3DISOP, 1, g, xyzw.ctypes.data_as(C.POINTER(C.c_double))) == 0
        d = [np.zeros(8) for _ in range(3)]
        assert lib.w3o_shape_derivs(abi.ETYPE_L3DISOP, *xyzw[:3], *[a.ctypes.data_as(C.POINTER(C.c_double)) for a in d]) == 0
        out.append((xyzw, np.stack(d)))
    return out


def test_hex8_gauss_rule_and_shape_derivatives():
    pts = _gp_and_derivs()
    assert sum(p[0][3] for p in pts) == 8.0
    for xyzw, dn in pts:
        xi = xyzw[:3]
        assert np.allclose(np.abs(xi), 0.5773502691896257645, rtol=0, atol=0)
        np.testing.assert_allclose(dn.sum(axis=1), 0.0, atol=1e-16)
        # derivatives of N_a = (1+xi xi_a)(1+eta eta_a)(1+zeta zeta_a)/8
        for a, s in enumerate(HEX8_NODES):
            f = 1 + s * xi
            ref = np.array([s[0] * f[1] * f[2], f[0] * s[1] * f[2], f[0] * f[1] * s[2]]) / 8.0
            np.testing.assert_allclose(dn[:, a], ref, rtol=1e-15, atol=1e-16)


def _single_state(model, du, step=1, it=1):
    ora = oracle.Oracle(model)
    c, u = model.c, np.zeros(model.nodof)
    ifv = np.zeros(model.nodof)
    st, info = ora.recover(step, it, False, c, u, du, ifv)
    return ora, st, info, ifv


def _textbook_hex8_K(X, E, nu):
    """Small-strain 8-node brick stiffness with 2x2x2 Gauss, written
    independently of the oracle (dofs u1..u8, v1..v8, w1..w8; strains
    xx, yy, zz, gxy, gyz, gxz)."""
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    mu = E / (2 * (1 + nu))
    D = np.zeros((6, 6))
    D[:3, :3] = lam
    D[np.arange(3), np.arange(3)] += 2 * mu
    D[3, 3] = D[4, 4] = D[5, 5] = mu
    g = 1 / np.sqrt(3.0)
    K = np.zeros((24, 24))
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
                G = np.linalg.solve(J, dN)
                B = np.zeros((6, 24))
                B[0, 0:8] = G[0]; B[1, 8:16] = G[1]; B[2, 16:24] = G[2]
                B[3, 0:8] = G[1]; B[3, 8:16] = G[0]
                B[4, 8:16] = G[2]; B[4, 16:24] = G[1]
                B[5, 0:8] = G[2]; B[5, 16:24] = G[0]
                K += B.T @ D @ B * np.linalg.det(J)
    return K


def _unpack(ke, n=24):
    K = np.zeros((n, n))
    pos = 0
    for c in range(n):
        for r in range(c + 1):
            K[r, c] = K[c, r] = ke[pos]
            pos += 1
    return K


@pytest.mark.parametrize("jitter", [0.0, 0.2])
def test_elastic_tangent_matches_textbook_brick(jitter):
    coords, incid = cube_mesh(1, h=2.0)
    if jitter:
        rng = np.random.default_rng(3)
        coords = coords + rng.uniform(-jitter, jitter, coords.shape)
    model = Model(coords, incid)
    ora, st, _, _ = _single_state(model, np.zeros(model.nodof), step=1, it=0)
    assert st == 0
    est = model.estiff_blocks()
    ora.tanstf(1, 0, model.c, np.zeros(model.nodof), np.zeros(model.nodof), est)
    K = _unpack(est[0][0])
    p = model.props[0]
    X = coords[incid[0]]
    Kref = _textbook_hex8_K(X, float(p[6]), float(p[7]))
    assert rel_err(K, Kref) < 1e-13


@pytest.mark.parametrize("etype", ETYPES)
def test_tangent_rigid_body_modes_vanish(etype):
    model, coords, incid = _mesh_model(etype, 2, jitter=0.15, seed=5)
    nn = incid.shape[1]
    ora, st, _, _ = _single_state(model, np.zeros(model.nodof), step=1, it=0)
    est = model.estiff_blocks()
    ora.tanstf(1, 0, model.c, np.zeros(model.nodof), np.zeros(model.nodof), est)
    assert np.max(np.abs(est[0])) > 0
    for e in range(model.noelem):
        K = _unpack(est[0][e], 3 * nn)
        X = coords[incid[e]]
        modes = []
        for d in range(3):
            r = np.zeros((3, nn)); r[d] = 1.0; modes.append(r.ravel())
        for ax in np.eye(3):
            r = np.cross(ax, X).T      # (3, 8)
            modes.append(r.ravel())
        for r in modes:
            assert np.max(np.abs(K @ r)) < 1e-12 * np.max(np.abs(K)) * np.max(np.abs(r))


@pytest.mark.parametrize("etype", ETYPES)
def test_finite_rigid_rotation_is_stress_free(etype):
    model, coords, incid = _mesh_model(etype, 2, jitter=0.1, seed=9)
    th = np.deg2rad(35.0)
    ax = np.array([1.0, 2.0, 2.0]) / 3.0
    Kx = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]])
    R = np.eye(3) + np.sin(th) * Kx + (1 - np.cos(th)) * Kx @ Kx
    du = ((R - np.eye(3)) @ coords.T).T.ravel()
    ora, st, info, ifv = _single_state(model, du, step=1, it=1)
    assert st == 0
    s = ora.state
    sig = np.concatenate(s.urcs_n1)[:, :, :6]
    assert np.max(np.abs(sig)) < 1e-9 * 200000.0
    rot = np.concatenate(s.rot_n1).reshape(-1, 3, 3, order="C")
    # rot_n1 (9) is column-major 3x3
    rot = np.swapaxes(rot, 1, 2)
    assert np.max(np.abs(rot - R)) < 1e-13
    assert np.max(np.abs(ifv)) < 1e-9 * 200000.0


@pytest.mark.parametrize("etype", ETYPES)
def test_uniform_strain_patch_test(etype):
    n = 3
    model, coords, incid = _mesh_model(etype, n, jitter=0.12, seed=11)
    A = np.array([[1.0, 0.3, -0.2], [0.1, -0.5, 0.4], [0.25, 0.2, 0.7]]) * 1e-4
    du = (A @ coords.T).T.ravel()
    ora, st, info, ifv = _single_state(model, du, step=1, it=1)
    assert st == 0
    s = ora.state
    eps = np.concatenate(s.eps_n1).reshape(-1, 6)
    sig = np.concatenate(s.urcs_n1)[:, :, :6].reshape(-1, 6)
    assert rel_err(eps, np.broadcast_to(eps.mean(0), eps.shape)) < 1e-10
    assert rel_err(sig, np.broadcast_to(sig.mean(0), sig.shape)) < 1e-10
    # interior nodes carry no net internal force
    inside = np.all((coords > 1e-9) & (coords < n - 1e-9), axis=1)
    interior = np.nonzero(inside)[0]
    dofs = np.concatenate([[3 * q, 3 * q + 1, 3 * q + 2] for q in interior])
    assert np.max(np.abs(ifv[dofs])) < 1e-10 * np.max(np.abs(ifv))


@pytest.mark.parametrize("etype,beta", [(abi.ETYPE_L3DISOP, 1.0), (abi.ETYPE_L3DISOP, 0.0),
                                         (abi.ETYPE_Q3DISOP, 1.0), (abi.ETYPE_TET10, 1.0)])
def test_uniaxial_bilinear_closed_form(etype, beta):
    n = 4 if etype == abi.ETYPE_L3DISOP else 2
    mat = Bilinear.from_hprime(200000.0, 0.3, 400.0, 2000.0, beta=beta)
    model, coords, incid = _mesh_model(etype, n, materials=[mat])
    ora = oracle.Oracle(model)
    fixed, topz = uniaxial_bcs(model, (n, n, n))
    drv = NewtonDriver(model, ora, fixed, tol=1e-8)
    nsteps, total = 10, 0.01 * n
    p = model.props[0]
    E = float(p[6]); sy = float(p[22]); H = float(p[14])
    Et = E * H / (E + H)
    log_incr = 0.0
    for s in range(1, nsteps + 1):
        imp = np.zeros(model.nodof)
        imp[topz] = total / nsteps
        drv.step(s, imp)
        # midpoint rule of the axial rate of deformation: d = du / L_mid
        lam0, lam1 = 1 + 0.01 * (s - 1) / nsteps, 1 + 0.01 * s / nsteps
        log_incr += (lam1 - lam0) / (0.5 * (lam0 + lam1))
        st = ora.state
        ezz = np.concatenate(st.eps_n)[:, :, 2]
        szz = np.concatenate(st.urcs_n)[:, :, 2]
        e = ezz.mean()
        assert abs(e - log_incr) < 1e-8 * log_incr   # Newton tolerance
        ref = E * e if E * e <= sy else sy + Et * (e - sy / E)
        # mean: closed form; scatter over Gauss points: the Newton
        # tolerance and the round-off of the Cardano polar decomposition
        assert abs(szz.mean() - ref) < 1e-10 * ref
        assert rel_err(szz, np.full_like(szz, ref)) < 1e-7
        lateral = np.concatenate(st.urcs_n)[:, :, [0, 1, 3, 4, 5]]
        assert np.max(np.abs(lateral)) < 1e-7 * sy


def _mm01_fd(step, hist_n, cgn, deps, h=1e-7):
    n = 1
    e, nu, beta, hp, yld = [np.array([v]) for v in (200000.0, 0.3, 1.0, 2000.0, 400.0)]
    cgn1, hist1, hist0, cep = oracle.mm01_points(step, e, nu, beta, hp, yld, cgn[None], deps[None], hist_n[None])
    fd = np.zeros((6, 6))
    for k in range(6):
        dp = deps.copy(); dp[k] += h
        dm = deps.copy(); dm[k] -= h
        sp, *_ = oracle.mm01_points(step, e, nu, beta, hp, yld, cgn[None], dp[None], hist_n[None])
        sm, *_ = oracle.mm01_points(step, e, nu, beta, hp, yld, cgn[None], dm[None], hist_n[None])
        fd[:, k] = (sp[0, :6] - sm[0, :6]) / (2 * h)
    return cep[0], fd, hist1[0]


def test_cnst1_is_the_derivative_of_mm01():
    rng = np.random.default_rng(1)
    # a point with prior plastic history at n (state word 1 = yielding)
    hist = np.zeros(11)
    hist[1] = 420.0 / np.sqrt(3.0)
    hist[2] = 0.004
    hist[4] = 2000.0
    hist[3] = np.frombuffer(np.array([1, 0], dtype=np.int32).tobytes(), dtype=np.float64)[0]
    cgn = np.zeros(9)
    cgn[:6] = [300.0, -50.0, 100.0, 150.0, -80.0, 60.0]
    dev = cgn[:6].copy()
    dev[:3] -= dev[:3].mean()
    direction = dev * np.array([1, 1, 1, 2, 2, 2]) / np.linalg.norm(dev)   # engineering shears
    for trial in range(5):
        deps = 2e-3 * direction + rng.normal(0.0, 2e-4, 6)
        cep, fd, h1 = _mm01_fd(2, hist, cgn, deps)
        yielding = int(np.frombuffer(np.float64(h1[3]).tobytes(), dtype=np.int32)[0]) == 1
        assert yielding
        assert rel_err(cep, fd) < 2e-6
    # elastic unloading: [D] is the elastic matrix
    deps = -1e-5 * np.array([1.0, -0.3, 0.2, 0.5, -0.5, 0.1])
    cep, fd, h1 = _mm01_fd(2, hist, cgn * 0.5, deps)
    assert rel_err(cep, fd) < 1e-7


def test_inverted_element_requests_step_cut():
    coords, incid = cube_mesh(3)
    model = Model(coords, incid)
    du = np.zeros(model.nodof)
    du[3 * incid[13, 7] + 2] = -2.5      # drive a corner through its element
    ora, st, info, ifv = _single_state(model, du, step=2, it=1)
    assert st == abi.STEP_CUT and info.material_cut_step == 1
    assert info.first_bad_element >= 1
    du[3 * incid[13, 7] + 2] = -1.5      # distorted but every Gauss point det[F] > 0
    ora, st, info, ifv = _single_state(model, du, step=2, it=1)
    assert st == 0 and info.material_cut_step == 0
