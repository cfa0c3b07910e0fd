"""WARP3D's regression problem verification/test82/voche_model replayed
through an element engine (the oracle or the GPU engine): mm10 crystal
plasticity (one bcc crystal of fixed orientation per Gauss point, Voce
hardening) on 208 small-displacement b-bar 8-node bricks of the unit
cube, symmetry planes x = y = z = 0, element face pressures in steps of
50, the checker's answer read after step 8. Data and answer from
tests/golden/warp3d_test82_voce.npz (make_warp3d_test82_voce.py).

Face pressures become nodal forces as WARP3D's element loads do for a
flat 4-node face (hex_face_nloads / face_load, elem_load_b.f:425-560,
elem_load_c.f:141-272): the face nodes of eqelfn (elem_load_c.f:886-891),
positive pressure along the inward normal, and for these flat square
faces the consistent share of each node, p A / 4. Each step is converged
to 1e-8 (the deck asks ||R|| <= 1e-4 ||F||, cvtest.f:158-181); the tangent
is assembled symmetric (the deck's asymmetric assembly changes only the
Newton path). The checked value is element 64's center_output row, the
stresses of its Gauss points averaged (small displacement: no rotation),
sigma_xx first."""
from __future__ import annotations

import os

import numpy as np
import scipy.sparse.linalg as spla

from tests import warp3d_test24 as t24
from warp3d_gb300.model import Crystal, Model
from warp3d_gb300.newton import Assembler

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "warp3d_test82_voce.npz")
CHECKER_RTOL = 1e-4

# 8-node brick faces, element-local nodes 1..8 (eqelfn f8nod)
HEX8_FACES = ((4, 3, 2, 1), (5, 6, 7, 8), (1, 2, 6, 5), (3, 4, 8, 7), (2, 3, 7, 6), (4, 1, 5, 8))


def load():
    return dict(np.load(FIXTURE))


def build_model(d):
    e, nu, n, m, theta0, tau_y, tau_v = (float(x) for x in d["crystal"])
    xtal = Crystal(e=e, nu=nu, harden_n=n, voche_m=m, theta_o=theta0, tau_y=tau_y, tau_v=tau_v, slip_type=2)
    geonl, bbar, _ = (bool(x) for x in d["flags"])
    ne = d["incid"].shape[0]
    return Model(d["coords"], d["incid"], materials=[xtal], angles=np.tile(d["angles"], (ne, 1)),
                 dt=float(d["dt"]), geonl=geonl, bbar=bbar)


def load_pattern(d):
    """Nodal forces of the face pressures at unit step factor."""
    xyz, inc = d["coords"], d["incid"]
    F = np.zeros_like(xyz)
    for elem, face, p in d["face_loads"]:
        nodes = inc[int(elem), [k - 1 for k in HEX8_FACES[int(face) - 1]]]
        P = xyz[nodes]
        cr = np.cross(P[2] - P[0], P[3] - P[1])
        area = 0.5 * np.linalg.norm(cr)
        n_out = cr / np.linalg.norm(cr)
        if np.dot(n_out, P.mean(axis=0) - xyz[inc[int(elem)]].mean(axis=0)) < 0.0:
            n_out = -n_out
        F[nodes] += -p * n_out * area / 4.0
    return F.ravel()


def solve(engine_cls, d=None, tol=1e-8, maxit=30):
    """Runs the deck's steps up to the checked one with engine_cls(model).
    Returns (element 64's center stresses, displacements, Newton
    iterations per step)."""
    d = load() if d is None else d
    model = build_model(d)
    eng = engine_cls(model)
    asm = Assembler(model)
    free = np.setdiff1d(np.arange(model.nodof), d["plane_fixed_dofs"])
    pattern = load_pattern(d)
    u = np.zeros(model.nodof)
    F = np.zeros(model.nodof)
    ifv = np.zeros(model.nodof)
    est = model.estiff_blocks()
    its = []
    for step in range(1, int(d["last_step"]) + 1):
        F += d["step_factors"][step - 1] * pattern
        du = np.zeros(model.nodof)
        st, _ = eng.recover(step, 0, False, model.c, u, du, ifv)
        assert st == 0, f"step {step}: recovery status {st}"
        eng.tanstf(step, 0, model.c, u, du, est)
        fnorm = np.linalg.norm(F[free])
        for it in range(1, maxit + 1):
            K = asm.assemble(est)
            r = (F - ifv)[free]
            du[free] += spla.spsolve(K[free][:, free].tocsc(), r)
            st, _ = eng.recover(step, it, False, model.c, u, du, ifv)
            assert st == 0, f"step {step}: recovery status {st} at iteration {it}"
            if np.linalg.norm((F - ifv)[free]) <= tol * fnorm:
                break
            eng.tanstf(step, it, model.c, u, du, est)
        else:
            raise RuntimeError(f"step {step}: no convergence in {maxit} iterations")
        its.append(it)
        eng.update()
        u += du
    return t24.center_stress(eng, model, element=int(d["expected_element"])), u, its
