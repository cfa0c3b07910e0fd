"""WARP3D's regression problem verification/test24 replayed through an
element engine (the oracle or the GPU engine): the hollow sphere under
internal pressure (45 finite-strain b-bar 8-node bricks, bilinear Mises,
constraints in nodal coordinate systems, nodal forces over 21 steps).
The deck's data and the answer WARP3D's checker expects come from
tests/golden/warp3d_test24.npz (written by make_warp3d_test24.py).

The global loop restates what WARP3D's driver does for this deck, in the
part the answer depends on: nodal coordinate systems (constraints and
loads rotated into them, eqivld.f rotate_loads :786-862, the element
vectors rotated back by the element gathers), the residual R = F - ifv on
the unconstrained local dofs, load steps of the deck's factors, each
converged (the deck asks ||R|| <= 1e-5 ||F||, cvtest.f:158-181; here to
1e-8, so that the converged state does not depend on the iterate path;
the deck's nodal rotation matrices are orthonormal to ~6e-7 and, used as
WARP3D uses them (T forward, T^T back), leave a residual floor near 1e-9).
The checked quantity is what `output stresses` prints for element 1 with
center_output: the Cauchy stresses of its Gauss points (R sigma_hat R^T
from the unrotated stresses, ougts1) averaged over the points (oumkcv),
sigma_xx first (oulbst_solid, ouhel)."""
from __future__ import annotations

import os

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from warp3d_gb300.model import Bilinear, Model
from warp3d_gb300.newton import Assembler

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "warp3d_test24.npz")
# verification/run_tests.py: |computed / expected - 1| within 1e-4
CHECKER_RTOL = 1e-4


def load():
    return dict(np.load(FIXTURE))


def build_model(d):
    e, nu, yld, tan_e = (float(x) for x in d["props"])
    geonl, bbar, _ = (bool(x) for x in d["flags"])
    return Model(d["coords"], d["incid"], materials=[Bilinear(e, nu, yld, tan_e)], geonl=geonl, bbar=bbar)


def transformation(d, nodof):
    """Q with u_local = Q u_global (identity away from the transformed
    nodes) and the local dofs held at zero: the transformed nodes'
    constrained directions and the symmetry planes' normal dofs (at the
    transformed nodes on a plane the two coincide in this deck)."""
    Q = sp.lil_matrix((nodof, nodof))
    Q.setdiag(1.0)
    fixed = set(int(x) for x in d["plane_fixed_dofs"])
    start = 0
    for mat, cnt, fx in zip(d["trn_mats"], d["trn_counts"], d["trn_fixed"]):
        for n in d["trn_node_lists"][start:start + cnt]:
            Q[3 * n:3 * n + 3, 3 * n:3 * n + 3] = mat
            fixed.update(3 * int(n) + k for k in range(3) if fx[k])
        start += cnt
    return Q.tocsr(), np.array(sorted(fixed))


def solve(engine_cls, d=None, tol=1e-8, maxit=20):
    """Runs the deck's 21 load steps with engine_cls(model) as the element
    engine. Returns (element 1's center Cauchy stresses, the final
    displacements, Newton iterations per step)."""
    d = load() if d is None else d
    model = build_model(d)
    eng = engine_cls(model)
    asm = Assembler(model)
    Q, fixed = transformation(d, model.nodof)
    free = np.setdiff1d(np.arange(model.nodof), fixed)
    pattern = d["load_pattern"].ravel()
    u = np.zeros(model.nodof)
    F = np.zeros(model.nodof)
    ifv = np.zeros(model.nodof)
    est = model.estiff_blocks()
    its = []
    for step, fac in enumerate(d["step_factors"], start=1):
        F += fac * pattern
        du = np.zeros(model.nodof)
        st, _ = eng.recover(step, 0, False, model.c, u, du, ifv)
        assert st == 0, f"step {step}: recovery status {st}"
        eng.tanstf(step, 0, model.c, u, du, est)
        fnorm = np.linalg.norm((Q @ F)[free])
        for it in range(1, maxit + 1):
            K = asm.assemble(est)
            Kl = (Q @ K @ Q.T).tocsr()
            rl = Q @ (F - ifv)
            dl = np.zeros(model.nodof)
            dl[free] = spla.spsolve(Kl[free][:, free].tocsc(), rl[free])
            du += Q.T @ dl
            st, _ = eng.recover(step, it, False, model.c, u, du, ifv)
            assert st == 0, f"step {step}: recovery status {st} at iteration {it}"
            if np.linalg.norm((Q @ (F - ifv))[free]) <= tol * fnorm:
                break
            eng.tanstf(step, it, model.c, u, du, est)
        else:
            raise RuntimeError(f"step {step}: no convergence in {maxit} iterations")
        its.append(it)
        eng.update()
        u += du
    return center_stress(eng, model, element=0), u, its


def center_stress(eng, model, element):
    """Cauchy stresses (xx yy zz xy yz xz) of `element` (0-based) averaged
    over its Gauss points, from the engine's converged state."""
    if hasattr(eng, "download"):   # the GPU engine
        state = model.new_state()
        eng.download(state)
    else:                          # the oracle keeps its host state
        state = eng.state
    b = int(np.searchsorted(model.felem, element, side="right") - 1)
    i = element - int(model.felem[b])
    sig = np.zeros((3, 3))
    ngp = state.urcs_n[b].shape[1]
    for g in range(ngp):
        s = state.urcs_n[b][i, g, :6]
        S = np.array([[s[0], s[3], s[5]], [s[3], s[1], s[4]], [s[5], s[4], s[2]]])
        R = state.rot_n1[b][i, g].reshape(3, 3, order="F")
        sig += R @ S @ R.T
    sig /= ngp
    return np.array([sig[0, 0], sig[1, 1], sig[2, 2], sig[0, 1], sig[1, 2], sig[0, 2]])
