"""A small host Newton driver around the element-block engine.

WARP3D keeps its own driver (mnralg, src/mnralg.f:20) and sparse solver;
this module restates the part of that loop the element-block path sees,
so that the engine can be exercised end to end on synthetic problems:

  iteration 0  du = imposed increments on constrained dofs (zero or the
               extrapolated previous increment elsewhere), recovery with
               iter = 0, tangent (mnralg.f:249-402)
  iteration i  solve K d = r on the free dofs, du += d, recovery with
               iter = i, residual test, new tangent (mnralg.f:435-569);
               with line search, du = du0 + alpha d with alpha from
               mnralg_ls (mnralg.f:758-914)
  converged    update n+1 -> n, u += du (update.f:73-94)

Displacement-controlled problems only (no applied loads): the residual on
the free dofs is -ifv. Convergence: ||r_free|| <= tol * ||ifv|| (2-norms).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def upper_pairs(totdof: int):
    """(row, col) of the column-packed upper triangle, pos = c(c+1)/2 + r."""
    rows, cols = [], []
    for c in range(totdof):
        for r in range(c + 1):
            rows.append(r)
            cols.append(c)
    return np.array(rows), np.array(cols)


class Assembler:
    """Global sparse stiffness from blocked element matrices (the role of
    drive_assemble_solve, src/drive_assemble_solve.f:11)."""

    def __init__(self, model):
        self.model = model
        self.full = bool(getattr(model, "asymmetric", False))
        I, J, self.off = [], [], []
        pairs = {}
        for b in range(model.nelblk):
            td = model.block_totdof[b]
            ed = model.edest[b].astype(np.int64) - 1          # (span, totdof)
            if self.full:   # column-major full matrices: entry c*totdof + r is (r, c)
                c, r = np.divmod(np.arange(td * td), td)
                I.append(ed[:, r].ravel())
                J.append(ed[:, c].ravel())
                self.off.append(None)
                continue
            if td not in pairs:
                pairs[td] = upper_pairs(td)
            r, c = pairs[td]
            gi, gj = ed[:, r], ed[:, c]
            off = r != c
            I += [gi.ravel(), gj[:, off].ravel()]
            J += [gj.ravel(), gi[:, off].ravel()]
            self.off.append(off)
        self.I = np.concatenate(I)
        self.J = np.concatenate(J)

    def assemble(self, estiff_blocks) -> sp.csr_matrix:
        """estiff_blocks: per block (span, utsz) packed element matrices, or
        (span, totdof**2) full ones with asymmetric assembly."""
        v = []
        for est, off in zip(estiff_blocks, self.off):
            v += [est.ravel()] if off is None else [est.ravel(), est[:, off].ravel()]
        n = self.model.nodof
        K = sp.coo_matrix((np.concatenate(v), (self.I, self.J)), shape=(n, n)).tocsr()
        K.sum_duplicates()
        return K


# line-search defaults of WARP3D's input (indypm.f:1278-1283) and the
# r-reduction fraction of mnralg_ls (mnralg.f:802)
LS_RHO, LS_SLACK_TOL, LS_MIN_STEP, LS_MAX_STEP, LS_REDUCE = 0.7, 0.5, 0.01, 1.0, 0.9


def line_search(s0: float, trial, rho: float = LS_RHO, slack_tol: float = LS_SLACK_TOL,
                alpha_min: float = LS_MIN_STEP, alpha_max: float = LS_MAX_STEP, reduce: float = LS_REDUCE):
    """The step-length search of mnralg_ls (src/mnralg.f:758-914) for a
    Newton correction idu with s0 = -res.idu < 0 over the free dofs.
    trial(alpha) sets du = du0 + alpha idu, recomputes the internal forces
    (mnralg_ls_update_res) and returns s(alpha); the search backtracks
    alpha = rho alpha from alpha_max until |s / s0| < slack_tol, and falls
    back to alpha = 1 (recomputing there) when the ratio stops falling by
    `reduce` or alpha drops below alpha_min. Returns (alpha, trials)."""
    alpha, ell, r_prev = alpha_max, 1, None
    while True:
        r = abs(trial(alpha) / s0)
        if r < slack_tol:
            return alpha, ell
        if ell >= 2 and r > reduce * r_prev:     # ratio not decreasing: full step
            trial(1.0)
            return 1.0, ell + 1
        r_prev = r
        alpha = rho * alpha                      # simple backtrack
        if alpha < alpha_min:
            trial(1.0)
            return 1.0, ell + 1
        ell += 1


class NewtonDriver:
    def __init__(self, model, engine, fixed: np.ndarray, tol: float = 1e-8, maxit: int = 25,
                 extrapolate: bool = False, line_search: bool = False):
        self.model = model
        self.engine = engine
        self.fixed = np.asarray(fixed, dtype=np.int64)
        self.free = np.setdiff1d(np.arange(model.nodof), self.fixed)
        self.tol = tol
        self.maxit = maxit
        self.extrapolate = extrapolate
        self.asm = Assembler(model)
        self.u = np.zeros(model.nodof)
        self.du_prev = None
        self.ifv = np.zeros(model.nodof)
        self.estiff = model.estiff_blocks()
        self.line_search = line_search
        self.history = []   # (step, iterations, residual list)
        self.alphas = []    # (step, [accepted step length per iteration]) with line search

    def _tangent(self, step, it, du):
        self.engine.tanstf(step, it, self.model.c, self.u, du, self.estiff)
        return self.asm.assemble(self.estiff)

    def step(self, step: int, imposed: np.ndarray):
        """imposed: full-length vector; its values on fixed dofs are the
        displacement increments of this step."""
        m = self.model
        extrap = self.extrapolate and self.du_prev is not None and step > 1
        du = self.du_prev.copy() if extrap else np.zeros(m.nodof)
        du[self.fixed] = imposed[self.fixed]
        st, _ = self.engine.recover(step, 0, extrap, m.c, self.u, du, self.ifv)
        if st != 0:
            raise RuntimeError(f"step {step}: recovery requested a step cut at iteration 0")
        K = self._tangent(step, 0, du)
        res_hist, alphas = [], []
        for it in range(1, self.maxit + 1):
            r = -self.ifv[self.free]
            Kff = K[self.free][:, self.free].tocsc()
            d = spla.spsolve(Kff, r)

            def trial(alpha, du0=du.copy(), it=it):
                du[:] = du0
                du[self.free] += alpha * d if alpha != 1.0 else d
                st, _ = self.engine.recover(step, it, extrap, m.c, self.u, du, self.ifv)
                if st != 0:
                    raise RuntimeError(f"step {step}: step cut requested at iteration {it}")
                return float(np.dot(self.ifv[self.free], d))   # s = -res.idu, res = -ifv

            # mnralg_ls: s0 from the residual the correction was solved for;
            # s0 >= 0 (or no line search) takes the full step
            s0 = float(np.dot(self.ifv[self.free], d))
            if self.line_search and s0 < 0.0:
                alpha, _ = line_search(s0, trial)
            else:
                alpha = 1.0
                trial(1.0)
            alphas.append(alpha)
            rn = np.linalg.norm(self.ifv[self.free])
            scale = max(np.linalg.norm(self.ifv), 1e-300)
            res_hist.append(rn / scale)
            if rn <= self.tol * scale:
                break
            K = self._tangent(step, it, du)
        else:
            raise RuntimeError(f"step {step}: no convergence in {self.maxit} iterations: {res_hist}")
        self.engine.update()
        self.u += du
        self.du_prev = du
        self.history.append((step, len(res_hist), res_hist))
        self.alphas.append((step, alphas))
        return res_hist


def uniaxial_bcs(model, n_xyz, h: float = 1.0, origins=None):
    """Bottom face (z = 0) fixed in z, top face (z = nz h) loaded in z;
    minimal in-plane supports: the node at (0,0,0) fixed in x and y, the
    node at (nx h, 0, 0) fixed in y. Faces are found from the (unjittered)
    boundary coordinates, so any element type works. ``origins`` lists
    (x0, nx) per bar of a several-bar model (mixed_mesh), each bar getting
    its own in-plane supports. Returns (fixed dofs, top-face z dofs)."""
    nx, ny, nz = n_xyz
    X = model.coords
    tol = 1e-9 * h
    bottom = np.nonzero(np.abs(X[:, 2]) < tol)[0]
    top = np.nonzero(np.abs(X[:, 2] - nz * h) < tol)[0]
    fixed = set((3 * bottom + 2).tolist())
    for x0, bnx in (origins or [(0.0, nx)]):
        o = np.nonzero(np.linalg.norm(X - np.array([x0, 0.0, 0.0]), axis=1) < tol)[0][0]
        xe = np.nonzero(np.linalg.norm(X - np.array([x0 + bnx * h, 0.0, 0.0]), axis=1) < tol)[0][0]
        fixed.update([3 * o, 3 * o + 1, 3 * xe + 1])
    top_z = 3 * top + 2
    fixed.update(top_z.tolist())
    return np.array(sorted(fixed)), top_z
