"""A small host Newton driver around the element-block engine.

WARP3D keeps its own driver (mnralg, src/mnralg.f:20) and sparse solver;
this module restates the part of that loop the element-block path sees,
so that the engine can be exercised end to end on synthetic problems:

  iteration 0  du = imposed increments on constrained dofs (zero or the
               extrapolated previous increment elsewhere), recovery with
               iter = 0, tangent (mnralg.f:249-402)
  iteration i  solve K d = r on the free dofs, du += d, recovery with
               iter = i, residual test, new tangent (mnralg.f:435-569)
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
        r, c = upper_pairs(model.totdof)
        ed = np.concatenate(model.edest).astype(np.int64) - 1          # (noelem, totdof)
        gi = ed[:, r]
        gj = ed[:, c]
        off = r != c
        self.I = np.concatenate([gi.ravel(), gj[:, off].ravel()])
        self.J = np.concatenate([gj.ravel(), gi[:, off].ravel()])
        self.off = off
        n = model.nodof
        coo = sp.coo_matrix((np.ones(len(self.I)), (self.I, self.J)), shape=(n, n)).tocsr()
        coo.sum_duplicates()
        self.pattern = coo

    def assemble(self, estiff_elem: np.ndarray) -> sp.csr_matrix:
        """estiff_elem: (noelem, utsz) element matrices."""
        v = np.concatenate([estiff_elem.ravel(), estiff_elem[:, self.off].ravel()])
        n = self.model.nodof
        K = sp.coo_matrix((v, (self.I, self.J)), shape=(n, n)).tocsr()
        K.sum_duplicates()
        return K


class NewtonDriver:
    def __init__(self, model, engine, fixed: np.ndarray, tol: float = 1e-8, maxit: int = 25,
                 extrapolate: bool = False):
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
        self.history = []   # (step, iterations, residual list)

    def _tangent(self, step, it, du):
        self.engine.tanstf(step, it, self.model.c, self.u, du, self.estiff)
        return self.asm.assemble(np.concatenate(self.estiff))

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
        res_hist = []
        for it in range(1, self.maxit + 1):
            r = -self.ifv[self.free]
            Kff = K[self.free][:, self.free].tocsc()
            d = spla.spsolve(Kff, r)
            du[self.free] += d
            st, _ = self.engine.recover(step, it, extrap, m.c, self.u, du, self.ifv)
            if st != 0:
                raise RuntimeError(f"step {step}: step cut requested at iteration {it}")
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
        return res_hist


def uniaxial_bcs(model, n_xyz, h: float = 1.0):
    """Bottom face (z = 0) fixed in z, top face (z = nz h) loaded in z;
    minimal in-plane supports: node (0,0,0) fixed in x and y, node
    (nx,0,0) fixed in y. Returns (fixed dofs, top-face z dofs)."""
    nx, ny, nz = n_xyz
    nid = lambda i, j, k: i + (nx + 1) * (j + (ny + 1) * k)
    ii, jj = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), indexing="ij")
    bottom = nid(ii, jj, 0).ravel()
    top = nid(ii, jj, nz).ravel()
    fixed = set((3 * bottom + 2).tolist())
    fixed.update([3 * nid(0, 0, 0), 3 * nid(0, 0, 0) + 1, 3 * nid(nx, 0, 0) + 1])
    top_z = 3 * top + 2
    fixed.update(top_z.tolist())
    return np.array(sorted(fixed)), top_z
