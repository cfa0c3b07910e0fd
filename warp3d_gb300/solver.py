"""Global stiffness, its solve and the Newton loop, all on the device.

``DeviceCsr`` mirrors the assembly-and-solve step that follows the element
path in WARP3D's Newton iteration (drive_assemble_solve,
src/drive_assemble_solve.f:11): the element stiffnesses left resident by
``Engine.tanstf_dev`` are assembled into a CSR matrix on the device
(row-wise gather in a fixed order, as assem_by_row builds whole rows,
src/assemble_code.f:659) and solved by a Jacobi-preconditioned conjugate
gradient on the free dofs.

``DeviceNewtonDriver`` restates the host driver of ``newton.py`` (the loop
of mnralg, src/mnralg.f:249-569) with every vector on the device: the
element path, the assembly, the solve and the convergence norms (cvtest,
src/cvtest.f:20) run there; per iteration the host reads only the
recovery status, the solver's iteration count and two norms (and, with
the line search of mnralg_ls, one s-value per trial step length). PyTorch
provides the device vectors and the few vector updates of the driver.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import scipy.sparse as sp

from . import abi


class DeviceCsr:
    def __init__(self, engine):
        self.engine = engine
        self.lib = engine.lib
        self.h = C.c_void_p()
        abi.check(self.lib, self.lib.w3g_csr_create(engine.ctx, C.byref(self.h)))
        n, nnz = C.c_int(), C.c_longlong()
        abi.check(self.lib, self.lib.w3g_csr_info(self.h, C.byref(n), C.byref(nnz), None, None, None))
        self.n, self.nnz = n.value, nnz.value

    def close(self):
        if self.h:
            self.lib.w3g_csr_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_node_blocks(self, enable: bool) -> bool:
        """Node-block product and preconditioner (default when the pattern
        allows) or the row kernels with the diagonal preconditioner."""
        r = self.lib.w3g_csr_set_node_blocks(self.h, 1 if enable else 0)
        abi.check(self.lib, r, allow=(0, 1))
        return r == 1

    def assemble(self, stream: int = 0):
        """K from the context's current element stiffnesses (FP64, or the
        FP32 element matrices of a precision form)."""
        abi.check(self.lib, self.lib.w3g_csr_assemble_dev(self.h, stream or None))

    def to_scipy(self) -> sp.csr_matrix:
        rowptr = np.empty(self.n + 1, dtype=np.int32)
        colind = np.empty(self.nnz, dtype=np.int32)
        val = np.empty(self.nnz, dtype=np.float64)
        abi.check(self.lib, self.lib.w3g_csr_download(self.h, rowptr.ctypes.data, colind.ctypes.data,
                                                      val.ctypes.data))
        return sp.csr_matrix((val, colind, rowptr), shape=(self.n, self.n))

    def pcg(self, d_fixed: int, d_b: int, b_scale: float, d_x: int, rtol: float, maxit: int, stream: int = 0):
        """Solves K_ff x = b_scale b on the free dofs. Returns (status,
        iterations, ||r|| / ||b_f||), status 0, abi.PCG_MAXIT or
        abi.PCG_BREAKDOWN."""
        its, rel = C.c_int(), C.c_double()
        st = self.lib.w3g_pcg_dev(self.h, d_fixed, d_b, b_scale, d_x, rtol, maxit, stream or None, C.byref(its),
                                  C.byref(rel))
        abi.check(self.lib, st, allow=(abi.OK, abi.PCG_MAXIT, abi.PCG_BREAKDOWN))
        return st, its.value, rel.value

    def residual_norms(self, d_v: int, d_fixed: int, d_out: int, stream: int = 0):
        abi.check(self.lib, self.lib.w3g_residual_norms_dev(self.h, d_v, d_fixed, d_out, stream or None))

    def newton_iteration(self, step: int, it: int, extrap: bool, d_c: int, d_u: int, d_du: int, d_ifv: int,
                         d_fixed: int, d_d: int, rtol: float, maxit: int, d_norms: int, stream: int = 0):
        """One Newton iteration as one graph (w3g_newton_iteration_dev):
        solve, du += d, recovery, tangent, assembly, norms. Returns (PCG
        status, PCG iterations, relative residual, recovery status,
        ||ifv_f||^2, ||ifv||^2)."""
        its, rel, rst = C.c_int(), C.c_double(), C.c_int()
        nrm = (C.c_double * 2)()
        st = self.lib.w3g_newton_iteration_dev(self.h, step, it, 1 if extrap else 0, d_c, d_u, d_du, d_ifv, d_fixed,
                                               d_d, rtol, maxit, d_norms, stream or None, C.byref(its),
                                               C.byref(rel), C.byref(rst), nrm)
        abi.check(self.lib, st, allow=(abi.OK, abi.PCG_MAXIT, abi.PCG_BREAKDOWN))
        return st, its.value, rel.value, rst.value, nrm[0], nrm[1]

    def free_dot(self, d_a: int, d_b: int, d_fixed: int, d_out: int, stream: int = 0):
        """d_out[0] = sum over the free dofs of a_i b_i (w3g_free_dot_dev)."""
        abi.check(self.lib, self.lib.w3g_free_dot_dev(self.h, d_a, d_b, d_fixed, d_out, stream or None))


# Eisenstat-Walker forcing terms (choice 2, gamma = 0.9, exponent 2) for the
# inexact Newton solves: the linear solve of each iteration only needs to
# be as accurate as the Newton iteration can use; the convergence test is
# on the true residual of the recovery either way
EW_ETA_MAX, EW_GAMMA = 0.1, 0.9


def ew_forcing(eta_prev: float, rn: float, rn_prev: float, target: float, eta_max: float = EW_ETA_MAX) -> float:
    """Next relative tolerance of the linear solve: gamma (rn / rn_prev)^2,
    not below gamma eta_prev^2 when that is still large (safeguard against
    a sudden drop), at most eta_max, and no tighter than what reaching the
    Newton target `target` from rn needs. Problems whose Newton iterations
    converge only linearly (an inexact tangent) need a small eta_max: with
    0.1 the 100k-element mixed bars diverge in their first step."""
    eta = EW_GAMMA * (rn / rn_prev) ** 2
    sg = EW_GAMMA * eta_prev ** 2
    if sg > 0.1:
        eta = max(eta, sg)
    eta = min(eta, eta_max)
    return max(eta, 0.5 * target / rn)


class IncrementFailed(RuntimeError):
    """A (sub-)increment did not converge, or its recovery or solve asked
    for a smaller step."""


def run_subdivided(attempt, adaptive: bool, divisions: int = 4, min_fact: float = 1.0 / 16.0):
    """One load step under WARP3D's adaptive solution (adapt_check,
    src/adapt_check.f:15-120): attempt(fraction, after_cut) runs the whole
    step first; when it raises IncrementFailed, the failed increment is
    replaced by `divisions` equal sub-increments, down to `min_fact` of the
    step, and the first sub-increment after a cut runs with after_cut =
    True (the reference starts it without extrapolation). Returns the
    fractions that converged, in order, and the number of cuts; raises
    RuntimeError when a failed increment cannot be divided further."""
    pending, after_cut, done, cuts = [1.0], False, [], 0
    while pending:
        f = pending.pop(0)
        try:
            attempt(f, after_cut)
        except IncrementFailed as exc:
            sub = f / divisions
            if not adaptive or sub < min_fact * (1.0 - 1e-12):
                raise RuntimeError(str(exc)) from None
            cuts += 1
            pending = [sub] * divisions + pending
            after_cut = True
            continue
        after_cut = False
        done.append(f)
    return done, cuts


class DeviceNewtonDriver:
    """Displacement-controlled Newton loop on the device; same interface,
    convergence test and history as ``newton.NewtonDriver``.

    With ``adaptive`` a load step whose Newton iterations fail (no
    convergence within maxit, a step-cut request of the recovery, or a
    tangent that is not positive definite) is subdivided as WARP3D's
    adaptive solution does it (adapt_check, src/adapt_check.f:15-120;
    defaults :181-182): the failed increment is replaced by
    ``adapt_divisions`` equal sub-increments, down to ``adapt_min_fact`` of
    the step, and the first sub-increment after a cut starts without
    extrapolation. WARP3D does not subdivide step 1 (mnralg.f:131);
    ``adaptive_step1`` lifts that restriction. Extrapolated starts scale
    the last converged increment by the ratio of the increments' sizes
    (mnralg.f:257-285). ``history`` gets one entry per converged
    (sub-)increment; ``cuts`` counts subdivisions."""

    def __init__(self, model, engine, fixed, tol: float = 1e-8, maxit: int = 25, extrapolate: bool = False,
                 lin_rtol: float = 1e-10, lin_maxit: int = 50000, device: int = 0, csr: DeviceCsr | None = None,
                 adaptive: bool = False, adaptive_step1: bool = False, adapt_divisions: int = 4,
                 adapt_min_fact: float = 1.0 / 16.0, line_search: bool = False, forcing: str = "fixed",
                 eta_max: float = EW_ETA_MAX, graph: bool = False):
        import torch
        self.torch = torch
        self.model = model
        self.engine = engine
        self.tol, self.maxit, self.extrapolate = tol, maxit, extrapolate
        self.lin_rtol, self.lin_maxit = lin_rtol, lin_maxit
        if forcing not in ("fixed", "ew"):
            raise ValueError("forcing must be 'fixed' or 'ew'")
        self.forcing, self.eta_max = forcing, eta_max
        # one graph per Newton iteration (w3g_newton_iteration_dev); the line
        # search needs the host between its trial step lengths
        self.graph = graph and not line_search
        self.adaptive, self.adaptive_step1 = adaptive, adaptive_step1
        self.adapt_divisions, self.adapt_min_fact = adapt_divisions, adapt_min_fact
        dev = torch.device("cuda", device)
        n = model.nodof
        z = lambda: torch.zeros(n, dtype=torch.float64, device=dev)
        self.c = torch.from_numpy(np.ascontiguousarray(model.c)).to(dev)
        self.ud, self.du, self.ifv, self.d = z(), z(), z(), z()
        self.du_prev = None
        self.frac_prev = 1.0
        self.fixed_idx = torch.from_numpy(np.asarray(fixed, dtype=np.int64)).to(dev)
        self.mask = torch.zeros(n, dtype=torch.uint8, device=dev)
        self.mask[self.fixed_idx] = 1
        self.norms = torch.zeros(2, dtype=torch.float64, device=dev)
        self.sval = torch.zeros(1, dtype=torch.float64, device=dev)
        self.line_search = line_search
        self.alphas = []        # (step, [accepted step length per iteration]) with line search
        self.csr = csr if csr is not None else DeviceCsr(engine)   # the pattern is the model's: shareable
        self.history = []       # (step, iterations, relative residuals) per converged increment
        self.lin_history = []   # (step, [PCG iterations per Newton iteration])
        self.fractions = []     # fraction of its step each converged increment carried
        self.trace = []         # last increment: (PCG status, iterations, relative residual, Newton residual)
        self.cuts = 0

    @property
    def u(self) -> np.ndarray:
        return self.ud.cpu().numpy()

    def _ptrs(self):
        return self.c.data_ptr(), self.ud.data_ptr(), self.du.data_ptr()

    def _recover(self, step, it, extrap):
        c, u, du = self._ptrs()
        self.engine.recover_dev(step, it, extrap, c, u, du, self.ifv.data_ptr())
        st, _ = self.engine.recover_info()
        return st

    def _tangent(self, step, it):
        c, u, du = self._ptrs()
        self.engine.tanstf_dev(step, it, c, u, du)
        self.csr.assemble()

    def _increment(self, step: int, imp, extrap_scale):
        """One (sub-)increment: imposed increments imp (device vector,
        values on fixed dofs), extrapolated start du_prev * extrap_scale
        when extrap_scale is not None."""
        extrap = extrap_scale is not None
        if extrap:
            self.du.copy_(self.du_prev)
            self.du *= extrap_scale
        else:
            self.du.zero_()
        self.du[self.fixed_idx] = imp[self.fixed_idx]
        res_hist, lin, alphas = [], [], []
        self.alphas_last = alphas
        self.trace = []
        if self._recover(step, 0, extrap) != 0:
            raise IncrementFailed(f"step {step}: recovery requested a step cut at iteration 0")
        self._tangent(step, 0)
        eta, rn_prev = self.eta_max, None
        for it in range(1, self.maxit + 1):
            rtol = self.lin_rtol if self.forcing == "fixed" else max(self.lin_rtol, eta)
            if self.graph:
                # solve, du += d, recovery, norms and the next tangent in one graph
                c, u, du = self._ptrs()
                st, nits, rel, rst, rf, ra = self.csr.newton_iteration(
                    step, it, extrap, c, u, du, self.ifv.data_ptr(), self.mask.data_ptr(), self.d.data_ptr(), rtol,
                    self.lin_maxit, self.norms.data_ptr())
                lin.append(nits)
                self.trace.append([st, nits, rel, None])
                if st == abi.PCG_BREAKDOWN:
                    raise IncrementFailed(f"step {step}: tangent not positive definite on the free dofs "
                                          f"(iteration {it})")
                if rst != 0:
                    raise IncrementFailed(f"step {step}: step cut requested at iteration {it}")
                alphas.append(1.0)
                rn, scale = float(np.sqrt(rf)), max(float(np.sqrt(ra)), 1e-300)
                res_hist.append(rn / scale)
                self.trace[-1][3] = rn / scale
                if rn <= self.tol * scale:
                    return res_hist, lin
                if self.forcing == "ew" and rn_prev is not None:
                    eta = ew_forcing(eta, rn, rn_prev, self.tol * scale, self.eta_max)
                rn_prev = rn
                continue
            st, nits, rel = self.csr.pcg(self.mask.data_ptr(), self.ifv.data_ptr(), -1.0, self.d.data_ptr(),
                                         rtol, self.lin_maxit)
            lin.append(nits)
            self.trace.append([st, nits, rel, None])
            if st == abi.PCG_BREAKDOWN:
                raise IncrementFailed(f"step {step}: tangent not positive definite on the free dofs "
                                       f"(iteration {it})")
            alphas.append(self._search(step, it, extrap))
            self.csr.residual_norms(self.ifv.data_ptr(), self.mask.data_ptr(), self.norms.data_ptr())
            rf, ra = self.norms.cpu().numpy()
            rn, scale = float(np.sqrt(rf)), max(float(np.sqrt(ra)), 1e-300)
            res_hist.append(rn / scale)
            self.trace[-1][3] = rn / scale
            if rn <= self.tol * scale:
                return res_hist, lin
            if self.forcing == "ew" and rn_prev is not None:
                eta = ew_forcing(eta, rn, rn_prev, self.tol * scale, self.eta_max)
            rn_prev = rn
            self._tangent(step, it)
        raise IncrementFailed(f"step {step}: no convergence in {self.maxit} iterations: {res_hist}")

    def _s_value(self) -> float:
        """s = -res.idu over the free dofs (res = -ifv), one device reduction."""
        self.csr.free_dot(self.ifv.data_ptr(), self.d.data_ptr(), self.mask.data_ptr(), self.sval.data_ptr())
        return float(self.sval.item())

    def _search(self, step, it, extrap) -> float:
        """du += alpha d with alpha from mnralg_ls (newton.line_search), the
        internal forces recomputed for the accepted length; returns alpha."""
        from .newton import line_search

        def trial(alpha, du0=self.du.clone()):
            self.du.copy_(du0)
            if alpha == 1.0:
                self.du += self.d
            else:
                self.du.add_(self.d, alpha=alpha)
            if self._recover(step, it, extrap) != 0:
                raise IncrementFailed(f"step {step}: step cut requested at iteration {it}")
            return self._s_value()

        s0 = self._s_value() if self.line_search else 0.0
        if self.line_search and s0 < 0.0:
            return line_search(s0, trial)[0]
        trial(1.0)
        return 1.0

    def step(self, step: int, imposed: np.ndarray):
        """imposed: full-length vector; its values on fixed dofs are the
        displacement increments of this step."""
        torch = self.torch
        imp = torch.from_numpy(np.asarray(imposed, dtype=np.float64)).to(self.du.device)
        adaptive = self.adaptive and (step > 1 or self.adaptive_step1)
        out = []

        def attempt(f, after_cut):
            extrap_scale = None
            if self.extrapolate and self.du_prev is not None and step > 1 and not after_cut:
                extrap_scale = f / self.frac_prev
            res_hist, lin = self._increment(step, imp * f, extrap_scale)
            self.engine.update()
            self.ud += self.du
            self.du_prev = self.du.clone()
            self.frac_prev = f
            self.history.append((step, len(res_hist), res_hist))
            self.lin_history.append((step, lin))
            self.alphas.append((step, list(self.alphas_last)))
            self.fractions.append(f)
            out.extend(res_hist)

        _, cuts = run_subdivided(attempt, adaptive, self.adapt_divisions, self.adapt_min_fact)
        self.cuts += cuts
        return out
