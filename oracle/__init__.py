"""Python binding of the oracle (oracle/w3o.cpp).

TEST INFRASTRUCTURE ONLY: the CPU restatement of WARP3D's element-block
path that checks the CUDA engine and serves as the timed CPU baseline.
No Fortran compiler or MKL on these machines to execute the reference;
pinned end to end by two of WARP3D's own regression problems
(verification/test24, mm01, to 3.6e-6; verification/test82/voche_model,
mm10, to 4.0e-5 of the checked stress; tests/test_oracle_warp3d_*.py),
the rest by the closed-form tests in tests/.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from warp3d_gb300 import abi
from warp3d_gb300.model import HostState, Model, block_ptrs, dptr

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libw3o.so")
# the same restatement compiled with multiply-add contraction: the timed CPU
# baseline only (see build.sh), never a checker
FAST_LIB_PATH = os.path.join(HERE, "_build", "libw3o_fast.so")
FAST_FLAGS = "g++ -O3 -fopenmp -ffp-contract=fast -fno-math-errno -fno-trapping-math -funroll-loops"

_libs = {}


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, f) for f in ("w3o.cpp", "w3o.h", "w3o_mm10.cpp", "w3o_mm10.h", "w3o_umat.cpp",
                                             "w3o_umat.h", "build.sh")]
    newest = max(map(os.path.getmtime, srcs))
    stale = any(not os.path.exists(p) or os.path.getmtime(p) < newest for p in (LIB_PATH, FAST_LIB_PATH))
    if force or stale:
        subprocess.run(["sh", os.path.join(HERE, "build.sh")], check=True)
    return LIB_PATH


def load(fast: bool = False) -> C.CDLL:
    """The checker library, or with fast=True the contracted build that the
    CPU baseline times."""
    if fast not in _libs:
        build()
        lib = C.CDLL(FAST_LIB_PATH if fast else LIB_PATH)
        _d = C.POINTER(C.c_double)
        _pd = C.POINTER(_d)
        mp = C.POINTER(abi.ModelDesc)
        sp = C.POINTER(abi.BlockState)
        lib.w3o_set_threads.argtypes = [C.c_int]
        lib.w3o_set_deterministic.argtypes = [C.c_int]
        lib.w3o_tanstf.argtypes = [mp, sp, C.c_int, C.c_int, _d, _d, _d, _pd]
        lib.w3o_recover.argtypes = [mp, sp, C.c_int, C.c_int, C.c_int, _d, _d, _d, _d,
                                    C.POINTER(abi.RecoverInfo)]
        lib.w3o_update.argtypes = [mp, sp]
        lib.w3o_gauss_point.argtypes = [C.c_int, C.c_int, C.c_int, _d]
        lib.w3o_shape_derivs.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, _d, _d, _d]
        lib.w3o_mm01_point.argtypes = [C.c_int, C.c_int] + [_d] * 11
        lib.w3o_mm10_point.argtypes = [C.POINTER(abi.Crystal), _d, C.c_int, C.c_int, C.c_int, C.c_double] + [_d] * 6
        lib.w3o_umat_point.argtypes = [_d, C.c_int, C.c_int, C.c_int] + [_d] * 7
        _libs[fast] = lib
    return _libs[fast]


class Oracle:
    """Same calls as warp3d_gb300.engine.Engine, on a HostState."""

    def __init__(self, model: Model, state: HostState | None = None, threads: int = 0,
                 deterministic: bool = True, fast: bool = False):
        self.lib = load(fast)
        self.model = model
        self.state = state if state is not None else model.new_state()
        self.desc = model.desc()
        self.lib.w3o_set_threads(threads)
        self.lib.w3o_set_deterministic(1 if deterministic else 0)

    def tanstf(self, step, it, c, u, du, estiff_blocks):
        s = self.state.struct()
        ptrs = block_ptrs(estiff_blocks)
        return self.lib.w3o_tanstf(C.byref(self.desc), C.byref(s), step, it, dptr(c), dptr(u), dptr(du),
                                   C.cast(ptrs, C.POINTER(C.POINTER(C.c_double))))

    def recover(self, step, it, extrapolated, c, u, du, ifv):
        s = self.state.struct()
        info = abi.RecoverInfo()
        st = self.lib.w3o_recover(C.byref(self.desc), C.byref(s), step, it, 1 if extrapolated else 0, dptr(c),
                                  dptr(u), dptr(du), dptr(ifv), C.byref(info))
        return st, info

    def update(self):
        s = self.state.struct()
        return self.lib.w3o_update(C.byref(self.desc), C.byref(s))


def mm01_points(step, e, nu, beta, hprime, yld, cgn, deps, history):
    """One mm01 + cnst1 update of len(e) points (column-major (span,k) I/O)."""
    lib = load()
    n = len(e)
    f = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    e, nu, beta, hprime, yld = map(f, (e, nu, beta, hprime, yld))
    cgn = f(np.asarray(cgn).T.reshape(-1))          # (9, n)
    deps = f(np.asarray(deps).T.reshape(-1))        # (6, n)
    hist = f(np.asarray(history).T.reshape(-1))     # (11, n)
    cgn1 = np.zeros(9 * n)
    hist1 = np.zeros(11 * n)
    cep = np.zeros(36 * n)
    st = lib.w3o_mm01_point(n, step, dptr(e), dptr(nu), dptr(beta), dptr(hprime), dptr(yld), dptr(cgn),
                            dptr(cgn1), dptr(deps), dptr(hist), dptr(hist1), dptr(cep))
    assert st == 0
    # cep (span, 36) column-major with (r,c) -> r + 6c  -> [n, 6(c), 6(r)] -> transpose
    cep_m = cep.reshape(36, n).T.reshape(n, 6, 6).transpose(0, 2, 1)
    return cgn1.reshape(9, n).T, hist1.reshape(11, n).T, hist.reshape(11, n).T, cep_m


def umat_point(props, step, it, extrapolated, urcs_n, eps_n, uddt, hist):
    """One point of the UMAT path: (status, urcs_n1 (9), hist1 (20), [D] 6x6
    symmetric in WARP3D order)."""
    lib = load()
    f = lambda a, n: np.ascontiguousarray(np.resize(np.asarray(a, dtype=np.float64), n))
    pr = np.zeros(abi.UMAT_NPROPS)
    pr[:len(props)] = props
    un1, h1, c21 = np.zeros(9), np.zeros(abi.HIST_UMAT), np.zeros(21)
    st = lib.w3o_umat_point(dptr(pr), step, it, 1 if extrapolated else 0, dptr(f(urcs_n, 9)), dptr(f(eps_n, 6)),
                            dptr(f(uddt, 6)), dptr(f(hist, abi.HIST_UMAT)), dptr(un1), dptr(h1), dptr(c21))
    D = np.zeros((6, 6))
    k = 0
    for r in range(6):
        for c in range(r + 1):
            D[r, c] = D[c, r] = c21[k]
            k += 1
    return st, un1, h1, D

