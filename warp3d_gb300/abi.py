"""ctypes mirror of include/w3g.h and loader of the CUDA engine.

The engine is the in-tree shared library ``warp3d_gb300/_build/libw3g.so``
(built by :mod:`warp3d_gb300.build`). There is no CPU fallback: if the
library or a CUDA device is missing, :func:`load` raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libw3g.so")

MXELPR = 43
MXVL = 128
ETYPE_Q3DISOP = 1
ETYPE_L3DISOP = 2
ETYPE_TET10 = 6
MAT_BILINEAR = 1
MAT_UMAT = 8
MAT_CRYSTAL = 10
UMAT_NPROPS = 50

OK = 0
STEP_CUT = 1
LOCAL_FAIL = 2
EARG = -1
EUNSUPPORTED = -2
ECUDA = -3
ENOMEM = -4
EFATAL = -5
UPDATE_COPY = 0
UPDATE_SWAP = 1

HIST_MM01 = 11
HIST_MM10 = 158       # one 12-system (fcc or bcc) crystal, one hardening variable
HIST_UMAT = 20        # state variables of the UMAT compiled into the library (w3g_umat_features)

TANGENT_FP64 = 0
TANGENT_FP32 = 1
TANGENT_TF32 = 2
TANGENT_BF16 = 3
TANGENT_TF32X3 = 4
TANGENT_BF16X3 = 5
PCG_MAXIT = 1
PCG_BREAKDOWN = 2

SCHED_PER_TYPE = 0
SCHED_PERSISTENT = 1
ORDER_BLOCKS = 0
ORDER_HEAVY_FIRST = 1
ITER_RECOVER = 1
ITER_TANGENT = 2

_dpp = C.POINTER(C.POINTER(C.c_double))
_ipp = C.POINTER(C.POINTER(C.c_int))


class Crystal(C.Structure):
    """w3g_crystal: one mm10 crystal definition."""
    _fields_ = [
        ("slip_type", C.c_int),
        ("elastic_type", C.c_int),
        ("h_type", C.c_int),
        ("miter", C.c_int),
        ("e", C.c_double),
        ("nu", C.c_double),
        ("harden_n", C.c_double),
        ("tau_y", C.c_double),
        ("tau_v", C.c_double),
        ("theta_o", C.c_double),
        ("voche_m", C.c_double),
        ("iD_v", C.c_double),
        ("k_o", C.c_double),
        ("b", C.c_double),
        ("atol", C.c_double),
        ("atol1", C.c_double),
        ("rtol", C.c_double),
        ("rtol1", C.c_double),
    ]


class ModelDesc(C.Structure):
    _fields_ = [
        ("nelblk", C.c_int),
        ("elblks", C.POINTER(C.c_int)),
        ("noelem", C.c_int),
        ("props", C.POINTER(C.c_float)),
        ("iprops", C.POINTER(C.c_int)),
        ("lprops", C.POINTER(C.c_int)),
        ("edest", _ipp),
        ("cdest", _ipp),
        ("nodof", C.c_int),
        ("ncoord", C.c_int),
        ("qbar_flag", C.c_int),
        ("beta_fact", C.c_double),
        ("crystals", C.POINTER(Crystal)),
        ("ncrystals", C.c_int),
        ("elem_crystal", C.POINTER(C.c_int)),
        ("elem_angles", C.POINTER(C.c_double)),
        ("dt", C.c_double),
        ("eps_bbar", C.c_double),
        ("asymmetric_assembly", C.c_int),
        ("umat_props", C.POINTER(C.c_double)),
    ]


class BlockState(C.Structure):
    _fields_ = [
        ("history", _dpp),
        ("history1", _dpp),
        ("urcs_n", _dpp),
        ("urcs_n1", _dpp),
        ("eps_n", _dpp),
        ("eps_n1", _dpp),
        ("rot_n1", _dpp),
        ("cep", _dpp),
        ("einfvec", _dpp),
        ("element_vol", _dpp),
    ]


class RecoverInfo(C.Structure):
    _fields_ = [
        ("internal_energy", C.c_double),
        ("plastic_work", C.c_double),
        ("sum_ifv", C.c_double),
        ("num_term_ifv", C.c_longlong),
        ("material_cut_step", C.c_int),
        ("first_bad_element", C.c_int),
    ]


class Schedule(C.Structure):
    _fields_ = [
        ("mode", C.c_int),
        ("recover_ctas_per_sm", C.c_int),
        ("tangent_ctas_per_sm", C.c_int),
        ("recover_grain", C.c_int),
        ("tangent_grain", C.c_int),
        ("order", C.c_int),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Timers(C.Structure):
    _fields_ = [("tangent_s", C.c_double), ("recover_s", C.c_double), ("update_s", C.c_double),
                ("tangent_calls", C.c_longlong), ("recover_calls", C.c_longlong), ("update_calls", C.c_longlong)]


# exported symbols and their prototypes: (name, restype, argtypes)
_vp = C.c_void_p
_d = C.POINTER(C.c_double)
PROTOTYPES = [
    ("w3g_create", C.c_int, [C.c_int, C.POINTER(ModelDesc), C.POINTER(_vp)]),
    ("w3g_destroy", C.c_int, [_vp]),
    ("w3g_last_error", C.c_char_p, []),
    ("w3g_set_tangent_precision", C.c_int, [_vp, C.c_int]),
    ("w3g_set_wait_limit", C.c_int, [_vp, C.c_longlong]),
    ("w3g_set_update_mode", C.c_int, [_vp, C.c_int]),
    ("w3g_umat_features", C.c_int, [C.POINTER(C.c_int)]),
    ("w3g_state_upload", C.c_int, [_vp, C.POINTER(BlockState)]),
    ("w3g_state_download", C.c_int, [_vp, C.POINTER(BlockState)]),
    ("w3g_store_blocks", C.c_int, [_vp, C.c_char_p, C.c_int]),
    ("w3g_reopen_blocks", C.c_int, [_vp, C.c_char_p, C.c_longlong, C.POINTER(C.c_longlong)]),
    ("w3g_tanstf", C.c_int, [_vp, C.c_int, C.c_int, _d, _d, _d, C.POINTER(_d)]),
    ("w3g_recover", C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _d, _d, _d, _d, C.POINTER(RecoverInfo)]),
    ("w3g_update", C.c_int, [_vp]),
    ("w3g_tanstf_dev", C.c_int, [_vp, C.c_int, C.c_int, _vp, _vp, _vp, _vp]),
    ("w3g_recover_dev", C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp, _vp]),
    ("w3g_recover_info_get", C.c_int, [_vp, C.POINTER(RecoverInfo)]),
    ("w3g_estiff_device", C.c_int, [_vp, C.POINTER(_vp), C.POINTER(C.c_longlong)]),
    ("w3g_last_launch_count", C.c_int, [_vp]),
    ("w3g_measure_fp64_peak", C.c_int, [C.c_int, C.POINTER(C.c_double)]),
    ("w3g_assemble_ifv_noalloc", C.c_int, [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int, _vp, _vp,
                                           _vp, _vp, _vp]),
    ("w3g_set_schedule", C.c_int, [_vp, C.POINTER(Schedule)]),
    ("w3g_local_iterations", C.c_int, [_vp, C.POINTER(C.c_int), C.c_int]),
    ("w3g_get_schedule", C.c_int, [_vp, C.POINTER(Schedule)]),
    ("w3g_iteration_dev", C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp, _vp]),
    ("w3g_autotune", C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp, _vp, C.c_int,
                               C.POINTER(Schedule), C.POINTER(C.c_double)]),
    ("w3g_csr_create", C.c_int, [_vp, C.POINTER(_vp)]),
    ("w3g_csr_destroy", C.c_int, [_vp]),
    ("w3g_csr_info", C.c_int, [_vp, C.POINTER(C.c_int), C.POINTER(C.c_longlong), C.POINTER(_vp), C.POINTER(_vp),
                               C.POINTER(_vp)]),
    ("w3g_csr_assemble_dev", C.c_int, [_vp, _vp]),
    ("w3g_csr_download", C.c_int, [_vp, _vp, _vp, _vp]),
    ("w3g_csr_set_node_blocks", C.c_int, [_vp, C.c_int]),
    ("w3g_pcg_dev", C.c_int, [_vp, _vp, _vp, C.c_double, _vp, C.c_double, C.c_int, _vp, C.POINTER(C.c_int),
                              C.POINTER(C.c_double)]),
    ("w3g_residual_norms_dev", C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    ("w3g_free_dot_dev", C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp]),
    ("w3g_newton_iteration_dev", C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp, _vp, _vp, C.c_double,
                                          C.c_int, _vp, _vp, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                          C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    ("w3g_timers_get", C.c_int, [_vp, C.POINTER(Timers)]),
    ("w3g_timers_reset", C.c_int, [_vp]),
    ("w3g_check_finite", C.c_int, [_vp, C.POINTER(C.c_longlong)]),
    ("w3g_device_name", C.c_int, [C.c_int, C.c_char_p, C.c_int]),
]

_lib = None


def declare(lib: C.CDLL) -> C.CDLL:
    for name, res, args in PROTOTYPES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def load(path: str | None = None) -> C.CDLL:
    """Loads libw3g.so (building it first when only the sources exist)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        from . import build as _build
        _build.build()
    lib = declare(C.CDLL(p))
    if path is None:
        _lib = lib
    return lib


class W3GError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"w3g status {code}: {msg}")
        self.code = code


def check(lib: C.CDLL, code: int, allow=(OK,)) -> int:
    if code not in allow:
        raise W3GError(code, lib.w3g_last_error().decode(errors="replace"))
    return code
