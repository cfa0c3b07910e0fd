"""CPU checks of the C-ABI boundary: the library builds for sm_103a and
loads, exports every entry point include/w3g.h declares, and the engine
refuses to run without a GPU (no CPU fallback). No kernel is launched."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from tests.conftest import ROOT, cuda_available
from warp3d_gb300 import abi, build
from warp3d_gb300.model import Model, cube_mesh


def _declared_functions():
    text = open(os.path.join(ROOT, "include", "w3g.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(w3g_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_tanstf_recover_update_entry_points():
    names = _declared_functions()
    for n in ("w3g_create", "w3g_tanstf", "w3g_recover", "w3g_update", "w3g_tanstf_dev", "w3g_recover_dev"):
        assert n in names


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(build.build())
    for n in _declared_functions():
        assert hasattr(lib, n), n
    # the Python prototypes cover the same set
    assert sorted(p[0] for p in abi.PROTOTYPES) == _declared_functions()


def test_struct_layouts_match_header_sizes():
    # field sizes as declared in include/w3g.h (LP64)
    assert C.sizeof(abi.RecoverInfo) == 8 * 3 + 8 + 4 + 4
    assert C.sizeof(abi.BlockState) == 10 * C.sizeof(C.c_void_p)


@pytest.mark.skipif(cuda_available(), reason="checks the no-GPU failure path")
def test_engine_fails_loudly_without_a_gpu():
    from warp3d_gb300.engine import Engine
    coords, incid = cube_mesh(1)
    with pytest.raises(abi.W3GError) as ei:
        Engine(Model(coords, incid))
    assert ei.value.code == abi.ECUDA


def test_oracle_library_builds_and_exports():
    import oracle
    lib = oracle.load()
    for n in ("w3o_tanstf", "w3o_recover", "w3o_update", "w3o_mm01_point"):
        assert hasattr(lib, n)


def test_umat_features_describe_the_compiled_umat():
    """w3g_umat_features answers as WARP3D's umat_set_features does for the
    UMAT compiled into the library (a host call: no kernel)."""
    lib = C.CDLL(build.build())
    lib.w3g_umat_features.argtypes = [C.POINTER(C.c_int)]
    info = (C.c_int * 4)()
    assert lib.w3g_umat_features(info) == 0
    assert list(info) == [abi.HIST_UMAT, 21, 0, 14]
