"""The C-ABI's refusals of malformed or unsupported input (w3g_create and
the setters): each case returns the documented status with a message that
names the block or element, creates no context and launches nothing. The
descriptions are built from a valid model and then damaged on the host."""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import make_model
from warp3d_gb300 import abi
from warp3d_gb300.model import Crystal, Model, Umat, cube_mesh, mixed_mesh, random_orientations, Part

pytestmark = pytest.mark.gpu


def _create(desc, model):
    """w3g_create over `desc`; `model` owns the arrays desc points into and
    must stay alive until the call returns."""
    assert model is not None
    lib = abi.load()
    ctx = C.c_void_p()
    st = lib.w3g_create(0, C.byref(desc), C.byref(ctx))
    if st == 0:
        lib.w3g_destroy(ctx)
    return st, lib.w3g_last_error().decode()


def _brick_model():
    return make_model(n=3, jitter=0.05, spans=[10, 17])[0]


def test_valid_description_is_accepted():
    m = _brick_model()
    assert _create(m.desc(), m)[0] == 0


def test_empty_model_is_refused():
    m = _brick_model()
    d = m.desc()
    d.nelblk = 0
    assert _create(d, m) == (abi.EARG, "incomplete model description")


def test_bad_block_span_and_order():
    m = _brick_model()
    m.elblks[1, 0] = 0                      # a block of no elements
    st, msg = _create(m.desc(), m)
    assert st == abi.EARG and "block 2" in msg
    m = _brick_model()
    m.elblks[1, 1] = 5                      # blocks not covering 1..noelem in order
    st, msg = _create(m.desc(), m)
    assert st == abi.EARG and "in order" in msg


def test_unsupported_element_type_and_material():
    m = _brick_model()
    m.iprops[:, 5] = 27                     # 8-node brick with 27 Gauss points: no path
    st, msg = _create(m.desc(), m)
    assert st == abi.EUNSUPPORTED and "element type" in msg
    m = _brick_model()
    m.iprops[:, 24] = 5                     # mm05 cyclic plasticity: not built
    st, msg = _create(m.desc(), m)
    assert st == abi.EUNSUPPORTED and "material model" in msg


def test_umat_without_properties_and_with_bbar():
    coords, incid = cube_mesh(2)
    m = Model(coords, incid, materials=[Umat((200000.0, 0.3, 400.0, 2000.0, 0.0))])
    d = m.desc()
    d.umat_props = None
    st, msg = _create(d, m)
    assert st == abi.EARG and "umat_props" in msg
    m = Model(coords, incid, materials=[Umat((200000.0, 0.3, 400.0, 2000.0, 0.0))], bbar=True)
    st, msg = _create(m.desc(), m)
    assert st == abi.EUNSUPPORTED and "b-bar" in msg


def test_crystal_plasticity_checks():
    coords, incid = cube_mesh(2)
    m = Model(coords, incid, materials=[Crystal()], angles=random_orientations(8, 3), dt=1.0)
    m.elem_crystal[3] = 5                   # no crystal 5
    st, msg = _create(m.desc(), m)
    assert st == abi.EARG and "element 4" in msg
    m = Model(coords, incid, materials=[Crystal()], angles=random_orientations(8, 3), dt=0.0)
    st, msg = _create(m.desc(), m)
    assert st == abi.EARG and "dt" in msg


def test_edest_index_outside_the_dofs():
    m = _brick_model()
    m.edest[1][3, 5] = m.nodof + 1
    st, msg = _create(m.desc(), m)
    assert st == abi.EARG and "block 2" in msg


def test_setters_refuse_unknown_values():
    from warp3d_gb300.engine import Engine
    eng = Engine(_brick_model())
    lib = eng.lib
    assert lib.w3g_set_tangent_precision(eng.ctx, 99) == abi.EARG
    assert lib.w3g_set_update_mode(eng.ctx, 2) == abi.EARG
    bad = abi.Schedule(7, 0, 0, 1, 1, 0)
    assert lib.w3g_set_schedule(eng.ctx, C.byref(bad)) == abi.EARG
    eng.close()
