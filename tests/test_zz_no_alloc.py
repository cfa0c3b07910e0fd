"""The allocation-free internal-force assembly, w3g_assemble_ifv_noalloc.

For callers that cannot allocate device memory (their device arrays come
from a pool or a framework that owns the allocator, or allocation is
forbidden after start-up) and therefore cannot create a w3g_context. The
test allocates its own device buffers with torch -- the entry point under
test allocates nothing -- and checks that two calls in a row reproduce
the nodal vector and sum |einfvec| of the regular recovery entry point
(w3g_recover) within the parity tolerance of the other GPU tests.

Kept in its own file, collected last, so that a run stopping at the first
failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import make_model
from warp3d_gb300 import abi

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _reference_forces():
    from warp3d_gb300.engine import Engine
    model, _ = make_model(n=6, jitter=0.1, spans=[128, 37, 1, 50])
    rng = np.random.default_rng(5)
    du = rng.normal(0.0, 2e-3, model.nodof)
    eng = Engine(model)
    ifv = np.zeros(model.nodof)
    st, info = eng.recover(1, 1, False, model.c, np.zeros(model.nodof), du, ifv)
    assert st == 0
    state = model.new_state()
    eng.download(state, names=("einfvec",))
    eng.close()
    return model, state, ifv, info.sum_ifv


def test_noalloc_assembly_matches_recover_on_two_calls():
    torch = pytest.importorskip("torch")
    model, state, ifv_ref, sum_ref = _reference_forces()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    einf = torch.from_numpy(np.concatenate([a.ravel() for a in state.einfvec])).to(dev)
    edest = torch.from_numpy(np.concatenate([e.ravel() for e in model.edest]).astype(np.int32)).to(dev)
    ifv = torch.full((model.nodof,), 7.0, dtype=torch.float64, device=dev)   # garbage: must be overwritten
    ssum = torch.zeros(1, dtype=torch.float64, device=dev)
    elblks = np.ascontiguousarray(model.elblks.ravel(), dtype=np.int32)
    totdof = np.full(model.nelblk, model.totdof, dtype=np.int32)
    lib = abi.load()
    stream = torch.cuda.current_stream().cuda_stream
    scale = max(np.max(np.abs(a)) for a in state.einfvec)
    for call in range(2):
        st = lib.w3g_assemble_ifv_noalloc(model.nelblk, elblks.ctypes.data_as(C.POINTER(C.c_int)),
                                          totdof.ctypes.data_as(C.POINTER(C.c_int)), model.nodof,
                                          einf.data_ptr(), edest.data_ptr(), ifv.data_ptr(), ssum.data_ptr(),
                                          stream)
        assert st == 0, lib.w3g_last_error()
        got = ifv.cpu().numpy()
        assert np.max(np.abs(got - ifv_ref)) <= TOL * scale, call
        assert abs(float(ssum.item()) - sum_ref) <= TOL * sum_ref, call


def test_noalloc_rejects_more_blocks_than_its_scratch_holds():
    lib = abi.load()
    n = 65537
    elblks = np.tile(np.array([128, 1, 0], dtype=np.int32), n)
    totdof = np.full(n, 24, dtype=np.int32)
    dummy = C.c_void_p(16)   # never dereferenced: the size check comes first
    st = lib.w3g_assemble_ifv_noalloc(n, elblks.ctypes.data_as(C.POINTER(C.c_int)),
                                      totdof.ctypes.data_as(C.POINTER(C.c_int)), 10, dummy, dummy, dummy, dummy,
                                      None)
    assert st == abi.EARG
    assert b"exceed the fixed scratch" in lib.w3g_last_error()
