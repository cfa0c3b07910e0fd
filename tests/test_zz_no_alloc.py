"""The allocation-free internal-force assembly, w3g_assemble_ifv_noalloc.

For callers that cannot allocate device memory (their device arrays come
from a pool or a framework that owns the allocator, or allocation is
forbidden after start-up) and therefore cannot create a w3g_context. The
test allocates its own device buffers with torch -- the entry point under
test allocates nothing -- and checks that two calls in a row reproduce
the nodal vector and sum |einfvec| of the regular recovery entry point
(w3g_recover) within the parity tolerance of the other GPU tests, on a
model of 8-node bricks and on one that mixes 8-node bricks, 20-node
bricks and tetrahedra in blocks of uneven size (per-block totdof 24, 60
and 30). An edest table holding an index outside 1..nodof is refused
without any write outside ifv.

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


def _reference_forces(model):
    from warp3d_gb300.engine import Engine
    rng = np.random.default_rng(5)
    du = rng.normal(0.0, 2e-3, model.nodof)
    eng = Engine(model)
    ifv = np.zeros(model.nodof)
    st, info = eng.recover(1, 1, False, model.c, np.zeros(model.nodof), du, ifv)
    assert st == 0
    state = model.new_state()
    eng.download(state, names=("einfvec",))
    eng.close()
    return state, ifv, info.sum_ifv


def _brick_model():
    return make_model(n=6, jitter=0.1, spans=[128, 37, 1, 50])[0]


def _mixed_model():
    from tests.test_gpu_parity_types import _mixed_model as mixed
    return mixed()[0]


class _Call:
    """Device copies of a model's einfvec and edest and the call itself."""

    def __init__(self, model, state):
        import torch
        dev = torch.device("cuda", 0)
        torch.cuda.set_device(dev)
        self.torch = torch
        self.model = model
        # einfvec blocks as (span, totdof) Fortran arrays: the host state
        # holds them as (totdof, span) C arrays, the same bytes
        self.einf = torch.from_numpy(np.concatenate([a.ravel() for a in state.einfvec])).to(dev)
        self.edest = torch.from_numpy(np.concatenate([e.ravel() for e in model.edest]).astype(np.int32)).to(dev)
        self.ifv = torch.full((model.nodof,), 7.0, dtype=torch.float64, device=dev)   # must be overwritten
        self.ssum = torch.zeros(1, dtype=torch.float64, device=dev)
        self.elblks = np.ascontiguousarray(model.elblks.ravel(), dtype=np.int32)
        self.totdof = np.ascontiguousarray(model.block_totdof, dtype=np.int32)
        self.lib = abi.load()

    def __call__(self):
        stream = self.torch.cuda.current_stream().cuda_stream
        return self.lib.w3g_assemble_ifv_noalloc(
            self.model.nelblk, self.elblks.ctypes.data_as(C.POINTER(C.c_int)),
            self.totdof.ctypes.data_as(C.POINTER(C.c_int)), self.model.nodof, self.einf.data_ptr(),
            self.edest.data_ptr(), self.ifv.data_ptr(), self.ssum.data_ptr(), stream)


@pytest.mark.parametrize("build", [_brick_model, _mixed_model], ids=["hex8", "hex8_hex20_tet10"])
def test_noalloc_assembly_matches_recover_on_two_calls(build):
    model = build()
    state, ifv_ref, sum_ref = _reference_forces(model)
    call = _Call(model, state)
    scale = max(np.max(np.abs(a)) for a in state.einfvec)
    for k in range(2):
        st = call()
        assert st == 0, call.lib.w3g_last_error()
        got = call.ifv.cpu().numpy()
        assert np.max(np.abs(got - ifv_ref)) <= TOL * scale, k
        assert abs(float(call.ssum.item()) - sum_ref) <= TOL * sum_ref, k


def test_noalloc_refuses_an_edest_index_outside_the_nodal_vector():
    model = _mixed_model()
    state, ifv_ref, _ = _reference_forces(model)
    call = _Call(model, state)
    # one entry of the third block points past the end of ifv: the call
    # skips it (no write outside ifv) and names the block
    off = sum(int(model.spans[b]) * model.block_totdof[b] for b in range(2))
    call.edest[off + 3] = model.nodof + 5
    assert call() == abi.EARG
    assert b"block 3" in call.lib.w3g_last_error()
    # the next call with a good table is correct again (the bad-index
    # record is cleared at the start of every call)
    call.edest[off + 3] = int(model.edest[2].ravel()[3])
    assert call() == 0, call.lib.w3g_last_error()
    scale = max(np.max(np.abs(a)) for a in state.einfvec)
    assert np.max(np.abs(call.ifv.cpu().numpy() - ifv_ref)) <= TOL * scale


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
