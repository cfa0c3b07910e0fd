"""w3g_store_blocks / w3g_reopen_blocks: the engine writes the element-
block section of a WARP3D restart file byte for byte as the independent
writer of tests/restart_records.py does from the same state, reads it back
(also from an offset inside a longer file) with the n+1 arrays equal to
the n arrays, as reopen does, and continues the analysis bitwise as the
engine that wrote it; a damaged record is refused with W3G_EARG."""
import numpy as np
import pytest

import oracle
from tests import restart_records as rr
from tests.helpers import loaded_state, make_model
from warp3d_gb300 import abi

pytestmark = pytest.mark.gpu


def _engine(model):
    from warp3d_gb300.engine import Engine
    return Engine(model)


@pytest.fixture(scope="module", params=["geonl", "small_bbar", "mixed"])
def loaded(request):
    opts = {"geonl": {}, "small_bbar": dict(geonl=False, bbar=True), "mixed": {}}[request.param]
    model, nxyz = make_model(n=4, jitter=0.1, spans=[40, 24], **opts)
    if request.param == "mixed":
        model.lprops[40:, 17] = 0          # second block small-displacement
    ora, drv, du = loaded_state(model, nxyz, oracle.Oracle, steps=2, strain_per_step=0.0015)
    return model, ora.state, drv.u.copy(), du


def test_store_matches_independent_writer(loaded, tmp_path):
    model, state, _, _ = loaded
    eng = _engine(model)
    eng.upload(state)
    path = str(tmp_path / "blocks.bin")
    eng.store_blocks(path)
    data = open(path, "rb").read()
    assert data == rr.write_section(model, state)


def test_reopen_restores_state_and_continues(loaded, tmp_path):
    model, state, u, du = loaded
    e1 = _engine(model)
    e1.upload(state)
    path = str(tmp_path / "restart.bin")
    prefix = rr._record(b"earlier sections of the restart file") + rr._key()
    with open(path, "wb") as f:
        f.write(prefix)
    e1.store_blocks(path, append=True)
    e2 = _engine(model)
    end = e2.reopen_blocks(path, offset=len(prefix))
    assert end == len(open(path, "rb").read())
    got = model.new_state()
    e2.download(got)
    for n, n1 in (("history", "history1"), ("urcs_n", "urcs_n1"), ("eps_n", "eps_n1")):
        assert np.array_equal(got.concat(n), state.concat(n))
        assert np.array_equal(got.concat(n1), state.concat(n))      # reopen: n+1 = n
    for name in ("cep", "element_vol"):
        assert np.array_equal(got.concat(name), state.concat(name))
    for b in range(model.nelblk):
        if rr.geonl(model, b):
            assert np.array_equal(got.rot_n1[b], state.rot_n1[b])
    # the next Newton iteration from the reopened engine is the writer's,
    # once the writer's n+1 arrays are set the same way
    e1.upload(got, names=["history1", "urcs_n1", "eps_n1"])
    f1, f2 = np.zeros(model.nodof), np.zeros(model.nodof)
    assert e1.recover(3, 1, False, model.c, u, du, f1)[0] == e2.recover(3, 1, False, model.c, u, du, f2)[0] == 0
    assert np.array_equal(f1, f2)
    k1, k2 = model.estiff_blocks(), model.estiff_blocks()
    e1.tanstf(3, 1, model.c, u, du, k1)
    e2.tanstf(3, 1, model.c, u, du, k2)
    assert all(np.array_equal(a, b) for a, b in zip(k1, k2))


def test_damaged_record_is_refused(loaded, tmp_path):
    model, state, _, _ = loaded
    eng = _engine(model)
    eng.upload(state)
    path = str(tmp_path / "bad.bin")
    eng.store_blocks(path)
    data = bytearray(open(path, "rb").read())
    data[0] ^= 0x01                         # first length marker
    open(path, "wb").write(bytes(data))
    with pytest.raises(abi.W3GError):
        _engine(model).reopen_blocks(path)
