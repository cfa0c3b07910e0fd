"""The test-side writer and reader of the restart block section
(tests/restart_records.py) against each other and against the record
structure of store_blocks (src/store.f:915-1010): record lengths, check
records, section order, geonl-only rotations."""
import struct

import numpy as np

from tests import restart_records as rr
from tests.helpers import make_model


def _state(model, seed=0):
    st = model.new_state()
    rng = np.random.default_rng(seed)
    for name in st.NAMES:
        for a in getattr(st, name):
            a[...] = rng.normal(size=a.shape)
    return st


def test_round_trip_and_layout():
    model, _ = make_model(n=3, spans=[20, 7])
    st = _state(model)
    data = rr.write_section(model, st)
    got, end = rr.read_section(model, data)
    assert end == len(data)
    for name in ("history", "cep", "urcs_n", "rot_n1", "eps_n", "element_vol"):
        for b in range(model.nelblk):
            assert np.array_equal(got[name][b], getattr(st, name)[b].reshape(-1))
    # first record: block 1's history (11 words x 8 points x 20 elements)
    (n,) = struct.unpack_from("<i", data, 0)
    assert n == 8 * 11 * 8 * 20
    # then its check record
    assert struct.unpack_from("<iii", data, 8 + n) == (4, rr.KEY, 4)


def test_small_displacement_blocks_carry_no_rotations():
    model, _ = make_model(n=3, spans=[20, 7], geonl=False)
    st = _state(model, 1)
    data = rr.write_section(model, st)
    geonl_model, _ = make_model(n=3, spans=[20, 7])
    assert len(rr.write_section(geonl_model, st)) - len(data) == sum(8 + 8 * a.size + 12 for a in st.rot_n1)
    got, end = rr.read_section(model, data)
    assert end == len(data) and got["rot_n1"] == [None, None]
