"""An independent writer and reader of the element-block section of a
WARP3D restart file, for the tests: the records store (src/store.f:329-341)
writes with store_blocks (src/store.f:915-1010) in Fortran sequential
unformatted form -- each record a 4-byte little-endian length, the bytes,
the same length; a check record holds the int32 2147483647.

Section order: per block history (state n) + check, cep + check; per block
urcs_n + check, then one check; per geonl block rot_n1 + check, one check;
per block eps_n + check, one check; per block element volumes + check, one
check."""
from __future__ import annotations

import struct

import numpy as np

KEY = 2147483647


def _record(payload: bytes) -> bytes:
    n = struct.pack("<i", len(payload))
    return n + payload + n


def _key() -> bytes:
    return _record(struct.pack("<i", KEY))


def geonl(model, b: int) -> bool:
    """lprops(18) of the block's first element (rot_n1 is kept for geonl
    blocks only, src/reopen.f rotation_init)."""
    return bool(model.lprops[model.felem[b], 17])


def write_section(model, state) -> bytes:
    """The section for a HostState (warp3d_gb300.model.HostState)."""
    out = []
    for b in range(model.nelblk):
        out += [_record(np.ascontiguousarray(state.history[b], dtype="<f8").tobytes()), _key(),
                _record(np.ascontiguousarray(state.cep[b], dtype="<f8").tobytes()), _key()]
    for b in range(model.nelblk):
        out += [_record(np.ascontiguousarray(state.urcs_n[b], dtype="<f8").tobytes()), _key()]
    out.append(_key())
    for b in range(model.nelblk):
        if geonl(model, b):
            out += [_record(np.ascontiguousarray(state.rot_n1[b], dtype="<f8").tobytes()), _key()]
    out.append(_key())
    for b in range(model.nelblk):
        out += [_record(np.ascontiguousarray(state.eps_n[b], dtype="<f8").tobytes()), _key()]
    out.append(_key())
    for b in range(model.nelblk):
        out += [_record(np.ascontiguousarray(state.element_vol[b], dtype="<f8").tobytes()), _key()]
    out.append(_key())
    return b"".join(out)


class Reader:
    def __init__(self, data: bytes, offset: int = 0):
        self.data, self.pos = data, offset

    def record(self) -> bytes:
        (n,) = struct.unpack_from("<i", self.data, self.pos)
        body = self.data[self.pos + 4:self.pos + 4 + n]
        (m,) = struct.unpack_from("<i", self.data, self.pos + 4 + n)
        assert m == n, "record length markers differ"
        self.pos += 8 + n
        return body

    def key(self):
        (k,) = struct.unpack("<i", self.record())
        assert k == KEY

    def doubles(self) -> np.ndarray:
        a = np.frombuffer(self.record(), dtype="<f8").copy()
        self.key()
        return a


def read_section(model, data: bytes, offset: int = 0) -> tuple[dict, int]:
    """Arrays per name and block (flat), and the offset after the section."""
    r = Reader(data, offset)
    out = {k: [] for k in ("history", "cep", "urcs_n", "rot_n1", "eps_n", "element_vol")}
    for _ in range(model.nelblk):
        out["history"].append(r.doubles())
        out["cep"].append(r.doubles())
    for _ in range(model.nelblk):
        out["urcs_n"].append(r.doubles())
    r.key()
    for b in range(model.nelblk):
        out["rot_n1"].append(r.doubles() if geonl(model, b) else None)
    r.key()
    for _ in range(model.nelblk):
        out["eps_n"].append(r.doubles())
    r.key()
    for _ in range(model.nelblk):
        out["element_vol"].append(r.doubles())
    r.key()
    return out, r.pos
