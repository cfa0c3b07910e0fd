"""WARP3D-style model tables for the element-block engine.

Builds what WARP3D holds after input processing -- coordinates ``c``,
element property tables ``props/iprops/lprops`` (43 x noelem, float32 /
int32 / logical), blocking ``elblks`` and the per-block index tables
``edest``/``cdest`` -- plus the host copies of the blocked element state
(module elem_block_data, src/mod_eleblocks.f:17-150).

numpy arrays are laid out so that their C order equals the Fortran order
of the reference arrays:
  history (span, ngp, hist)   == Fortran (hist, ngp, span)
  urcs    (span, ngp, 9), eps (span, ngp, 6), rot (span, ngp, 9)
  cep     (ngp, span, 21)     == Fortran (21, span, ngp)
  estiff  (span, utsz)        == Fortran (utsz, span)
  einfvec (totdof, span)      == Fortran (span, totdof)
  edest   (span, totdof)      == Fortran (totdof, span)

The synthetic meshes stand in for WARP3D input decks: structured cubes of
8-node bricks (element type l3disop) with optional seeded nodal jitter.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import abi

HIST_MM01 = 11
NSTR = 6
NSTRS = 9

# WARP3D 8-node brick node order in parent coordinates (xi, eta, zeta),
# src/derivs.f:302-325
HEX8_NODES = np.array(
    [[-1, -1, 1], [-1, -1, -1], [-1, 1, -1], [-1, 1, 1], [1, -1, 1], [1, -1, -1], [1, 1, -1], [1, 1, 1]],
    dtype=np.int64,
)


@dataclass
class Bilinear:
    """mm01 bilinear Mises material, WARP3D input ``properties bilinear
    e .. nu .. yld_pt .. tan_e .. beta ..`` (src/inmat.f). beta = 1 is
    isotropic hardening, 0 kinematic."""

    e: float
    nu: float
    yld: float
    tan_e: float
    beta: float = 1.0

    @staticmethod
    def from_hprime(e: float, nu: float, yld: float, hprime: float, beta: float = 1.0) -> "Bilinear":
        return Bilinear(e, nu, yld, e * hprime / (e + hprime), beta)

    def props_values(self) -> dict:
        """Entries of props(:, elem) as elprp2 stores them (src/elprp.f:629-665):
        single precision, with H' = (E*Et)/(E-Et) evaluated in float32."""
        e = np.float32(self.e)
        et = np.float32(self.tan_e)
        with np.errstate(all="ignore"):
            h = np.float32(np.float32(e * et) / np.float32(e - et))
        return {7: e, 8: np.float32(self.nu), 14: np.float32(self.beta), 15: h, 23: np.float32(self.yld)}


def cube_mesh(n: int, h: float = 1.0, jitter: float = 0.0, seed: int = 12345, n_xyz=None):
    """Structured brick mesh: nodes (i, j, k) at (i h, j h, k h); interior
    nodes moved by U(-jitter, jitter)*h per coordinate (numpy PCG64(seed)).
    Returns (coords[nnode,3], incid[noelem,8]) with 0-based node ids in
    WARP3D's hex8 node order."""
    nx, ny, nz = (n, n, n) if n_xyz is None else n_xyz
    ii, jj, kk = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    # node id = i + (nx+1)*(j + (ny+1)*k)
    coords = np.zeros(((nx + 1) * (ny + 1) * (nz + 1), 3))
    nid = lambda i, j, k: i + (nx + 1) * (j + (ny + 1) * k)
    ids = nid(ii, jj, kk).ravel()
    coords[ids, 0] = ii.ravel() * h
    coords[ids, 1] = jj.ravel() * h
    coords[ids, 2] = kk.ravel() * h
    if jitter > 0.0:
        rng = np.random.Generator(np.random.PCG64(seed))
        pert = rng.uniform(-jitter, jitter, size=coords.shape) * h
        interior = (
            (ii > 0) & (ii < nx) & (jj > 0) & (jj < ny) & (kk > 0) & (kk < nz)
        ).ravel()
        mask = np.zeros(len(coords), dtype=bool)
        mask[ids[interior]] = True
        coords[mask] += pert[mask]
    ex, ey, ez = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    # element id = ex + nx*(ey + ny*ez)
    order = np.argsort((ex + nx * (ey + ny * ez)).ravel())
    ex, ey, ez = ex.ravel()[order], ey.ravel()[order], ez.ravel()[order]
    incid = np.empty((nx * ny * nz, 8), dtype=np.int64)
    for a, (sx, sy, sz) in enumerate(HEX8_NODES):
        incid[:, a] = nid(ex + (sx > 0), ey + (sy > 0), ez + (sz > 0))
    return coords, incid


@dataclass
class Model:
    """A WARP3D model restricted to what the element-block path reads."""

    coords: np.ndarray            # (nnode, 3)
    incid: np.ndarray             # (noelem, nnode_per_elem), 0-based
    block_size: int = 128
    etype: int = abi.ETYPE_L3DISOP
    geonl: bool = True
    bbar: bool = False
    qbar: bool = True
    materials: list = field(default_factory=list)   # one Bilinear per block or one for all
    block_spans: list | None = None

    def __post_init__(self):
        self.nnode_el = self.incid.shape[1]
        self.ngp = 8
        self.totdof = 3 * self.nnode_el
        self.utsz = self.totdof * (self.totdof + 1) // 2
        self.noelem = self.incid.shape[0]
        self.nnode = self.coords.shape[0]
        self.nodof = 3 * self.nnode
        self.ncoord = 3 * self.nnode
        # crdmap/dstmap: node n -> 3n (0-based)
        self.c = np.ascontiguousarray(self.coords.reshape(-1))
        spans = self.block_spans
        if spans is None:
            spans = [self.block_size] * (self.noelem // self.block_size)
            if self.noelem % self.block_size:
                spans.append(self.noelem % self.block_size)
        assert sum(spans) == self.noelem and all(1 <= s <= abi.MXVL for s in spans)
        self.spans = list(spans)
        self.nelblk = len(spans)
        self.felem = np.concatenate([[0], np.cumsum(spans)[:-1]]).astype(np.int64)
        self.elblks = np.zeros((self.nelblk, 3), dtype=np.int32)
        self.elblks[:, 0] = spans
        self.elblks[:, 1] = self.felem + 1
        self._tables()

    # -- property tables (src/elprp.f elprp2, src/mod_main.f:47-52) ----
    def _tables(self):
        ne = self.noelem
        self.props = np.zeros((ne, abi.MXELPR), dtype=np.float32)
        self.iprops = np.zeros((ne, abi.MXELPR), dtype=np.int32)
        self.lprops = np.zeros((ne, abi.MXELPR), dtype=np.int32)
        self.iprops[:, 0] = self.etype
        self.iprops[:, 1] = self.nnode_el
        self.iprops[:, 2] = 24 * 65536 + 6
        self.iprops[:, 3] = 3
        self.iprops[:, 4] = 1          # 2x2x2 for l3disop
        self.iprops[:, 5] = self.ngp
        self.iprops[:, 24] = abi.MAT_BILINEAR
        self.iprops[:, 37] = 1
        self.lprops[:, 17] = 1 if self.geonl else 0
        self.lprops[:, 18] = 1 if self.bbar else 0
        mats = self.materials or [Bilinear.from_hprime(200000.0, 0.3, 400.0, 2000.0)]
        for b in range(self.nelblk):
            m = mats[b] if len(mats) == self.nelblk else mats[0]
            f, s = self.felem[b], self.spans[b]
            for k, v in m.props_values().items():
                self.props[f:f + s, k - 1] = v
        # edest/cdest per block: (span, totdof) with u1..un, v1..vn, w1..wn
        nn = self.nnode_el
        self.edest = []
        for b in range(self.nelblk):
            f, s = self.felem[b], self.spans[b]
            nodes = self.incid[f:f + s]                       # (span, nn)
            d = np.empty((s, 3 * nn), dtype=np.int32)
            for k in range(3):
                d[:, k * nn:(k + 1) * nn] = 3 * nodes + k + 1   # 1-based
            self.edest.append(np.ascontiguousarray(d))
        self.cdest = [e.copy() for e in self.edest]

    def desc(self) -> abi.ModelDesc:
        """ModelDesc over this model's arrays (keeps references alive)."""
        self._ed_ptrs = (C.POINTER(C.c_int) * self.nelblk)(
            *[e.ctypes.data_as(C.POINTER(C.c_int)) for e in self.edest])
        self._cd_ptrs = (C.POINTER(C.c_int) * self.nelblk)(
            *[e.ctypes.data_as(C.POINTER(C.c_int)) for e in self.cdest])
        d = abi.ModelDesc()
        d.nelblk = self.nelblk
        d.elblks = self.elblks.ctypes.data_as(C.POINTER(C.c_int))
        d.noelem = self.noelem
        d.props = self.props.ctypes.data_as(C.POINTER(C.c_float))
        d.iprops = self.iprops.ctypes.data_as(C.POINTER(C.c_int))
        d.lprops = self.lprops.ctypes.data_as(C.POINTER(C.c_int))
        d.edest = C.cast(self._ed_ptrs, C.POINTER(C.POINTER(C.c_int)))
        d.cdest = C.cast(self._cd_ptrs, C.POINTER(C.POINTER(C.c_int)))
        d.nodof = self.nodof
        d.ncoord = self.ncoord
        d.qbar_flag = 1 if self.qbar else 0
        d.beta_fact = 1.0
        return d

    def new_state(self) -> "HostState":
        return HostState(self)

    def estiff_blocks(self):
        return [np.zeros((s, self.utsz)) for s in self.spans]


def _ptrs(arrs):
    return (C.POINTER(C.c_double) * len(arrs))(*[a.ctypes.data_as(C.POINTER(C.c_double)) for a in arrs])


class HostState:
    """Host copies of the blocked element state, initialised as WARP3D
    does: zeros, with rot_n1 = identity (src/reopen.f:1912-1915)."""

    NAMES = ("history", "history1", "urcs_n", "urcs_n1", "eps_n", "eps_n1", "rot_n1", "cep", "einfvec",
             "element_vol")

    def __init__(self, model: Model):
        self.model = model
        ng = model.ngp
        sp = model.spans
        self.history = [np.zeros((s, ng, HIST_MM01)) for s in sp]
        self.history1 = [np.zeros((s, ng, HIST_MM01)) for s in sp]
        self.urcs_n = [np.zeros((s, ng, NSTRS)) for s in sp]
        self.urcs_n1 = [np.zeros((s, ng, NSTRS)) for s in sp]
        self.eps_n = [np.zeros((s, ng, NSTR)) for s in sp]
        self.eps_n1 = [np.zeros((s, ng, NSTR)) for s in sp]
        self.rot_n1 = []
        for s in sp:
            r = np.zeros((s, ng, 9))
            r[:, :, 0] = r[:, :, 4] = r[:, :, 8] = 1.0
            self.rot_n1.append(r)
        self.cep = [np.zeros((ng, s, 21)) for s in sp]
        self.einfvec = [np.zeros((model.totdof, s)) for s in sp]
        self.element_vol = [np.zeros(s) for s in sp]

    def copy(self) -> "HostState":
        o = HostState.__new__(HostState)
        o.model = self.model
        for n in self.NAMES:
            setattr(o, n, [a.copy() for a in getattr(self, n)])
        return o

    def struct(self, names=None) -> abi.BlockState:
        """BlockState with pointers to the selected arrays (others NULL)."""
        names = self.NAMES if names is None else names
        self._keep = {}
        s = abi.BlockState()
        for n in names:
            p = _ptrs(getattr(self, n))
            self._keep[n] = p
            setattr(s, n, C.cast(p, C.POINTER(C.POINTER(C.c_double))))
        return s

    def concat(self, name: str) -> np.ndarray:
        """All blocks of one array, element-major (cep/einfvec per element)."""
        arrs = getattr(self, name)
        if name == "cep":
            return np.concatenate([a.transpose(1, 0, 2) for a in arrs])      # (noelem, ngp, 21)
        if name == "einfvec":
            return np.concatenate([a.T for a in arrs])                        # (noelem, totdof)
        return np.concatenate(arrs)


def dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def block_ptrs(arrs):
    return _ptrs(arrs)
