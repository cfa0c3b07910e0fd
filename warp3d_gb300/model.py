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

A model is a list of parts, each one element type (8-node brick
``l3disop``, 20-node brick ``q3disop``, 10-node tetrahedron) cut into
blocks of at most 128 elements, as WARP3D's blocking does. The synthetic
meshes stand in for input decks: structured cubes with optional seeded
nodal jitter.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import abi

HIST_MM01 = abi.HIST_MM01
HIST_MM10 = abi.HIST_MM10
HIST_UMAT = abi.HIST_UMAT
NSTR = 6
NSTRS = 9

# element type -> (nodes, Gauss points, integration order) as elprp1,
# elprp2 and the tet10 routines set iprops(2), (6), (5)
ELEMENT_TYPES = {
    abi.ETYPE_L3DISOP: (8, 8, 1),
    abi.ETYPE_Q3DISOP: (20, 27, 1),
    abi.ETYPE_TET10: (10, 4, 4),
}

# WARP3D 8-node brick node order in parent coordinates (xi, eta, zeta),
# src/derivs.f:302-325; the 20-node brick adds the mid-edge nodes 9-20 in
# the order of deriv1 (src/derivs.f:182-281)
HEX8_NODES = np.array(
    [[-1, -1, 1], [-1, -1, -1], [-1, 1, -1], [-1, 1, 1], [1, -1, 1], [1, -1, -1], [1, 1, -1], [1, 1, 1]],
    dtype=np.int64,
)
HEX20_NODES = np.concatenate([HEX8_NODES, np.array(
    [[-1, -1, 0], [-1, 0, -1], [-1, 1, 0], [-1, 0, 1], [1, -1, 0], [1, 0, -1], [1, 1, 0], [1, 0, 1],
     [0, -1, 1], [0, -1, -1], [0, 1, -1], [0, 1, 1]], dtype=np.int64)])
# 10-node tetrahedron: corners 1-4 then mid-edge nodes of edges
# (1,2) (2,3) (1,3) (1,4) (2,4) (3,4) (deriv6, src/derivs.f:606-662)
TET10_EDGES = [(0, 1), (1, 2), (0, 2), (0, 3), (1, 3), (2, 3)]


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


@dataclass
class Umat:
    """WARP3D material model 8, the Abaqus UMAT interface, with the UMAT
    compiled into the library (the reference's example: Mises plasticity
    with linear kinematic hardening). ``props`` are the material's umat
    values (dmatprp(151:200), up to 50); the example reads E, nu, yield
    stress, H' and the thermal expansion coefficient."""

    props: tuple = (200000.0, 0.3, 400.0, 2000.0, 0.0)

    def values(self) -> np.ndarray:
        v = np.zeros(abi.UMAT_NPROPS)
        v[:len(self.props)] = self.props
        return v


@dataclass
class Crystal:
    """mm10 crystal plasticity, WARP3D's crystal input (src/incrystal.f,
    defaults of src/mod_crystals.f:250-416): fcc or bcc (12-system) slip, isotropic
    elasticity, Voce hardening tau_tilde' = theta_0 sum |1 - (tau_tilde -
    tau_y)/tau_v|^m |gamma_dot|, slip rate gamma = dg/tau |tau_s/tau|^(n-1)
    tau_s. One crystal per Gauss point."""

    e: float = 200000.0
    nu: float = 0.3
    harden_n: float = 20.0
    tau_y: float = 90.0
    tau_v: float = 200.0
    theta_o: float = 500.0
    voche_m: float = 1.0
    iD_v: float = 0.0
    k_o: float = 0.0
    b: float = 2.87e-7
    atol: float = 1.0e-5
    atol1: float = 1.0e-5
    rtol: float = 5.0e-5
    rtol1: float = 1.0e-5
    miter: int = 30
    slip_type: int = 1          # 1 fcc, 2 bcc (12 systems)

    def struct(self) -> abi.Crystal:
        c = abi.Crystal()
        c.slip_type, c.elastic_type, c.h_type, c.miter = self.slip_type, 1, 1, self.miter
        for k in ("e", "nu", "harden_n", "tau_y", "tau_v", "theta_o", "voche_m", "iD_v", "k_o", "b", "atol",
                  "atol1", "rtol", "rtol1"):
            setattr(c, k, float(getattr(self, k)))
        return c


def random_orientations(n: int, seed: int = 4242) -> np.ndarray:
    """Euler angles (degrees, Kocks convention psi, theta, phi) uniform on
    SO(3): psi, phi uniform in [0, 360), cos(theta) uniform in [-1, 1]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    psi = rng.uniform(0.0, 360.0, n)
    phi = rng.uniform(0.0, 360.0, n)
    theta = np.degrees(np.arccos(rng.uniform(-1.0, 1.0, n)))
    return np.ascontiguousarray(np.stack([psi, theta, phi], axis=1))


def _lattice(nx, ny, nz, h, jitter, seed, level=1):
    """Nodes (i, j, k) of a lattice with `level` points per element edge
    (1: corners, 2: corners + mid-edge); interior corner nodes moved by
    U(-jitter, jitter)*h per coordinate, mid nodes placed at the centre of
    their (jittered) corners. Returns (positions of every lattice point,
    id function)."""
    mx, my, mz = level * nx, level * ny, level * nz
    ii, jj, kk = np.meshgrid(np.arange(mx + 1), np.arange(my + 1), np.arange(mz + 1), indexing="ij")
    P = np.stack([ii, jj, kk], axis=-1).astype(np.float64) * (h / level)
    if jitter > 0.0:
        rng = np.random.Generator(np.random.PCG64(seed))
        pert = rng.uniform(-jitter, jitter, size=(nx + 1, ny + 1, nz + 1, 3)) * h
        ci, cj, ck = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
        interior = (ci > 0) & (ci < nx) & (cj > 0) & (cj < ny) & (ck > 0) & (ck < nz)
        pert[~interior] = 0.0
        corner = P[::level, ::level, ::level] + pert
        if level == 1:
            P = corner
        else:
            # mid points: average of the lattice corners that bracket them
            def lerp(arr, axis):
                sl0 = [slice(None)] * 4
                sl1 = [slice(None)] * 4
                sl0[axis] = slice(0, -1)
                sl1[axis] = slice(1, None)
                mid = 0.5 * (arr[tuple(sl0)] + arr[tuple(sl1)])
                shape = list(arr.shape)
                shape[axis] = 2 * shape[axis] - 1
                out = np.empty(shape)
                so = [slice(None)] * 4
                so[axis] = slice(0, None, 2)
                out[tuple(so)] = arr
                so[axis] = slice(1, None, 2)
                out[tuple(so)] = mid
                return out
            P = lerp(lerp(lerp(corner, 0), 1), 2)
    return P


def cube_mesh(n: int, h: float = 1.0, jitter: float = 0.0, seed: int = 12345, n_xyz=None):
    """Structured brick mesh of 8-node bricks: nodes (i, j, k) at
    (i h, j h, k h); interior nodes moved by U(-jitter, jitter)*h per
    coordinate (numpy PCG64(seed)). Returns (coords[nnode,3],
    incid[noelem,8]) with 0-based node ids in WARP3D's hex8 node order."""
    nx, ny, nz = (n, n, n) if n_xyz is None else n_xyz
    P = _lattice(nx, ny, nz, h, jitter, seed, 1)
    nid = lambda i, j, k: i + (nx + 1) * (j + (ny + 1) * k)
    ii, jj, kk = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    coords = np.zeros(((nx + 1) * (ny + 1) * (nz + 1), 3))
    coords[nid(ii, jj, kk).ravel()] = P.reshape(-1, 3)
    ex, ey, ez = _cells(nx, ny, nz)
    incid = np.empty((nx * ny * nz, 8), dtype=np.int64)
    for a, (sx, sy, sz) in enumerate(HEX8_NODES):
        incid[:, a] = nid(ex + (sx > 0), ey + (sy > 0), ez + (sz > 0))
    return coords, incid


def _cells(nx, ny, nz):
    ex, ey, ez = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    order = np.argsort((ex + nx * (ey + ny * ez)).ravel())
    return ex.ravel()[order], ey.ravel()[order], ez.ravel()[order]


def cube_mesh_hex20(n: int, h: float = 1.0, jitter: float = 0.0, seed: int = 12345, n_xyz=None):
    """Structured mesh of 20-node bricks (q3disop): corner lattice as in
    cube_mesh, mid-edge nodes at the centres of their corners. Node ids are
    numbered over the half-step lattice points that are corners or edge
    mid-points."""
    nx, ny, nz = (n, n, n) if n_xyz is None else n_xyz
    P = _lattice(nx, ny, nz, h, jitter, seed, 2)
    ii, jj, kk = np.meshgrid(np.arange(2 * nx + 1), np.arange(2 * ny + 1), np.arange(2 * nz + 1), indexing="ij")
    odd = (ii % 2) + (jj % 2) + (kk % 2)
    keep = odd <= 1
    ids = -np.ones(ii.shape, dtype=np.int64)
    ids[keep] = np.arange(int(keep.sum()))
    coords = P[keep]
    ex, ey, ez = _cells(nx, ny, nz)
    incid = np.empty((nx * ny * nz, 20), dtype=np.int64)
    for a, (sx, sy, sz) in enumerate(HEX20_NODES):
        incid[:, a] = ids[2 * ex + 1 + sx, 2 * ey + 1 + sy, 2 * ez + 1 + sz]
    assert (incid >= 0).all()
    return coords, incid


def cube_mesh_tet10(n: int, h: float = 1.0, jitter: float = 0.0, seed: int = 12345, n_xyz=None):
    """Structured mesh of 10-node tetrahedra: every cell of the corner
    lattice split into 6 tetrahedra around its main diagonal, oriented so
    that det[J] > 0, mid-edge nodes at the centres of their corners."""
    nx, ny, nz = (n, n, n) if n_xyz is None else n_xyz
    P = _lattice(nx, ny, nz, h, jitter, seed, 2)
    ii, jj, kk = np.meshgrid(np.arange(2 * nx + 1), np.arange(2 * ny + 1), np.arange(2 * nz + 1), indexing="ij")
    # corners and every point that is the centre of a lattice edge used by
    # the tetrahedra (cell edges, face diagonals, the main diagonal)
    ex, ey, ez = _cells(nx, ny, nz)
    corners = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]])
    # Kuhn split around the diagonal 0-6
    tets = [(0, 1, 2, 6), (0, 2, 3, 6), (0, 3, 7, 6), (0, 7, 4, 6), (0, 4, 5, 6), (0, 5, 1, 6)]
    ne = nx * ny * nz * 6
    half = np.zeros((ne, 10, 3), dtype=np.int64)   # half-step lattice index of each node
    k = 0
    for t in tets:
        c = np.stack([2 * np.stack([ex, ey, ez], -1) + 2 * corners[v] for v in t], axis=1)   # (ncell, 4, 3)
        sl = slice(k, ne, 6)
        half[sl, :4] = c
        for m, (a, b) in enumerate(TET10_EDGES):
            half[sl, 4 + m] = (c[:, a] + c[:, b]) // 2
        k += 1
    used = np.unique(half.reshape(-1, 3), axis=0)
    ids = -np.ones(ii.shape, dtype=np.int64)
    ids[used[:, 0], used[:, 1], used[:, 2]] = np.arange(len(used))
    coords = P[used[:, 0], used[:, 1], used[:, 2]]
    incid = ids[half[..., 0], half[..., 1], half[..., 2]]
    # straight edges: every mid node at the centre of its two corners (the
    # Kuhn split uses the same face diagonals in neighbouring cells)
    for m, (a, b) in enumerate(TET10_EDGES):
        coords[incid[:, 4 + m]] = 0.5 * (coords[incid[:, a]] + coords[incid[:, b]])
    # orientation: (x2-x1, x3-x1, x4-x1) right-handed, else swap corners 3,4
    X = coords[incid[:, :4]]
    vol = np.einsum("ij,ij->i", np.cross(X[:, 1] - X[:, 0], X[:, 2] - X[:, 0]), X[:, 3] - X[:, 0])
    neg = vol < 0
    if neg.any():
        sw = incid[neg].copy()
        # swap corners 3 and 4; edges (1,2)(2,3)(1,3)(1,4)(2,4)(3,4) then
        # read (1,2)(2,4)(1,4)(1,3)(2,3)(4,3) of the old numbering
        perm = [0, 1, 3, 2, 4, 8, 7, 6, 5, 9]
        incid[neg] = sw[:, perm]
    return coords, incid


MESHES = {abi.ETYPE_L3DISOP: cube_mesh, abi.ETYPE_Q3DISOP: cube_mesh_hex20, abi.ETYPE_TET10: cube_mesh_tet10}


def mixed_mesh(parts_nx, ny: int, nz: int, h: float = 1.0, jitter: float = 0.0, seed: int = 12345,
               gap: int = 1):
    """Several structured bars side by side along x, one per element type:
    ``parts_nx`` is a list of (etype, nx); bar k is an nx x ny x nz cube
    mesh of that type (jittered with seed + k) shifted in x past the
    previous bars plus ``gap`` element lengths. The bars share no nodes.
    Returns (coords, [(etype, incid), ...], [(x0, nx), ...])."""
    coords, parts, origins = [], [], []
    x0, node0 = 0.0, 0
    for k, (etype, nx) in enumerate(parts_nx):
        c, inc = MESHES[etype](nx, h=h, jitter=jitter, seed=seed + k, n_xyz=(nx, ny, nz))
        c = c.copy()
        c[:, 0] += x0
        coords.append(c)
        parts.append((etype, inc + node0))
        origins.append((x0, nx))
        node0 += c.shape[0]
        x0 += (nx + gap) * h
    return np.concatenate(coords), parts, origins


def random_spans(ne: int, rng: np.random.Generator, lo: int = 16, hi: int = 128):
    """Block sizes uniform in [lo, hi] covering ne elements (the last block
    takes the remainder)."""
    spans, left = [], ne
    while left > 0:
        s = int(rng.integers(lo, hi + 1))
        s = min(s, left)
        spans.append(s)
        left -= s
    return spans


@dataclass
class Part:
    """One element type of a model: incidences and its blocking."""

    etype: int
    incid: np.ndarray                      # (n, nnode) 0-based node ids
    spans: list | None = None              # block sizes (default: block_size chunks)
    materials: list | None = None          # one Bilinear per block, or one for all


class Model:
    """A WARP3D model restricted to what the element-block path reads.

    ``Model(coords, incid)`` is a single-part model of 8-node bricks;
    ``Model(coords, parts=[Part(...), ...])`` mixes element types (blocks
    never mix types, as in WARP3D)."""

    def __init__(self, coords, incid=None, *, parts=None, block_size=128, etype=abi.ETYPE_L3DISOP, geonl=True,
                 bbar=False, qbar=True, materials=None, block_spans=None, angles=None, dt=1.0, eps_bbar=0.0,
                 asymmetric=False):
        if parts is None:
            parts = [Part(etype, np.asarray(incid), block_spans, materials)]
        self.coords = np.asarray(coords, dtype=np.float64)
        self.parts = parts
        self.block_size = block_size
        self.geonl, self.bbar, self.qbar = geonl, bbar, qbar
        self.eps_bbar = float(eps_bbar)
        # "assembly asymmetric on": full column-major element matrices
        self.asymmetric = bool(asymmetric)
        self.nnode = self.coords.shape[0]
        self.nodof = 3 * self.nnode
        self.ncoord = 3 * self.nnode
        # crdmap/dstmap: node n -> 3n (0-based)
        self.c = np.ascontiguousarray(self.coords.reshape(-1))
        spans, btype, bmat, bincid = [], [], [], []
        for p in parts:
            ne = p.incid.shape[0]
            sp = p.spans
            if sp is None:
                sp = [block_size] * (ne // block_size) + ([ne % block_size] if ne % block_size else [])
            assert sum(sp) == ne and all(1 <= s <= abi.MXVL for s in sp)
            mats = p.materials or [Bilinear.from_hprime(200000.0, 0.3, 400.0, 2000.0)]
            off = 0
            for b, s in enumerate(sp):
                spans.append(s)
                btype.append(p.etype)
                bmat.append(mats[b] if len(mats) == len(sp) else mats[0])
                bincid.append(p.incid[off:off + s])
                off += s
        self.spans = spans
        self.block_etype = btype
        self.block_material = bmat
        self.nelblk = len(spans)
        self.noelem = int(sum(spans))
        self.felem = np.concatenate([[0], np.cumsum(spans)[:-1]]).astype(np.int64)
        self.elblks = np.zeros((self.nelblk, 3), dtype=np.int32)
        self.elblks[:, 0] = spans
        self.elblks[:, 1] = self.felem + 1
        self.block_nnode = [ELEMENT_TYPES[t][0] for t in btype]
        self.block_ngp = [ELEMENT_TYPES[t][1] for t in btype]
        self.block_totdof = [3 * n for n in self.block_nnode]
        self.block_utsz = [d * (d + 1) // 2 for d in self.block_totdof]
        # rows of estiff_blocks(blk)%ptr: utsz, or totdof**2 with asymmetric
        # assembly (src/tanstf.f:223-225)
        self.block_ek_rows = [d * d if self.asymmetric else u for d, u in zip(self.block_totdof, self.block_utsz)]
        self._block_incid = bincid
        self.block_crystal = [isinstance(m, Crystal) for m in bmat]
        self.block_umat = [isinstance(m, Umat) for m in bmat]
        self.block_hist = [HIST_MM10 if cr else HIST_UMAT if um else HIST_MM01
                           for cr, um in zip(self.block_crystal, self.block_umat)]
        self.dt = float(dt)
        self.crystals = []
        self.elem_crystal = np.full(self.noelem, -1, dtype=np.int32)
        for b, m in enumerate(bmat):
            if isinstance(m, Crystal):
                if m not in self.crystals:
                    self.crystals.append(m)
                f = int(self.felem[b])
                self.elem_crystal[f:f + spans[b]] = self.crystals.index(m)
        self.elem_angles = (np.zeros((self.noelem, 3)) if angles is None
                            else np.ascontiguousarray(np.asarray(angles, dtype=np.float64).reshape(self.noelem, 3)))
        self.uniform = len(set(btype)) == 1
        # single-type conveniences
        t0 = btype[0]
        self.etype = t0
        self.nnode_el, self.ngp = ELEMENT_TYPES[t0][0], ELEMENT_TYPES[t0][1]
        self.totdof = 3 * self.nnode_el
        self.utsz = self.totdof * (self.totdof + 1) // 2
        self.ek_rows = self.totdof * self.totdof if self.asymmetric else self.utsz
        self.incid = np.concatenate(bincid) if self.uniform else None
        self._tables()

    # -- property tables (src/elprp.f elprp1/elprp2, src/mod_main.f:47-52) --
    def _tables(self):
        ne = self.noelem
        self.props = np.zeros((ne, abi.MXELPR), dtype=np.float32)
        self.iprops = np.zeros((ne, abi.MXELPR), dtype=np.int32)
        self.lprops = np.zeros((ne, abi.MXELPR), dtype=np.int32)
        # umat values per element (rknstr's local_work%umat_props); only
        # passed when the model has UMAT blocks
        self.umat_props = np.zeros((ne, abi.UMAT_NPROPS)) if any(self.block_umat) else None
        self.edest = []
        for b in range(self.nelblk):
            f, s, t = self.felem[b], self.spans[b], self.block_etype[b]
            nn, ngp, order = ELEMENT_TYPES[t]
            rows = slice(f, f + s)
            self.iprops[rows, 0] = t
            self.iprops[rows, 1] = nn
            self.iprops[rows, 2] = 3 * nn * 65536 + 6
            self.iprops[rows, 3] = 3
            self.iprops[rows, 4] = order
            self.iprops[rows, 5] = ngp
            mat = self.block_material[b]
            self.iprops[rows, 24] = (abi.MAT_CRYSTAL if isinstance(mat, Crystal) else
                                     abi.MAT_UMAT if isinstance(mat, Umat) else abi.MAT_BILINEAR)
            self.iprops[rows, 37] = 1
            self.lprops[rows, 17] = 1 if self.geonl else 0
            # b-bar is an option of the 8-node brick only (elprp.f sets
            # lprops(19) false for every other type)
            self.lprops[rows, 18] = 1 if (self.bbar and t == abi.ETYPE_L3DISOP) else 0
            if isinstance(mat, Crystal):
                self.props[rows, 6] = np.float32(mat.e)
                self.props[rows, 7] = np.float32(mat.nu)
            elif isinstance(mat, Umat):
                self.umat_props[rows] = mat.values()
            else:
                for k, v in mat.props_values().items():
                    self.props[rows, k - 1] = v
            nodes = self._block_incid[b]                     # (span, nn)
            d = np.empty((s, 3 * nn), dtype=np.int32)
            for k in range(3):
                d[:, k * nn:(k + 1) * nn] = 3 * nodes + k + 1   # 1-based, u1..un, v1..vn, w1..wn
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
        if self.crystals:
            self._crys = (abi.Crystal * len(self.crystals))(*[c.struct() for c in self.crystals])
            d.crystals = C.cast(self._crys, C.POINTER(abi.Crystal))
            d.ncrystals = len(self.crystals)
            d.elem_crystal = self.elem_crystal.ctypes.data_as(C.POINTER(C.c_int))
            d.elem_angles = self.elem_angles.ctypes.data_as(C.POINTER(C.c_double))
        d.dt = self.dt
        d.eps_bbar = self.eps_bbar
        d.asymmetric_assembly = 1 if self.asymmetric else 0
        if self.umat_props is not None:
            d.umat_props = self.umat_props.ctypes.data_as(C.POINTER(C.c_double))
        return d

    def new_state(self) -> "HostState":
        return HostState(self)

    def estiff_blocks(self):
        """Per block (span, rows): the packed upper triangle (utsz), or with
        asymmetric assembly the full matrix, column-major (totdof**2)."""
        return [np.zeros((s, u)) for s, u in zip(self.spans, self.block_ek_rows)]


def _ptrs(arrs):
    """C array of the arrays' data addresses (a ctypes view of a numpy
    address vector: about 0.3 us per array instead of a ctypes pointer
    object each); callers cast it to the pointer-to-pointer they need."""
    addr = np.fromiter((a.__array_interface__["data"][0] for a in arrs), dtype=np.uintp, count=len(arrs))
    return (C.c_void_p * len(arrs)).from_buffer(addr)


class HostState:
    """Host copies of the blocked element state, initialised as WARP3D
    does: zeros, with rot_n1 = identity (src/reopen.f:1912-1915)."""

    NAMES = ("history", "history1", "urcs_n", "urcs_n1", "eps_n", "eps_n1", "rot_n1", "cep", "einfvec",
             "element_vol")

    def __init__(self, model: Model):
        self.model = model
        sp, ng, td, hs = model.spans, model.block_ngp, model.block_totdof, model.block_hist
        self.history = [np.zeros((s, g, h)) for s, g, h in zip(sp, ng, hs)]
        self.history1 = [np.zeros((s, g, h)) for s, g, h in zip(sp, ng, hs)]
        self.urcs_n = [np.zeros((s, g, NSTRS)) for s, g in zip(sp, ng)]
        self.urcs_n1 = [np.zeros((s, g, NSTRS)) for s, g in zip(sp, ng)]
        self.eps_n = [np.zeros((s, g, NSTR)) for s, g in zip(sp, ng)]
        self.eps_n1 = [np.zeros((s, g, NSTR)) for s, g in zip(sp, ng)]
        self.rot_n1 = []
        for s, g in zip(sp, ng):
            r = np.zeros((s, g, 9))
            r[:, :, 0] = r[:, :, 4] = r[:, :, 8] = 1.0
            self.rot_n1.append(r)
        self.cep = [np.zeros((g, s, 21)) for s, g in zip(sp, ng)]
        self.einfvec = [np.zeros((d, s)) for s, d in zip(sp, td)]
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
        """All blocks of one array, element-major (cep/einfvec per element);
        for mixed element types, the flattened per-element values."""
        arrs = getattr(self, name)
        if name == "cep":
            arrs = [a.transpose(1, 0, 2) for a in arrs]                        # (span, ngp, 21)
        elif name == "einfvec":
            arrs = [a.T for a in arrs]                                          # (span, totdof)
        if self.model.uniform:
            return np.concatenate(arrs)
        return np.concatenate([a.reshape(-1) for a in arrs])


def dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def block_ptrs(arrs):
    return _ptrs(arrs)
