"""Golden cases of the element-block path: small seeded models, a loaded
element state, one recovery and one tangent call, all stored so that a
test can rebuild the model, restore the state and replay the calls.

A case is written by make_golden.py with the oracle (the CPU restatement
of WARP3D's element path) and read by tests/test_golden.py (the oracle
reproduces it: a regression pin) and tests/test_gpu_golden.py (the CUDA
engine reproduces it to 1e-12).

npz layout: model spec (coords; per part etype, incid, spans; per block
material numbers; crystal fields and Euler angles for mm10), the call
(step, iter, extrapolated, u, du), the input state (``in_<array>_<block>``)
and the outputs (``out_<array>_<block>``, ``ifv``, ``info``, ``ke_<block>``).
"""
from __future__ import annotations

import os

import numpy as np

from warp3d_gb300 import abi
from warp3d_gb300.model import Bilinear, Crystal, HostState, Model, Part, Umat, cube_mesh, random_orientations
from warp3d_gb300.newton import NewtonDriver, uniaxial_bcs

HERE = os.path.dirname(os.path.abspath(__file__))

STATE = HostState.NAMES
CRYSTAL_FIELDS = ("e", "nu", "harden_n", "tau_y", "tau_v", "theta_o", "voche_m", "iD_v", "k_o", "b", "atol",
                  "atol1", "rtol", "rtol1", "miter")


def path(name: str) -> str:
    return os.path.join(HERE, f"{name}.npz")


# ---- the cases (kept small: the fixtures are committed) -------------------
def _mm01_case(etype, nxyz, spans, shear, dyld=25.0, **opts):
    """dyld: yield-stress step between blocks; opts: Model options (geonl,
    bbar, eps_bbar)."""
    from tests.helpers import MESHES
    coords, incid = MESHES[etype](nxyz[0], jitter=0.08, seed=31, n_xyz=nxyz)
    mats = [Bilinear.from_hprime(200000.0, 0.3, 400.0 + dyld * b, 2000.0) for b in range(len(spans))]
    model = Model(coords, parts=[Part(etype, incid, spans, mats)], **opts)
    return model, nxyz, {"strain": 0.0015, "shear": shear, "extrapolate": False}


def _umat_case(etype, nxyz, spans, shear, **opts):
    """Material model 8 with the library's UMAT (the reference's example,
    Mises with linear kinematic hardening), one yield stress per block."""
    from tests.helpers import MESHES
    coords, incid = MESHES[etype](nxyz[0], jitter=0.08, seed=37, n_xyz=nxyz)
    mats = [Umat((200000.0, 0.3, 400.0 + 25.0 * b, 2000.0, 0.0)) for b in range(len(spans))]
    model = Model(coords, parts=[Part(etype, incid, spans, mats)], **opts)
    return model, nxyz, {"strain": 0.0015, "shear": shear, "extrapolate": False}


def _mm10_case(**opts):
    coords, incid = cube_mesh(1, jitter=0.05, seed=31, n_xyz=(1, 1, 2))
    model = Model(coords, incid, materials=[Crystal()], angles=random_orientations(2, 17), block_spans=[1, 1],
                  **opts)
    return model, (1, 1, 2), {"strain": 0.0005, "shear": 0.0, "extrapolate": True}


CASES = {
    "hex8_mm01": lambda: _mm01_case(abi.ETYPE_L3DISOP, (2, 2, 2), [5, 3], 0.001),
    "hex20_mm01": lambda: _mm01_case(abi.ETYPE_Q3DISOP, (2, 1, 1), [1, 1], 0.0),
    "tet10_mm01": lambda: _mm01_case(abi.ETYPE_TET10, (1, 1, 2), [7, 5], 0.0),
    "hex8_mm10": _mm10_case,
    # b-bar bricks (WARP3D's default l3disop formulation), finite strain
    # with a stabilization factor, and small displacement (rstgp2)
    "hex8_mm01_bbar": lambda: _mm01_case(abi.ETYPE_L3DISOP, (2, 2, 2), [5, 3], 0.001, bbar=True, eps_bbar=0.05),
    "hex8_mm01_small_bbar": lambda: _mm01_case(abi.ETYPE_L3DISOP, (2, 2, 2), [5, 3], 0.001, geonl=False,
                                               bbar=True),
    # (one yield stress: with the two of the other cases, the second load
    # step's Newton iterates grow to the element size and do not converge
    # without a line search, although the tangent matches central
    # differences of the internal forces to 1e-9)
    "hex8_mm10_bbar": lambda: _mm10_case(bbar=True),
    "tet10_mm01_small": lambda: _mm01_case(abi.ETYPE_TET10, (1, 1, 2), [7, 5], 0.0, dyld=0.0, geonl=False),
    # material model 8 (UMAT): finite-strain bricks, small-displacement
    # tetrahedra (one block: with two yield stresses on this 1 x 1 x 2
    # tetrahedral mesh the kinematic hardening of this UMAT -- and of mm01
    # with beta = 0 -- stalls the second step's Newton iterations)
    "hex8_umat": lambda: _umat_case(abi.ETYPE_L3DISOP, (2, 2, 2), [5, 3], 0.001),
    "tet10_umat_small": lambda: _umat_case(abi.ETYPE_TET10, (1, 1, 2), [12], 0.0, geonl=False),
}


# ---- model spec <-> npz ------------------------------------------------------
def model_spec(model: Model) -> dict:
    d = {"coords": model.coords, "nparts": np.int64(len(model.parts)), "geonl": np.int64(model.geonl),
         "qbar": np.int64(model.qbar), "bbar": np.int64(model.bbar), "eps_bbar": np.float64(model.eps_bbar)}
    for k, p in enumerate(model.parts):
        d[f"part{k}_etype"] = np.int64(p.etype)
        d[f"part{k}_incid"] = np.asarray(p.incid, dtype=np.int64)
        d[f"part{k}_spans"] = np.asarray(p.spans, dtype=np.int64)
    mats = model.block_material
    if isinstance(mats[0], Umat):
        d["umat"] = np.array([m.values() for m in mats])
    elif isinstance(mats[0], Crystal):
        d["crystal"] = np.array([float(getattr(mats[0], f)) for f in CRYSTAL_FIELDS])
        d["angles"] = np.asarray(model.elem_angles)
        d["dt"] = np.float64(model.dt)
    else:
        d["bilinear"] = np.array([[m.e, m.nu, m.yld, m.tan_e, m.beta] for m in mats])
    return d


def model_from(z) -> Model:
    parts = []
    for k in range(int(z["nparts"])):
        parts.append(Part(int(z[f"part{k}_etype"]), z[f"part{k}_incid"], [int(s) for s in z[f"part{k}_spans"]],
                          None))
    if "crystal" in z:
        vals = dict(zip(CRYSTAL_FIELDS, z["crystal"]))
        vals["miter"] = int(vals["miter"])
        cr = Crystal(**vals)
        p = parts[0]
        return Model(z["coords"], p.incid, etype=p.etype, block_spans=p.spans, materials=[cr],
                     angles=z["angles"], dt=float(z["dt"]), geonl=bool(z["geonl"]), qbar=bool(z["qbar"]),
                     bbar=bool(z["bbar"]) if "bbar" in z else False)
    mats = [Umat(tuple(row)) for row in z["umat"]] if "umat" in z else [Bilinear(*row) for row in z["bilinear"]]
    off = 0
    for p in parts:
        p.materials = mats[off:off + len(p.spans)]
        off += len(p.spans)
    bbar = bool(z["bbar"]) if "bbar" in z else False
    eps_bbar = float(z["eps_bbar"]) if "eps_bbar" in z else 0.0
    return Model(z["coords"], parts=parts, geonl=bool(z["geonl"]), qbar=bool(z["qbar"]), bbar=bbar,
                 eps_bbar=eps_bbar)


def state_from(z, model: Model, prefix: str) -> HostState:
    st = model.new_state()
    for name in STATE:
        arrs = getattr(st, name)
        for b in range(model.nelblk):
            arrs[b][...] = z[f"{prefix}_{name}_{b}"]
    return st


# ---- generation (oracle) ----------------------------------------------------
def generate(name: str) -> dict:
    import oracle
    model, nxyz, load = CASES[name]()
    ora = oracle.Oracle(model)
    fixed, topz = uniaxial_bcs(model, nxyz)
    top = (topz - 2) // 3
    if load["shear"]:
        fixed = np.union1d(fixed, 3 * top)
    drv = NewtonDriver(model, ora, fixed, tol=1e-8, maxit=60, extrapolate=load["extrapolate"])
    nz = nxyz[2]
    for s in range(1, 4):
        imp = np.zeros(model.nodof)
        imp[topz] = load["strain"] * nz
        if load["shear"]:
            imp[3 * top] = load["shear"] * nz
        drv.step(s, imp)
    rng = np.random.Generator(np.random.PCG64(77))
    du = np.zeros(model.nodof)
    du[topz] = load["strain"] * nz
    du[drv.free] = drv.du_prev[drv.free] + rng.normal(0.0, 1e-5, size=len(drv.free))
    u = drv.u.copy()
    out = model_spec(model)
    out.update({"step": np.int64(4), "iter": np.int64(1), "extrapolated": np.int64(0), "u": u, "du": du})
    state_in = ora.state.copy()
    for nm in STATE:
        for b, a in enumerate(getattr(state_in, nm)):
            out[f"in_{nm}_{b}"] = a
    o2 = oracle.Oracle(model, state=state_in.copy())
    ifv = np.zeros(model.nodof)
    st, info = o2.recover(4, 1, False, model.c, u, du, ifv)
    assert st == 0
    est = model.estiff_blocks()
    o2.tanstf(4, 1, model.c, u, du, est)
    for nm in STATE:
        for b, a in enumerate(getattr(o2.state, nm)):
            out[f"out_{nm}_{b}"] = a
    out["ifv"] = ifv
    out["info"] = np.array([info.internal_energy, info.plastic_work, info.sum_ifv, float(info.num_term_ifv)])
    for b, k in enumerate(est):
        out[f"ke_{b}"] = k
    return out


# ---- comparison ---------------------------------------------------------------
def compare(z, model: Model, state: HostState, ifv, info, est) -> dict:
    """Relative errors of every output against the fixture: per state
    array max |got - want| / max |want| (mm01's integer state word, history
    word 4, by its low 32 bits, reported as 0 or 1), ifv relative to the
    largest element force, the energy sums, Ke per element."""
    errs = {}

    def rel(a, b):
        a = np.asarray(a, dtype=np.float64).reshape(-1)
        b = np.asarray(b, dtype=np.float64).reshape(-1)
        den = np.max(np.abs(b)) if b.size else 0.0
        d = np.max(np.abs(a - b)) if b.size else 0.0
        return float(d / den) if den > 0 else float(d)

    for name in STATE:
        got = getattr(state, name)
        for b in range(model.nelblk):
            g = got[b]
            w = z[f"out_{name}_{b}"]
            # mm01 packs an integer state into the low word of history word 4
            # (a UMAT's history holds plain doubles there)
            mm01 = not model.block_crystal[b] and not model.block_umat[b]
            if name in ("history", "history1") and mm01:
                gi = g[..., 3].copy().view(np.int64) & 0xFFFFFFFF
                wi = w[..., 3].copy().view(np.int64) & 0xFFFFFFFF
                errs[f"{name}_state_word"] = max(errs.get(f"{name}_state_word", 0.0),
                                                 0.0 if np.array_equal(gi, wi) else 1.0)
                keep = [k for k in range(g.shape[-1]) if k != 3]
                g, w = g[..., keep], w[..., keep]
            errs[name] = max(errs.get(name, 0.0), rel(g, w))
    scale = max(np.max(np.abs(z[f"out_einfvec_{b}"])) for b in range(model.nelblk))
    errs["ifv"] = float(np.max(np.abs(np.asarray(ifv) - z["ifv"])) / scale)
    want = z["info"]
    got = [info.internal_energy, info.plastic_work, info.sum_ifv]
    for k, nm in enumerate(("internal_energy", "plastic_work", "sum_ifv")):
        errs[nm] = abs(got[k] - want[k]) / abs(want[k]) if want[k] != 0 else abs(got[k])
    errs["num_term_ifv"] = 0.0 if info.num_term_ifv == int(want[3]) else 1.0
    ke = 0.0
    for b in range(model.nelblk):
        w = z[f"ke_{b}"]
        d = np.max(np.abs(est[b] - w), axis=1) / np.max(np.abs(w), axis=1)
        ke = max(ke, float(np.max(d)))
    errs["ke"] = ke
    return errs
