"""Shared builders for the tests: synthetic models and element states.

States are produced by running the oracle's Newton driver (CPU) for a few
load steps, so they carry plastic history, rotations and stresses that a
WARP3D analysis would carry at the same point.
"""
from __future__ import annotations

import numpy as np

from warp3d_gb300 import abi
from warp3d_gb300.model import Bilinear, Model, cube_mesh, cube_mesh_hex20, cube_mesh_tet10
from warp3d_gb300.newton import NewtonDriver, uniaxial_bcs

MESHES = {abi.ETYPE_L3DISOP: cube_mesh, abi.ETYPE_Q3DISOP: cube_mesh_hex20, abi.ETYPE_TET10: cube_mesh_tet10}


def make_model(n=6, jitter=0.1, seed=12345, block_size=128, spans=None, beta=1.0, n_xyz=None, materials=None,
               etype=abi.ETYPE_L3DISOP, **kw):
    """kw: Model options (geonl, bbar, eps_bbar, qbar)."""
    nxyz = (n, n, n) if n_xyz is None else n_xyz
    coords, incid = MESHES[etype](n, jitter=jitter, seed=seed, n_xyz=nxyz)
    mats = materials or [Bilinear.from_hprime(200000.0, 0.3, 400.0, 2000.0, beta=beta)]
    return Model(coords, incid, block_size=block_size, block_spans=spans, materials=mats, etype=etype, **kw), nxyz


def loaded_state(model, nxyz, engine_cls, steps=3, strain_per_step=0.0015, shear_per_step=0.0,
                 tol=1e-8, seed=7, origins=None):
    """Runs `steps` converged load steps (uniaxial z plus optional x-shear
    of the top face) with an engine built by engine_cls(model), then
    returns (engine, driver, du_trial): du_trial is a perturbed increment
    for the next step, i.e. a mid-iteration state."""
    eng = engine_cls(model)
    fixed, topz = uniaxial_bcs(model, nxyz, origins=origins)
    top = (topz - 2) // 3
    fixed = np.union1d(fixed, 3 * top) if shear_per_step else fixed
    drv = NewtonDriver(model, eng, fixed, tol=tol)
    nz = nxyz[2]
    for s in range(1, steps + 1):
        imp = np.zeros(model.nodof)
        imp[topz] = strain_per_step * nz
        if shear_per_step:
            imp[3 * top] = shear_per_step * nz
        drv.step(s, imp)
    rng = np.random.Generator(np.random.PCG64(seed))
    du = np.zeros(model.nodof)
    du[topz] = strain_per_step * nz
    if shear_per_step:
        du[3 * top] = shear_per_step * nz
    # a plausible mid-iteration increment: scaled previous + noise
    du[drv.free] = drv.du_prev[drv.free] + rng.normal(0.0, 1e-4, size=len(drv.free))
    return eng, drv, du
