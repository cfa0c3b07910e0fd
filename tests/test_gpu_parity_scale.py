"""Parity of the CUDA engine with the oracle on models larger than the
per-call cases: a 16^3 jittered cube of 8-node bricks (4,096 elements,
32 blocks of 128, 32,768 Gauss points) and a model mixing 8-node bricks,
20-node bricks and tetrahedra in blocks of random size U{16..128} with a
yield stress drawn per block (U(250, 550) MPa), as in the batching-form
workload. Every output of one Newton iteration of element work is compared
on the whole model: urcs_n1, eps_n1, rot_n1, history1, cep, einfvec,
element volumes, ifv, the energy sums and Ke; plus the precision forms'
Ke against the FP64 oracle.

The state is that of the benchmark: load step 1 to 1% homogeneous
uniaxial strain (every Gauss point plastic), update, then step 2,
iteration 1 with a perturbed increment.

Tolerance (FP64 plain form): max |gpu - oracle| / max |oracle| per array
(per element for Ke) <= 1e-12.
"""
import numpy as np
import pytest

import oracle
from tests.conftest import rel_err
from warp3d_gb300 import abi
from warp3d_gb300.model import Bilinear, Model, Part, cube_mesh, mixed_mesh, random_spans

pytestmark = pytest.mark.gpu

TOL = 1e-12
# precision forms' Ke against the FP64 oracle, per element
TOL_FORMS = {abi.TANGENT_FP32: 2e-6, abi.TANGENT_TF32: 2e-3, abi.TANGENT_BF16: 1.5e-2,
             abi.TANGENT_TF32X3: 2e-5, abi.TANGENT_BF16X3: 1e-4}


def _loads(model, seed):
    X = model.coords
    u1 = ((np.diag([-0.005, -0.005, 0.01])) @ X.T).T.ravel()
    rng = np.random.Generator(np.random.PCG64(seed))
    du = ((np.diag([-0.0005, -0.0005, 0.001])) @ X.T).T.ravel() + rng.normal(0.0, 2e-5, model.nodof)
    return u1, du


def _run_both(model, u1, du):
    from warp3d_gb300.engine import Engine
    eng, ora = Engine(model), oracle.Oracle(model)
    z = np.zeros(model.nodof)
    fg, fo = np.zeros(model.nodof), np.zeros(model.nodof)
    assert eng.recover(1, 1, False, model.c, z, u1, fg)[0] == 0
    assert ora.recover(1, 1, False, model.c, z, u1, fo)[0] == 0
    eng.update()
    ora.update()
    st_g, info_g = eng.recover(2, 1, False, model.c, u1, du, fg)
    st_o, info_o = ora.recover(2, 1, False, model.c, u1, du, fo)
    assert st_g == st_o == 0
    kg, ko = model.estiff_blocks(), model.estiff_blocks()
    eng.tanstf(2, 1, model.c, u1, du, kg)
    ora.tanstf(2, 1, model.c, u1, du, ko)
    got = model.new_state()
    eng.download(got)
    errs = {n: rel_err(np.concatenate([a.ravel() for a in getattr(got, n)]),
                       np.concatenate([a.ravel() for a in getattr(ora.state, n)]))
            for n in ("urcs_n1", "eps_n1", "rot_n1", "history1", "cep", "einfvec", "element_vol")}
    errs["ifv"] = rel_err(fg, fo)
    errs["energy"] = rel_err([info_g.internal_energy, info_g.plastic_work], [info_o.internal_energy,
                                                                          info_o.plastic_work])
    errs["sum_ifv"] = rel_err([info_g.sum_ifv], [info_o.sum_ifv])
    errs["estiff"] = max(rel_err(a, b, axis=1) for a, b in zip(kg, ko))
    return eng, ko, errs


def _forms(eng, model, u1, du, ko):
    out = {}
    for p, tol in TOL_FORMS.items():
        eng.set_precision(p)
        kp = model.estiff_blocks()
        eng.tanstf(2, 1, model.c, u1, du, kp)
        out[p] = max(rel_err(a, b, axis=1) for a, b in zip(kp, ko))
        assert out[p] <= tol, (p, out[p])
    return out


def test_parity_16_cube_jittered():
    coords, incid = cube_mesh(16, jitter=0.1, seed=12345)
    model = Model(coords, incid, block_size=128,
                  materials=[Bilinear.from_hprime(200000.0, 0.3, 400.0, 2000.0, beta=1.0)])
    assert model.noelem == 4096 and model.nelblk == 32
    u1, du = _loads(model, 2024)
    eng, ko, errs = _run_both(model, u1, du)
    assert max(errs.values()) <= TOL, errs
    _forms(eng, model, u1, du, ko)
    eng.close()


def test_parity_mixed_types_random_spans_per_block_yield():
    rng = np.random.Generator(np.random.PCG64(2025))
    coords, parts, _ = mixed_mesh([(abi.ETYPE_L3DISOP, 12), (abi.ETYPE_Q3DISOP, 5), (abi.ETYPE_TET10, 3)],
                                  8, 8, jitter=0.05, seed=2025)
    plist = []
    for etype, inc in parts:
        spans = random_spans(inc.shape[0], rng, 16, 128)
        mats = [Bilinear.from_hprime(200000.0, 0.3, float(rng.uniform(250.0, 550.0)), 2000.0) for _ in spans]
        plist.append(Part(etype, inc, spans, mats))
    model = Model(coords, parts=plist)
    assert len(set(model.block_etype)) == 3 and model.nelblk >= 20
    assert len({m.yld for m in model.block_material}) == model.nelblk
    u1, du = _loads(model, 2026)
    eng, ko, errs = _run_both(model, u1, du)
    assert max(errs.values()) <= TOL, errs
    _forms(eng, model, u1, du, ko)
    eng.close()
