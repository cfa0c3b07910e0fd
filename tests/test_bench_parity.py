"""The benchmark's parity checker (bench.sub_model): the oracle replaying
a sample of blocks as a model of their own, from the same state, must
reproduce the outputs of those blocks in the whole model. CPU only: both
sides are the oracle, so the check is of the sampling (node map, block
order, materials, orientations), not of the CUDA engine."""
import numpy as np

import bench
import oracle
from tests.test_gpu_parity_types import _mixed_model
from warp3d_gb300 import abi


def _uniaxial(model, strain):
    X = model.coords
    F = np.diag([1 - strain / 2, 1 - strain / 2, 1 + strain])
    return ((F - np.eye(3)) @ X.T).T.ravel()


def test_sub_model_replays_the_sampled_blocks_of_a_mixed_model():
    model, _ = _mixed_model()
    u1 = _uniaxial(model, 0.01)
    rng = np.random.default_rng(3)
    du = _uniaxial(model, 0.001) + rng.normal(0.0, 2e-5, model.nodof)
    full = oracle.Oracle(model)
    ifv = np.zeros(model.nodof)
    assert full.recover(1, 1, False, model.c, np.zeros(model.nodof), u1, ifv)[0] == 0
    full.update()
    blocks = bench.spread_blocks(model, 2, types=(abi.ETYPE_L3DISOP, abi.ETYPE_Q3DISOP, abi.ETYPE_TET10))
    assert len({model.block_etype[b] for b in blocks}) == 3
    sub, dofs = bench.sub_model(model, blocks)
    pre = sub.new_state()
    for name in pre.NAMES:
        setattr(pre, name, [getattr(full.state, name)[b].copy() for b in blocks])
    assert full.recover(2, 1, False, model.c, u1, du, ifv)[0] == 0
    ke_full = model.estiff_blocks()
    full.tanstf(2, 1, model.c, u1, du, ke_full)
    part = oracle.Oracle(sub, state=pre)
    assert part.recover(2, 1, False, sub.c, u1[dofs], du[dofs], np.zeros(sub.nodof))[0] == 0
    ke_sub = sub.estiff_blocks()
    part.tanstf(2, 1, sub.c, u1[dofs], du[dofs], ke_sub)
    for name in bench.PARITY_ARRAYS:
        for k, b in enumerate(blocks):
            np.testing.assert_array_equal(getattr(part.state, name)[k], getattr(full.state, name)[b], err_msg=name)
    assert bench._ke_err(ke_sub, [ke_full[b] for b in blocks]) == 0.0


def test_sub_model_keeps_crystal_orientations():
    from warp3d_gb300.model import Crystal, Model, cube_mesh, random_orientations
    coords, incid = cube_mesh(4)
    model = Model(coords, incid, block_size=16, materials=[Crystal()], angles=random_orientations(64, 7))
    blocks = [3, 1]
    sub, _ = bench.sub_model(model, blocks)
    np.testing.assert_array_equal(sub.elem_angles[:16], model.elem_angles[48:64])
    np.testing.assert_array_equal(sub.elem_angles[16:], model.elem_angles[16:32])
    assert sub.spans == [16, 16] and sub.crystals
