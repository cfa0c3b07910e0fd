"""The oracle against the committed golden fixtures (tests/golden).

Each fixture holds a small seeded model (8-node bricks, 20-node bricks and
10-node tetrahedra with mm01, 8-node bricks with mm10), an element state
loaded by three Newton steps, and the outputs of one recovery and one
tangent call from that state. Replaying the calls with the oracle must
give every output within 1e-13 relative (the restatement is
deterministic: a regression pin; the CUDA engine is held to the same
fixtures in test_gpu_golden.py)."""
import numpy as np
import pytest

import oracle
from tests.golden import golden_cases as gc

TOL = 1e-13


@pytest.mark.parametrize("name", list(gc.CASES))
def test_oracle_reproduces_golden(name):
    z = np.load(gc.path(name))
    model = gc.model_from(z)
    ora = oracle.Oracle(model, state=gc.state_from(z, model, "in"))
    ifv = np.zeros(model.nodof)
    st, info = ora.recover(int(z["step"]), int(z["iter"]), bool(z["extrapolated"]), model.c, z["u"], z["du"], ifv)
    assert st == 0
    est = model.estiff_blocks()
    ora.tanstf(int(z["step"]), int(z["iter"]), model.c, z["u"], z["du"], est)
    errs = gc.compare(z, model, ora.state, ifv, info, est)
    bad = {k: v for k, v in errs.items() if v > TOL}
    assert not bad, bad


def test_golden_fixtures_are_small_and_complete():
    for name in gc.CASES:
        z = np.load(gc.path(name))
        model = gc.model_from(z)
        assert model.noelem <= 12
        for nm in gc.STATE:
            for b in range(model.nelblk):
                assert f"in_{nm}_{b}" in z and f"out_{nm}_{b}" in z
        # the loaded state is past yield (mm01) or has slipped (mm10)
        h = np.concatenate([z[f"in_history_{b}"].reshape(-1) for b in range(model.nelblk)])
        assert np.any(h != 0.0)
