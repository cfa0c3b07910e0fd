"""The CUDA engine against the committed golden fixtures (tests/golden):
one recovery and one tangent call from each fixture's stored element
state reproduce the stored oracle outputs to 1e-12 relative (Ke per
element, state arrays, ifv, energy sums), in the plain FP64 form."""
import numpy as np
import pytest

from tests.golden import golden_cases as gc

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.mark.parametrize("name", list(gc.CASES))
def test_engine_reproduces_golden(name):
    from warp3d_gb300.engine import Engine
    z = np.load(gc.path(name))
    model = gc.model_from(z)
    eng = Engine(model)
    eng.upload(gc.state_from(z, model, "in"))
    ifv = np.zeros(model.nodof)
    step, it = int(z["step"]), int(z["iter"])
    st, info = eng.recover(step, it, bool(z["extrapolated"]), model.c, z["u"], z["du"], ifv)
    assert st == 0
    est = model.estiff_blocks()
    eng.tanstf(step, it, model.c, z["u"], z["du"], est)
    got = model.new_state()
    eng.download(got)
    errs = gc.compare(z, model, got, ifv, info, est)
    print(name, {k: f"{v:.1e}" for k, v in errs.items()})
    bad = {k: v for k, v in errs.items() if v > TOL}
    assert not bad, bad
