"""The oracle against WARP3D's own regression problem
verification/test82/voche_model (mm10 crystal plasticity, one bcc crystal
per Gauss point, Voce hardening, 208 small-displacement b-bar bricks,
face pressures): the element-64 stress WARP3D's checker compares,
reproduced from the deck's data under the global loop of
tests/warp3d_test82.py within the checker's tolerance (1e-4 relative;
measured 4.0e-5 -- the deck converges each step only to a 1e-4 residual)."""
import numpy as np

import oracle
from tests import warp3d_test82 as t82


def test_fixture_holds_the_deck():
    d = t82.load()
    assert d["coords"].shape == (342, 3) and d["incid"].shape == (208, 8)
    assert list(d["flags"]) == [0, 1, 1]                # small displacement, bbar, center_output
    assert int(d["last_step"]) == 8 and int(d["expected_element"]) == 63
    # the face loads pull x = 1 with 1 and push z = 1 with 0.5 per unit step factor
    assert np.allclose(t82.load_pattern(d).reshape(-1, 3).sum(axis=0), [1.0, 0.0, -0.5])


def test_oracle_reproduces_the_reference_answer():
    d = t82.load()
    sig, u, its = t82.solve(oracle.Oracle, d)
    expected = float(d["expected_answer"])
    rel = abs(sig[0] / expected - 1.0)
    print(f"element 64 center sigma_xx {sig[0]:.6f} (WARP3D's checker: {expected}), rel {rel:.1e}, "
          f"Newton iterations {its}")
    assert rel <= t82.CHECKER_RTOL
