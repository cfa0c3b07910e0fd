"""The oracle against WARP3D's own regression problem verification/test24
(hollow sphere under internal pressure: 45 finite-strain b-bar 8-node
bricks, bilinear Mises, skew constraints, nodal forces in 21 steps): the
element-1 stress that WARP3D's checker compares, reproduced from the
deck's data by the oracle under the global loop of tests/warp3d_test24.py,
within the checker's own tolerance (1e-4 relative; measured 3.6e-6)."""
import numpy as np

import oracle
from tests import warp3d_test24 as t24


def test_fixture_holds_the_deck():
    d = t24.load()
    assert d["coords"].shape == (96, 3) and d["incid"].shape == (45, 8)
    assert d["incid"].min() == 0 and d["incid"].max() == 95
    assert list(d["flags"]) == [1, 1, 1]                # nonlinear, bbar, center_output
    assert len(d["step_factors"]) == 21 and np.isclose(d["step_factors"].sum(), 5.0)
    # the nodal rotation matrices are orthonormal to the deck's digits
    for T in d["trn_mats"]:
        assert np.abs(T @ T.T - np.eye(3)).max() < 1e-6


def test_oracle_reproduces_the_reference_answer():
    d = t24.load()
    sig, u, its = t24.solve(oracle.Oracle, d)
    expected = float(d["expected_answer"])
    rel = abs(sig[0] / expected - 1.0)
    print(f"element 1 center sigma_xx {sig[0]:.6f} (WARP3D's checker: {expected}), rel {rel:.1e}, "
          f"Newton iterations {its}")
    assert rel <= t24.CHECKER_RTOL
    # the rest of the printed row is consistent with the axisymmetric
    # problem: hoop stresses equal, shear small against them
    assert abs(sig[1] / sig[2] - 1.0) < 2e-3
