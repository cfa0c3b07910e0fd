"""The GPU engine (through the C-ABI) on WARP3D's own regression problem
verification/test24: the plain FP64 form reproduces the element-1 stress
WARP3D's checker compares (1e-4), with the oracle's Newton iteration
counts and its converged state to the convergence tolerance (each of the
21 steps stops at a 1e-8 residual, so element results equal to ~1e-15
leave end states ~1e-11 apart); the FP32 and TF32 tangents change only
the Newton path."""
import numpy as np
import pytest

import oracle
from tests import warp3d_test24 as t24
from warp3d_gb300 import abi

pytestmark = pytest.mark.gpu


def _engine(precision):
    from warp3d_gb300.engine import Engine

    def make(model):
        eng = Engine(model)
        eng.set_precision(precision)
        return eng
    return make


def test_gpu_engine_reproduces_the_reference_answer_and_the_oracle():
    d = t24.load()
    sig_o, u_o, its_o = t24.solve(oracle.Oracle, d)
    sig, u, its = t24.solve(_engine(abi.TANGENT_FP64), d)
    expected = float(d["expected_answer"])
    print(f"GPU element 1 center sigma_xx {sig[0]:.9f}, oracle {sig_o[0]:.9f}, WARP3D {expected}")
    assert abs(sig[0] / expected - 1.0) <= t24.CHECKER_RTOL
    assert its == its_o
    print(f"GPU vs oracle: sigma {np.max(np.abs(sig - sig_o)) / np.max(np.abs(sig_o)):.1e}, "
          f"u {np.max(np.abs(u - u_o)) / np.max(np.abs(u_o)):.1e}")
    assert np.max(np.abs(sig - sig_o)) <= 1e-8 * np.max(np.abs(sig_o))
    assert np.max(np.abs(u - u_o)) <= 1e-8 * np.max(np.abs(u_o))


@pytest.mark.parametrize("precision", [abi.TANGENT_FP32, abi.TANGENT_TF32])
def test_precision_forms_reach_the_same_answer(precision):
    d = t24.load()
    sig64, u64, _ = t24.solve(_engine(abi.TANGENT_FP64), d)
    sig, u, its = t24.solve(_engine(precision), d)
    print(f"precision {precision}: Newton iterations {its}, sigma_xx {sig[0]:.9f}")
    assert np.max(np.abs(u - u64)) <= 1e-6 * np.max(np.abs(u64))
    assert abs(sig[0] / float(d["expected_answer"]) - 1.0) <= t24.CHECKER_RTOL
