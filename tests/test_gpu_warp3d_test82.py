"""The GPU engine (through the C-ABI) on WARP3D's own regression problem
verification/test82/voche_model (mm10, bcc, Voce): the plain FP64 form
reproduces the element-64 stress WARP3D's checker compares (1e-4), with
the oracle's Newton iteration counts and its converged state to the
convergence tolerance; the FP32 tangent changes only the Newton path."""
import numpy as np
import pytest

import oracle
from tests import warp3d_test82 as t82
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
    d = t82.load()
    sig_o, u_o, its_o = t82.solve(oracle.Oracle, d)
    sig, u, its = t82.solve(_engine(abi.TANGENT_FP64), d)
    expected = float(d["expected_answer"])
    print(f"GPU element 64 center sigma_xx {sig[0]:.9f}, oracle {sig_o[0]:.9f}, WARP3D {expected}; "
          f"iterations {its}")
    assert abs(sig[0] / expected - 1.0) <= t82.CHECKER_RTOL
    assert its == its_o
    print(f"GPU vs oracle: sigma {np.max(np.abs(sig - sig_o)) / np.max(np.abs(sig_o)):.1e}, "
          f"u {np.max(np.abs(u - u_o)) / np.max(np.abs(u_o)):.1e}")
    assert np.max(np.abs(sig - sig_o)) <= 1e-7 * np.max(np.abs(sig_o))
    assert np.max(np.abs(u - u_o)) <= 1e-7 * np.max(np.abs(u_o))


def test_fp32_tangent_reaches_the_same_answer():
    d = t82.load()
    sig64, u64, _ = t82.solve(_engine(abi.TANGENT_FP64), d)
    sig, u, its = t82.solve(_engine(abi.TANGENT_FP32), d)
    print(f"FP32 tangent: Newton iterations {its}, sigma_xx {sig[0]:.9f}")
    assert np.max(np.abs(u - u64)) <= 1e-6 * np.max(np.abs(u64))
    assert abs(sig[0] / float(d["expected_answer"]) - 1.0) <= t82.CHECKER_RTOL
