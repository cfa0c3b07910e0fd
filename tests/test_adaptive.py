"""WARP3D's adaptive subdivision of a load step (adapt_check) as the device
Newton loop applies it, with a fake increment that fails above a size."""
import pytest

from warp3d_gb300.solver import IncrementFailed, run_subdivided


def _attempts(limit):
    seen = []

    def attempt(f, after_cut):
        seen.append((f, after_cut))
        if f > limit:
            raise IncrementFailed(f"increment {f} too large")
    return attempt, seen


def test_whole_step_when_it_converges():
    attempt, seen = _attempts(2.0)
    done, cuts = run_subdivided(attempt, True)
    assert done == [1.0] and cuts == 0 and seen == [(1.0, False)]


def test_one_cut_into_four():
    attempt, seen = _attempts(0.3)
    done, cuts = run_subdivided(attempt, True)
    assert done == [0.25] * 4 and cuts == 1
    # the first sub-increment after the cut starts without extrapolation
    assert [a for _, a in seen] == [False, True, False, False, False]


def test_two_levels_down_to_a_sixteenth():
    attempt, _ = _attempts(0.1)
    done, cuts = run_subdivided(attempt, True)
    assert done == [1.0 / 16.0] * 16 and cuts == 5   # the step, then each quarter
    assert abs(sum(done) - 1.0) < 1e-15


def test_limit_reached_raises():
    attempt, _ = _attempts(0.01)
    with pytest.raises(RuntimeError, match="too large"):
        run_subdivided(attempt, True)


def test_not_adaptive_raises_at_once():
    attempt, seen = _attempts(0.5)
    with pytest.raises(RuntimeError):
        run_subdivided(attempt, False)
    assert len(seen) == 1


def test_eisenstat_walker_forcing_terms():
    from warp3d_gb300.solver import EW_ETA_MAX, ew_forcing
    # quadratic in the residual ratio, capped at eta_max
    assert ew_forcing(0.1, 1e-2, 1e-1, 1e-12) == pytest.approx(0.9 * 1e-2)
    assert ew_forcing(0.1, 0.9, 1.0, 1e-12) == EW_ETA_MAX
    # safeguard: a sudden drop after a loose solve keeps gamma eta^2
    assert ew_forcing(0.5, 1e-6, 1.0, 1e-12) == pytest.approx(0.9 * 0.25 if 0.9 * 0.25 < EW_ETA_MAX else EW_ETA_MAX)
    # never tighter than reaching the Newton target needs
    assert ew_forcing(1e-3, 1e-7, 1e-3, 1e-8) == pytest.approx(0.05)
