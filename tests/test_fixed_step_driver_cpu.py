"""The world clock (world.FixedStepDriver) against the reference's own cases (FixedStepDriverTests.swift:4-139):
whole steps only, backlog reporting, decimal intervals, invalid and overflowing increments, subnormal steps, the
backlog cap and its saturating excess, and the dropped increment after the background."""
import math
import sys

import pytest

from bubblephysics_gb300.world import FixedStepDriver

TINY = 5e-324  # the least nonzero double


def test_accumulates_time_without_consuming_an_incomplete_step():
    d = FixedStepDriver(0.125)
    assert d.accumulate(0.0625) and not d.can_step and d.completed_steps == 0
    assert d.accumulate(0.3125)
    for _ in range(3):
        assert d.can_step
        d.complete_step()
    assert not d.can_step and d.simulation_time == 0.375 and d.backlog_seconds == 0


def test_persistent_backlog_is_reported_without_changing_the_step():
    d = FixedStepDriver(0.125, maximum_steps_per_advance=2)
    for expected in (0.75, 1.5):
        assert d.accumulate(1)
        for _ in range(d.maximum_steps_per_advance):
            d.complete_step()
        d.finish_advance()
        assert d.backlog_seconds == expected and d.fixed_time_step == 0.125
    assert d.consecutive_backlogged_advances == 2
    while d.can_step:
        d.complete_step()
    d.finish_advance()
    assert d.consecutive_backlogged_advances == 0 and d.simulation_time == 2


def test_decimal_intervals_do_not_lose_a_step_to_rounding():
    d = FixedStepDriver(0.1)
    assert d.accumulate(0.3)
    steps = 0
    while d.can_step:
        d.complete_step()
        steps += 1
    assert steps == 3 and abs(d.backlog_seconds) <= 1e-15


def test_invalid_time_and_overflow_leave_the_accumulator_untouched():
    d = FixedStepDriver(0.125)
    assert d.accumulate(0.0625)
    for invalid in (-1.0, math.nan, math.inf, -math.inf):
        assert not d.accumulate(invalid) and d.backlog_seconds == 0.0625
    assert d.accumulate(sys.float_info.max)
    assert not d.accumulate(sys.float_info.max)
    assert math.isfinite(d.backlog_seconds)


def test_rounding_tolerance_cannot_turn_half_a_subnormal_step_into_a_step():
    d = FixedStepDriver(TINY * 8)
    assert d.accumulate(TINY * 4) and not d.can_step


def test_subnormal_backlog_one_ulp_short_of_a_step_does_not_advance():
    step = 1e-309
    assert 0 < step < sys.float_info.min
    d = FixedStepDriver(step)
    below = math.nextafter(step, 0.0)
    assert d.accumulate(below) and not d.can_step
    assert d.accumulate(step - below) and d.can_step


def test_backlog_is_capped_and_the_excess_summed():
    d = FixedStepDriver(0.125, maximum_backlog=0.25)
    assert d.accumulate(10)
    assert d.backlog_seconds == 0.25 and d.discarded_backlog_seconds == pytest.approx(9.75, abs=1e-12)
    assert d.accumulate(0.125)
    assert d.backlog_seconds == 0.25 and d.discarded_backlog_seconds == pytest.approx(9.875, abs=1e-12)


def test_backlog_below_the_cap_is_never_discarded():
    d = FixedStepDriver(0.125, maximum_backlog=0.25)
    assert d.accumulate(0.1) and d.accumulate(0.15)
    assert d.backlog_seconds == pytest.approx(0.25, abs=1e-12) and d.discarded_backlog_seconds == pytest.approx(0, abs=1e-12)
    d.complete_step()
    assert d.accumulate(0.125)
    assert d.backlog_seconds == pytest.approx(0.25, abs=1e-12) and d.discarded_backlog_seconds == pytest.approx(0, abs=1e-12)


def test_a_cap_below_one_step_still_lets_a_step_happen():
    d = FixedStepDriver(0.5, maximum_backlog=0.25)
    assert d.accumulate(3) and d.can_step and d.backlog_seconds == 0.5


def test_capping_keeps_rejecting_non_finite_and_overflowing_time():
    d = FixedStepDriver(0.125, maximum_backlog=0.25)
    assert d.accumulate(0.0625)
    for invalid in (-1.0, math.nan, math.inf):
        assert not d.accumulate(invalid)
        assert d.backlog_seconds == 0.0625 and d.discarded_backlog_seconds == 0


def test_discarded_time_saturates_instead_of_overflowing():
    d = FixedStepDriver(0.125, maximum_backlog=0.25)
    for _ in range(3):
        assert d.accumulate(sys.float_info.max / 2)
    assert math.isfinite(d.discarded_backlog_seconds) and d.backlog_seconds == 0.25


def test_discard_next_advance_drops_only_the_next_increment():
    d = FixedStepDriver(0.125)
    assert d.accumulate(0.0625)
    d.discard_next_advance()
    assert d.accumulate(5)
    assert d.backlog_seconds == 0.0625 and d.discarded_backlog_seconds == 0
    assert d.accumulate(0.0625) and d.backlog_seconds == pytest.approx(0.125, abs=1e-12)


def test_discard_next_advance_still_rejects_invalid_time_without_consuming_the_discard():
    d = FixedStepDriver(0.125)
    d.discard_next_advance()
    assert not d.accumulate(-1)
    assert d.accumulate(1) and d.backlog_seconds == 0


def test_world_reports_advance_issues():
    from bubblephysics_gb300.world import AdvanceIssue, BubbleWorld, WorldConfiguration
    w = BubbleWorld(WorldConfiguration((0.0, 0.0, 100.0, 100.0)))
    w.advance(math.nan)
    assert w.diagnostics.last_advance_issue == AdvanceIssue.INVALID_TIME_DELTA
    w.advance(1.0 / 60)
    assert w.diagnostics.last_advance_issue is None and w.last_frame.step_index == 1
    w.enter_background()
    w.become_active()
    w.advance(10.0)  # the time spent away is dropped
    assert w.last_frame.step_index == 1 and w.diagnostics.backlog_seconds == pytest.approx(0.0, abs=1e-12)


def test_interpolation_fraction_is_the_backlog_over_the_step():
    """InterpolationFractionTests.swift:5-29: alpha = backlog / step, clamped to [0, 1]."""
    d = FixedStepDriver(0.125)
    assert d.interpolation_fraction == 0
    assert d.accumulate(0.03125) and d.interpolation_fraction == pytest.approx(0.25, abs=1e-12)
    assert d.accumulate(0.0625) and d.interpolation_fraction == pytest.approx(0.75, abs=1e-12)
    d = FixedStepDriver(0.125)
    assert d.accumulate(0.3125) and d.interpolation_fraction == 1
    d.complete_step()
    assert d.backlog_seconds == pytest.approx(0.1875, abs=1e-12) and d.interpolation_fraction == 1
    d.complete_step()
    assert d.interpolation_fraction == pytest.approx(0.5, abs=1e-12)
    d = FixedStepDriver(0.125)
    assert d.accumulate(0.125)
    d.complete_step()
    assert d.interpolation_fraction == 0
