"""The world's clock through BubbleWorld.advance, against BubbleWorldTimeTests.swift:5-151: presentation time
accumulates into fixed steps of 0.125 s, one batch and many small advances complete the same steps, transactions
publish only at a step boundary, several steps keep every receipt and rejection in order, pause keeps the queue, a
persistent backlog drains without changing the step, invalid time consumes nothing, and ten seconds at once are
clamped to the backlog cap (at most eight steps per advance). No bubble is needed: the clock runs without a device
world."""
import math

from bubblephysics_gb300.world import AdvanceIssue, BubbleWorld, TransactionRejectionReason as R, WorldConfiguration, \
    WorldTransaction


def world(step=0.125, maximum_backlog=10.0):
    return BubbleWorld(WorldConfiguration((-10.0, -10.0, 10.0, 10.0), fixed_time_step=step,
                                          maximum_backlog=maximum_backlog))


def test_advance_accumulates_presentation_time_into_deterministic_fixed_steps():
    w = world()
    initial = w.advance(0.0625)
    assert (initial.step_index, initial.simulation_time, w.diagnostics.backlog_seconds) == (0, 0.0, 0.0625)
    frame = w.advance(0.3125)
    assert (frame.step_index, frame.simulation_time) == (3, 0.375)
    assert w.diagnostics.steps_in_last_advance == 3 and w.diagnostics.backlog_seconds == 0
    split = world()
    for _ in range(3):
        split_frame = split.advance(0.125)
    assert split_frame == frame


def test_one_second_at_once_and_sixty_presentation_intervals_complete_the_same_sixty_steps():
    batched = world(1.0 / 60, 10.0)
    frame = batched.advance(1.0)
    for _ in range(8):
        frame = batched.advance(0.0)
    split = world(1.0 / 60, 10.0)
    split_frame = split.advance(0.0)
    for _ in range(60):
        split_frame = split.advance(1.0 / 60)
    assert frame.step_index == 60 and split_frame.step_index == 60
    assert abs(batched.diagnostics.backlog_seconds) <= 1e-12 and abs(split.diagnostics.backlog_seconds) <= 1e-12


def test_transactions_publish_only_at_a_fixed_step_boundary():
    w = world()
    token = w.submit(WorldTransaction().set_global_force((0.0, -3.0)))
    assert not w.advance(0.0625).transaction_receipts and w.diagnostics.pending_transaction_count == 1
    complete = w.advance(0.0625)
    assert [r.token for r in complete.transaction_receipts] == [token] and w.diagnostics.pending_transaction_count == 0
    assert w.advance(0.0) == complete
    assert not w.advance(0.125).transaction_receipts


def test_several_steps_keep_every_receipt_and_rejection_in_order():
    w = world()
    first = w.submit(WorldTransaction().set_global_force((1.0, 0.0)))
    rejected = w.submit(WorldTransaction().remove(42))
    last = w.submit(WorldTransaction().set_global_force((2.0, 0.0)))
    assert len({first, rejected, last}) == 3
    frame = w.advance(0.375)
    assert frame.step_index == 3 and [r.token for r in frame.transaction_receipts] == [first, last]
    assert [(e.kind, e.token, e.rejection.operation_index, e.rejection.reason) for e in frame.events] == \
        [("transactionRejected", rejected, 0, R.OBJECT_NOT_FOUND)]


def test_pause_prevents_steps_but_keeps_the_queued_transaction():
    w = world()
    before = w.advance(0.0625)
    w.pause()
    w.pause()
    token = w.submit(WorldTransaction().set_global_force((1.0, 2.0)))
    assert w.advance(60.0) == before
    assert w.diagnostics.is_paused and w.diagnostics.backlog_seconds == 0.0625
    assert w.diagnostics.pending_transaction_count == 1
    w.resume()
    w.resume()
    resumed = w.advance(0.0625)
    assert resumed.step_index == 1 and [r.token for r in resumed.transaction_receipts] == [token]
    assert not w.diagnostics.is_paused


def test_a_persistent_backlog_drains_without_changing_the_configured_step():
    w = world(maximum_backlog=1000.0)
    first = w.advance(100.0)
    assert 0 < first.step_index and first.simulation_time < 100
    assert first.simulation_time + w.diagnostics.backlog_seconds == 100
    assert w.diagnostics.consecutive_backlogged_advances == 1
    second = w.advance(100.0)
    assert second.simulation_time + w.diagnostics.backlog_seconds == 200
    assert w.diagnostics.consecutive_backlogged_advances == 2
    final = second
    while w.diagnostics.backlog_seconds >= 0.125:
        final = w.advance(0.0)
    assert (final.step_index, final.simulation_time) == (1600, 200.0)
    assert w.configuration.fixed_time_step == 0.125 and w.diagnostics.consecutive_backlogged_advances == 0


def test_invalid_time_is_reported_without_consuming_time_or_transactions():
    w = world()
    initial = w.advance(0.0625)
    token = w.submit(WorldTransaction())
    for invalid in (-1.0, math.nan, math.inf, -math.inf):
        assert w.advance(invalid) == initial
        assert w.diagnostics.last_advance_issue == AdvanceIssue.INVALID_TIME_DELTA
        assert w.diagnostics.backlog_seconds == 0.0625 and w.diagnostics.pending_transaction_count == 1
    valid = w.advance(0.0625)
    assert [r.token for r in valid.transaction_receipts] == [token] and w.diagnostics.last_advance_issue is None


def test_ten_seconds_at_once_are_clamped_to_the_backlog_cap():
    w = world(1.0 / 60, 0.25)
    first = w.advance(10.0)
    assert first.step_index == 8  # at most eight steps per advance
    assert abs(w.diagnostics.backlog_seconds + first.simulation_time - 0.25) <= 1e-9
    assert abs(w.diagnostics.discarded_backlog_seconds - 9.75) <= 1e-9
    final = first
    for _ in range(2):
        final = w.advance(0.0)
    assert final.step_index == 15  # 0.25 s is exactly 15 steps of 1/60
    assert abs(w.diagnostics.discarded_backlog_seconds - 9.75) <= 1e-9
    w.advance(10.0)
    assert abs(w.diagnostics.discarded_backlog_seconds - 19.5) <= 1e-9  # later long gaps add to the sum


def test_a_backlog_below_the_cap_discards_nothing():
    w = world(maximum_backlog=0.25)
    w.advance(0.2)
    assert w.diagnostics.discarded_backlog_seconds == 0
