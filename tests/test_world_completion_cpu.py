"""How a world completes, rejects or fails a step, against the reference's own cases
(BubbleWorldCompletionTests.swift:16-232), on a scripted stand-in device world: the candidate overflow counter
accumulates and the per-object maximum is the last step's; a failed step leaves both alone; solver errors other than a
failed command or a physics failure reject only the step (queue and time kept, retried at the next advance, the reason
in the diagnostics); a failed command ends the world and drops the queue; non-finite values end it with their own
reason; a failure after a completed step returns that step's frame and keeps only the unsimulated time."""
import numpy as np
import pytest

from bubblephysics_gb300 import _native as N
from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (AdvanceIssue, BubbleDescriptor, BubbleWorld, PhysicsMaterial, WorldConfiguration,
                                       WorldFailureReason, WorldRejectionReason, WorldTransaction)
from test_world_api_oracle_cpu import OracleBackedWorld

SCRIPT = []  # per device step: ("ok", overflow, maximum) | ("raise", status) | ("status", status)
CALLS = []


class ScriptedWorld(OracleBackedWorld):
    def step(self, steps):
        CALLS.append(1)
        action = SCRIPT.pop(0) if SCRIPT else ("ok", 0, 0)
        if action[0] == "raise":
            raise N.NativeError(action[1], "bp_world_step")
        status, reps = self.o.step(steps)
        if action[0] == "status":
            return action[1], reps
        reps["candidate_overflow"], reps["max_candidates_per_object"] = action[1], action[2]
        return status, reps


@pytest.fixture(autouse=True)
def scripted(monkeypatch):
    monkeypatch.setattr(W, "World", ScriptedWorld)
    monkeypatch.setattr(W, "default_context", lambda: None)
    SCRIPT.clear()
    CALLS.clear()


def world():
    w = BubbleWorld(WorldConfiguration((-10.0, -10.0, 10.0, 10.0), fixed_time_step=0.125, maximum_backlog=10.0))
    w.submit(WorldTransaction().update_physics_material("m", PhysicsMaterial(229.0))
             .add(BubbleDescriptor(1, (0.0, 0.0), 1.0, 1.0, "m")))
    return w


def test_candidate_overflow_accumulates_and_the_maximum_is_the_last_steps():
    SCRIPT.extend([("ok", 3, 7), ("ok", 0, 5), ("ok", 2, 9)])
    w = world()
    assert w.diagnostics.contact_candidate_overflow == 0
    for overflow, maximum in ((3, 7), (3, 5), (5, 9)):
        w.advance(0.125)
        assert (w.diagnostics.contact_candidate_overflow, w.diagnostics.maximum_contact_candidates_per_object) == \
            (overflow, maximum)


def test_a_failed_step_leaves_the_counters_alone():
    SCRIPT.extend([("ok", 4, 6), ("raise", N.E_INFLIGHT)])
    w = world()
    w.advance(0.125)
    w.advance(0.125)
    assert w.diagnostics.last_advance_issue == AdvanceIssue.STEP_FAILED
    assert (w.diagnostics.contact_candidate_overflow, w.diagnostics.maximum_contact_candidates_per_object) == (4, 6)


@pytest.mark.parametrize("status,reason", [(N.E_INVALID, WorldRejectionReason.INVALID_SNAPSHOT),
                                           (N.E_INFLIGHT, WorldRejectionReason.FRAME_IN_FLIGHT),
                                           (N.E_CAPACITY, WorldRejectionReason.UNEXPECTED),
                                           (N.E_ALLOC, WorldRejectionReason.UNEXPECTED)])
def test_non_terminal_solver_errors_reject_only_the_step(status, reason):
    SCRIPT.append(("raise", status))
    w = world()
    rejected = w.advance(0.125)
    d = w.diagnostics
    assert rejected.step_index == 0 and d.last_advance_issue == AdvanceIssue.STEP_FAILED
    assert d.last_rejection_reason == reason and d.failure_reason is None and d.pending_transaction_count == 1
    assert d.backlog_seconds == 0.125
    retried = w.advance(0)
    assert retried.step_index == 1 and len(retried.transaction_receipts) == 1 and w.diagnostics.last_advance_issue is None
    assert w.diagnostics.backlog_seconds == 0 and w.diagnostics.last_rejection_reason is None


def test_a_failed_command_ends_the_world_and_drops_the_queue():
    SCRIPT.extend([("ok", 0, 0), ("raise", N.E_CUDA)])
    w = world()
    first = w.advance(0.125)
    assert first.step_index == 1
    w.submit(WorldTransaction().set_global_force((1.0, 0.0)))
    failed = w.advance(0.125)
    d = w.diagnostics
    assert failed is first and d.failure_reason == WorldFailureReason.COMMAND_EXECUTION_FAILED
    assert d.last_advance_issue == AdvanceIssue.WORLD_FAILED and d.pending_transaction_count == 0
    calls = len(CALLS)
    w.submit(WorldTransaction().set_global_force((2.0, 0.0)))
    assert w.advance(1.0) is first and len(CALLS) == calls and w.diagnostics.pending_transaction_count == 0
    assert w.diagnostics.last_advance_issue == AdvanceIssue.WORLD_FAILED


def test_non_finite_values_end_the_world():
    SCRIPT.append(("status", N.E_NONFINITE))
    w = world()
    frame = w.advance(0.125)
    assert frame.step_index == 0 and w.diagnostics.failure_reason == WorldFailureReason.NON_FINITE_VALUES
    assert w.diagnostics.pending_transaction_count == 0


def test_a_failure_after_a_completed_step_returns_its_frame_and_keeps_the_unsimulated_time():
    SCRIPT.extend([("ok", 0, 0), ("raise", N.E_INFLIGHT)])
    w = world()
    partial = w.advance(0.375)
    assert partial.step_index == 1 and partial.simulation_time == 0.125 and len(partial.transaction_receipts) == 1
    assert w.diagnostics.backlog_seconds == 0.25 and w.diagnostics.last_advance_issue == AdvanceIssue.STEP_FAILED
    retried = w.advance(0)
    assert retried.step_index == 3 and retried.simulation_time == 0.375 and retried.transaction_receipts == ()
