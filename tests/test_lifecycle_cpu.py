"""Pause in the background and the dropped first increment after it (LifecycleTests.swift:39-160): automatic pause on
by default; in the background advance publishes nothing and no time accumulates; after the return the first
increment is dropped; a return without a background drops nothing; automatic_pause=False ignores the lifecycle; a
manual pause and the background pause do not lift each other; the lifecycle source does not keep the world alive. A
world without bubbles steps without a device, so these run on the CPU."""
import gc
import weakref

from bubblephysics_gb300.world import BubbleWorld, WorldConfiguration


class FakeLifecycle:
    will_enter_background = None
    did_become_active = None

    def enter_background(self):
        if self.will_enter_background:
            self.will_enter_background()

    def become_active(self):
        if self.did_become_active:
            self.did_become_active()


def make_world(source, automatic_pause=True):
    cfg = WorldConfiguration((-10.0, -10.0, 10.0, 10.0), fixed_time_step=0.125, maximum_backlog=10.0,
                             automatic_pause=automatic_pause)
    return BubbleWorld(cfg, lifecycle=source)


def test_automatic_pause_is_on_by_default():
    assert WorldConfiguration((-1.0, -1.0, 1.0, 1.0)).automatic_pause


def test_background_pauses_the_world_and_no_time_accumulates():
    source = FakeLifecycle()
    world = make_world(source)
    before = world.advance(0.125)
    source.enter_background()
    assert world.diagnostics.is_paused
    assert world.advance(1.0) is before and world.diagnostics.backlog_seconds == 0


def test_first_advance_after_the_return_drops_its_time():
    source = FakeLifecycle()
    world = make_world(source)
    before = world.advance(0.125)
    source.enter_background()
    world.advance(5.0)
    source.become_active()
    assert not world.diagnostics.is_paused
    first = world.advance(0.5)
    assert first is before and world.diagnostics.backlog_seconds == 0 and world.diagnostics.steps_in_last_advance == 0
    assert world.advance(0.125).step_index == before.step_index + 1


def test_return_without_a_background_drops_nothing():
    source = FakeLifecycle()
    world = make_world(source)
    source.become_active()
    assert world.advance(0.125).step_index == 1


def test_disabled_automatic_pause_ignores_the_lifecycle():
    source = FakeLifecycle()
    world = make_world(source, automatic_pause=False)
    source.enter_background()
    assert not world.diagnostics.is_paused and world.advance(0.125).step_index == 1
    source.become_active()
    assert world.advance(0.125).step_index == 2


def test_manual_pause_survives_the_return():
    source = FakeLifecycle()
    world = make_world(source)
    world.pause()
    source.enter_background()
    source.become_active()
    assert world.diagnostics.is_paused and world.advance(1.0).step_index == 0
    world.resume()
    assert not world.diagnostics.is_paused
    assert world.advance(0.5).step_index == 0  # the first increment after the background is still dropped
    assert world.advance(0.125).step_index == 1


def test_manual_resume_in_the_background_does_not_lift_the_automatic_pause():
    source = FakeLifecycle()
    world = make_world(source)
    world.pause()
    source.enter_background()
    world.resume()
    assert world.diagnostics.is_paused and world.advance(1.0).step_index == 0
    source.become_active()
    assert not world.diagnostics.is_paused


def test_background_during_a_manual_pause_is_not_lifted_by_the_return():
    source = FakeLifecycle()
    world = make_world(source)
    source.enter_background()
    world.pause()
    source.become_active()
    assert world.diagnostics.is_paused


def test_the_source_does_not_keep_the_world_alive():
    source = FakeLifecycle()
    world = make_world(source)
    ref = weakref.ref(world)
    del world
    gc.collect()
    assert ref() is None
    source.enter_background()
    source.become_active()
