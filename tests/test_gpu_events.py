"""Contact began / ended events compacted on the device (bp_world_contact_events) against the oracle's restatement of
the reference's contact transitions (NativePublicWorld.swift:347-391), bit for bit, step after step with the history
carried on the device: the reference's own scenes, a sample of the batched workload's worlds (bodies and polygon edges
included), caller records and removals."""
import numpy as np
import pytest

import fixtures
from bubblephysics_gb300 import _native as N
from bubblephysics_gb300 import scenes
from bubblephysics_gb300.solver import World
from oracle import oracle
from oracle.oracle import OracleWorld

pytestmark = pytest.mark.gpu


def all_objects(spec):
    ids = set(int(i) for i in spec.bubbles["id"])
    owners = spec.segments["owner_id"][(spec.segments["flags"] & N.SEGMENT_HAS_OWNER) != 0]
    return ids | set(int(o) for o in owners) | set(int(b) for b in spec.bodies["id"])


def run_steps(ctx, spec, steps, interested, extra_for=None, removed_for=None):
    gpu, cpu = World(spec, ctx), OracleWorld(spec, 32)
    history = np.zeros((0, 2), np.int64)
    total = 0
    for step in range(steps):
        sg, _ = gpu.step(1)
        sc, _ = cpu.step(1)
        assert sg == sc == N.OK
        contacts = cpu.contacts()
        assert np.array_equal(gpu.contacts(), contacts)
        extra = extra_for(step) if extra_for else None
        removed = removed_for(step) if removed_for else ()
        records = contacts if extra is None else np.concatenate([contacts, extra])
        want, history = oracle.contact_events(records, spec.segments, interested, history, removed, spec.time_step)
        got = gpu.contact_events(interested, removed, extra=extra)
        assert np.array_equal(got, want), (step, got[:4], want[:4])
        assert np.array_equal(gpu.contact_history(), history), step
        total += got.size
    return total


@pytest.mark.parametrize("name", ["pair_bounce", "segments", "bounce_1000", "press", "dense"])
def test_reference_scene_events_bit_exact(ctx, name):
    spec = {"pair_bounce": fixtures.pair_bounce_scene, "segments": fixtures.segment_scene,
            "bounce_1000": lambda: fixtures.bounce_scene(1000.0), "press": fixtures.press_scene,
            "dense": lambda: fixtures.dense_scene(128)}[name]()
    run_steps(ctx, spec, 20, all_objects(spec))


def test_batched_world_sample_events_bit_exact(ctx):
    rng = np.random.default_rng(31)
    events = 0
    for i, n in enumerate([24, 90, 250, 700]):
        spec = scenes.batched_world(rng, n, world_index=i, max_bodies=32)
        objects = sorted(all_objects(spec))
        interested = set(objects[::2])  # half of the objects ask for contact events
        events += run_steps(ctx, spec, 12, interested)
    assert events > 0


def test_caller_records_and_removals_bit_exact(ctx):
    spec = scenes.plain_world(seed=3, n=120)
    ids = [int(i) for i in spec.bubbles["id"]]
    rng = np.random.default_rng(5)

    def extra_for(step):  # bubble-body style records from the caller, some repeating a pair
        e = np.zeros(6, N.CONTACT_DTYPE)
        e["participants"] = [(ids[(step + 3 * q) % 20], 5_000 + q % 3) for q in range(6)]
        e["kind"] = 2
        e["point"] = rng.normal(size=(6, 2))
        e["normal"] = rng.normal(size=(6, 2))
        e["penetration"] = rng.uniform(-0.05, 0.5, 6)
        e["impulse"] = rng.uniform(0, 0.1, 6)
        return e

    def removed_for(step):
        return ids[step * 3: step * 3 + 2] + ([5_001] if step == 4 else [])

    run_steps(ctx, spec, 8, set(ids[:60]) | {5_000, 5_002}, extra_for, removed_for)


def test_history_can_be_set_and_capacity_truncates(ctx):
    spec = fixtures.pair_bounce_scene()
    gpu = World(spec, ctx)
    gpu.set_contact_history([[7, 3], [3, 7], [1, 2]])
    assert gpu.contact_history().tolist() == [[1, 2], [3, 7]]
    gpu.step(1)
    full = gpu.contact_events({1, 2, 3, 7})
    gpu.set_contact_history([[1, 2], [3, 7]])
    part = gpu.contact_events({1, 2, 3, 7}, capacity=1)
    assert part.size == 1 and np.array_equal(part[0], full[0])
