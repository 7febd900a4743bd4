"""The serving loop on the GPU: a world's result does not depend on what it is served with - alone, in a mix of
other worlds' requests, across evictions to host memory and back, batched or one launch per step - and it is the
result of stepping the same world by itself (bp_world_step)."""
import numpy as np
import pytest

import fixtures
from bubblephysics_gb300 import _native as N
from bubblephysics_gb300 import scenes
from bubblephysics_gb300.solver import Server, World

pytestmark = pytest.mark.gpu


def specs(count=24, seed=41):
    return scenes.batched_worlds(count, seed=seed)


def assert_same_bubbles(a, b):
    for f in ("center", "previous_center", "velocity", "rotation", "angular_velocity", "region_result", "flags"):
        assert np.array_equal(a[f], b[f]), f


def stepped_alone(ctx, spec, steps):
    w = World(spec, ctx)
    status, _ = w.step(steps)
    out = w.bubbles()
    w.close()
    return status, out


def serve(ctx, worlds, requests, **kw):
    """requests: list of (world, steps) submitted in order while the loop runs."""
    server = Server(len(worlds), ctx, **kw)
    for spec in worlds:
        server.add_world(spec)
    done = []
    for i, (w, steps) in enumerate(requests):
        server.submit(w, steps)
        if i % 3 == 0:
            server.progress()
            done.append(server.poll())
    done.append(server.drain())
    return server, np.concatenate(done)


def test_a_world_alone_and_in_the_mix_gives_the_same_result(ctx):
    worlds = specs()
    target = 5
    rng = np.random.default_rng(0)
    mix = [(int(w), int(rng.integers(1, 3))) for w in rng.integers(0, len(worlds), 120)]
    mix += [(target, 1)] * 4
    steps_of_target = sum(s for w, s in mix if w == target)
    alone, done_alone = serve(ctx, [worlds[target]], [(0, steps_of_target)])
    mixed, done_mixed = serve(ctx, worlds, mix)
    assert done_alone["status"].tolist() == [N.OK]
    assert (done_mixed["status"] == N.OK).all() and len(done_mixed) == len(mix)
    status, reference = stepped_alone(ctx, worlds[target], steps_of_target)
    assert status == N.OK
    assert_same_bubbles(alone.bubbles(0), reference)
    assert_same_bubbles(mixed.bubbles(target), reference)
    stats = mixed.stats()
    assert stats["batches"] < stats["batched_worlds"]  # requests really were batched together


def test_eviction_to_host_and_back_is_exact(ctx):
    worlds = specs(16, seed=42)
    probe = Server(1, ctx)
    probe.add_world(worlds[0])
    probe.submit(0, 1)
    probe.drain()
    one = probe.stats()["resident_bytes"]
    probe.close()
    rng = np.random.default_rng(1)
    requests = [(int(w), 1) for w in rng.integers(0, len(worlds), 160)]
    # room for about three worlds: almost every switch evicts someone
    server, done = serve(ctx, worlds, requests, hbm_budget_bytes=3 * max(one, 1) + (1 << 20))
    assert (done["status"] == N.OK).all()
    stats = server.stats()
    assert stats["evictions"] > 10 and stats["resident_bytes"] <= stats["hbm_budget_bytes"]
    counts = np.bincount([w for w, _ in requests], minlength=len(worlds))
    for w, spec in enumerate(worlds):
        status, reference = stepped_alone(ctx, spec, int(counts[w])) if counts[w] else (N.OK, None)
        got = server.bubbles(w)
        if reference is None:
            assert_same_bubbles(got, spec.bubbles)
        else:
            assert_same_bubbles(got, reference)


def test_plain_per_world_serving_matches_batched(ctx):
    worlds = specs(12, seed=43)
    rng = np.random.default_rng(2)
    requests = [(int(w), int(rng.integers(1, 3))) for w in rng.integers(0, len(worlds), 40)]
    batched, _ = serve(ctx, worlds, requests, streams=3)
    plain, _ = serve(ctx, worlds, requests, per_world=True)
    for w in range(len(worlds)):
        assert_same_bubbles(batched.bubbles(w), plain.bubbles(w))


def test_rigid_tree_worlds_are_served(ctx):
    worlds = [scenes.rigid_world(seed=s, n=600, bodies=150, side=800.0) for s in (51, 52)] + specs(4, seed=44)
    server, done = serve(ctx, worlds, [(0, 2), (1, 1), (2, 1), (0, 1), (3, 2), (1, 1)])
    assert (done["status"] == N.OK).all()
    for w, steps in ((0, 3), (1, 2)):
        _, reference = stepped_alone(ctx, worlds[w], steps)
        assert_same_bubbles(server.bubbles(w), reference)


def test_a_failing_world_fails_alone(ctx):
    bad = fixtures.bounce_scene(3000.0, 20.0)
    bad.substep_split_multiplier = 2000.0  # hits the substep limit on its first step
    worlds = [bad] + specs(3, seed=45)
    server, done = serve(ctx, worlds, [(0, 1), (1, 1), (0, 1), (2, 2)])
    by_world = {}
    for c in done:
        by_world.setdefault(int(c["world"]), []).append(int(c["status"]))
    assert by_world[0] == [N.E_SUBSTEP_LIMIT, N.E_WORLD_FAILED]
    assert by_world[1] == [N.OK] and by_world[2] == [N.OK]


def test_server_refuses_worlds_above_the_block_limit(ctx):
    server = Server(2, ctx)
    with pytest.raises(N.NativeError) as err:
        server.add_world(scenes.large_world(n=5000, side=2048.0))
    assert err.value.status == N.E_CAPACITY
