"""The reference's own test scenes on the GPU, through the C ABI, compared bit for bit with the oracle (which
tests/test_oracle_golden.py pins to the reference's known answers), plus the failure paths and the schedule
invariance of the batched path."""
import numpy as np
import pytest

import fixtures
from bubblephysics_gb300 import _native as N
from bubblephysics_gb300 import scenes
from bubblephysics_gb300.solver import Batch, World
from oracle.oracle import OracleWorld

pytestmark = pytest.mark.gpu

SCENES = {
    "broadphase_0.2": lambda: fixtures.broadphase_scene(0.2),
    "broadphase_1.9": lambda: fixtures.broadphase_scene(1.9),
    "broadphase_7": lambda: fixtures.broadphase_scene(7.0),
    "dense_truncation": lambda: fixtures.dense_scene(128),
    "segments": fixtures.segment_scene,
    "bounce_1000": lambda: fixtures.bounce_scene(1000.0),
    "bounce_3000": lambda: fixtures.bounce_scene(3000.0),
    "pair_bounce": fixtures.pair_bounce_scene,
    "press": fixtures.press_scene,
    "damped_force_5": lambda: fixtures.constant_force_scene(5.0),
}


def same(gpu, cpu, steps):
    sg, rg = gpu.step(steps)
    sc, rc = cpu.step(steps)
    assert sg == sc
    for key in ("status", "substep_count", "rebuild_count", "candidate_count", "body_candidate_count",
                "candidate_overflow", "max_candidates_per_object", "contact_count", "limiter_term", "limiter_object",
                "violation_kind", "violation_edge", "removed_count", "wrapped_count"):
        assert rg[key].tolist() == rc[key].tolist(), key
    assert np.array_equal(rg["violation_objects"], rc["violation_objects"])
    assert np.array_equal(rg["violation_distance"], rc["violation_distance"])
    bg, bc = gpu.bubbles(), cpu.bubbles()
    for f in ("center", "previous_center", "velocity", "rotation", "angular_velocity", "region_result"):
        assert np.array_equal(bg[f], bc[f]), (f, np.abs(bg[f].astype(np.float64) - bc[f]).max())
    assert np.array_equal(gpu.candidates(), cpu.candidates())
    assert np.array_equal(gpu.contacts(), cpu.contacts())
    return rg


@pytest.mark.parametrize("name", sorted(SCENES))
def test_reference_scene_bit_exact(ctx, name):
    spec = SCENES[name]()
    same(World(spec, ctx), OracleWorld(spec, 32), 30 if "bounce" in name or name == "press" else 3)


def test_injected_pair_violation_on_gpu(ctx):
    from test_oracle_golden import injected_pair_scene
    spec = injected_pair_scene()
    gpu, cpu = World(spec, ctx), OracleWorld(spec, 32)
    gpu.set_injection(0, (60.0, 0.0))
    cpu.set_injection(0, (60.0, 0.0))
    rep = same(gpu, cpu, 1)
    assert rep[0]["status"] == N.E_CONTACT_VIOLATION and rep[0]["violation_kind"] == N.VIOLATION_PAIR
    status, rep2 = gpu.step(1)
    assert status == N.E_WORLD_FAILED


def test_injected_edge_crossing_on_gpu(ctx):
    spec = fixtures.bounce_scene(10.0, 30.0)
    spec.flags |= N.WORLD_INJECT_STATE
    spec.inject_object = 1
    gpu, cpu = World(spec, ctx), OracleWorld(spec, 32)
    gpu.set_injection(0, (100.0, 5.0))
    cpu.set_injection(0, (100.0, 5.0))
    rep = same(gpu, cpu, 1)
    assert rep[0]["violation_kind"] == N.VIOLATION_EDGE_SIDE


def test_natural_edge_crossing_on_gpu(ctx):
    """Bubbles without contact stiffness run through the floor's bottom edge within one step, without injection.
    The end-of-step assertion reports the crossing exactly as the oracle does: kind, objects, edge and distance."""
    b = scenes.make_bubbles([(100.0, -10.0), (300.0, -40.0)], 12.0, velocities=[(0.0, 1200.0), (0.0, 1200.0)],
                            masses=0.36, stiffness=0.0)
    spec = scenes.WorldSpec(bubbles=b, segments=fixtures.floor_wall())
    rep = same(World(spec, ctx), OracleWorld(spec, 32), 2)
    assert rep[0]["status"] == N.E_CONTACT_VIOLATION and rep[0]["violation_kind"] == N.VIOLATION_EDGE_SIDE
    assert rep[0]["violation_edge"] == 1000 and rep[0]["rebuild_count"] == 0


def test_substep_limit_on_gpu(ctx):
    spec = fixtures.bounce_scene(3000.0, 20.0)
    spec.substep_split_multiplier = 2000.0
    rep = same(World(spec, ctx), OracleWorld(spec, 32), 1)
    assert rep[0]["status"] == N.E_SUBSTEP_LIMIT and rep[0]["substep_count"] == 1024


def test_worlds_with_bodies_bit_exact(ctx):
    rng = np.random.default_rng(11)
    done = 0
    for i, n in enumerate([30, 150, 600] * 4):
        spec = scenes.batched_world(rng, n, world_index=i, max_bodies=32)
        if len(spec.bodies) == 0:
            continue
        same(World(spec, ctx), OracleWorld(spec, 32), 10)
        done += 1
    assert done >= 3


@pytest.mark.parametrize("threads,warp_max", [(128, 0), (256, 64), (512, 128), (128, 32)])
def test_batched_schedule_does_not_change_results(ctx, threads, warp_max):
    specs = scenes.batched_worlds(64, seed=21)
    ref = Batch(specs, ctx, use_graph=False, per_world_launch=True)
    ref.step(4)
    b = Batch(specs, ctx, use_graph=True, threads_per_world=threads, warp_world_max=warp_max or 0xFFFFFFFF)
    assert b.tuning()["threads"] == threads and b.tuning()["warp_max"] == warp_max
    st, reps = b.step(4)
    for w in range(len(specs)):
        x, y = b.bubbles(w), ref.bubbles(w)
        assert np.array_equal(x["center"], y["center"]) and np.array_equal(x["velocity"], y["velocity"])


def test_autotuned_batch_matches_the_per_world_path(ctx):
    specs = scenes.batched_worlds(200, seed=22)
    plain = Batch(specs, ctx, per_world_launch=True, use_graph=False)
    fused = Batch(specs, ctx, use_graph=True, autotune=True)
    sp, rp = plain.step(6)
    sf, rf = fused.step(6)
    assert rp["substep_count"].tolist() == rf["substep_count"].tolist()
    assert rp["status"].tolist() == rf["status"].tolist()
    for w in range(len(specs)):
        assert np.array_equal(plain.bubbles(w)["center"], fused.bubbles(w)["center"])


def test_host_state_round_trip(ctx):
    specs = scenes.batched_worlds(16, seed=23)
    b = Batch(specs, ctx, use_graph=False)
    b.step(1)
    state = b.read_state()
    state[:, 2:] *= 0.5
    b.write_state(np.ascontiguousarray(state))
    assert np.array_equal(b.read_state(), state)
    first = b.bubbles(0)
    assert np.array_equal(first["velocity"], state[: len(first), 2:])


def test_host_state_through_page_locked_buffers(ctx):
    """Page-locked, 16-byte aligned host buffers are read and written by the state kernels directly (no staging
    copy): the same state as through pageable buffers, and steps from it equal steps from the staged write."""
    torch = pytest.importorskip("torch")
    specs = scenes.batched_worlds(64, seed=29)
    a, b = Batch(specs, ctx, use_graph=False), Batch(specs, ctx, use_graph=False)
    a.step(2)
    b.step(2)
    state = a.read_state()
    pinned_t = torch.empty(state.shape, dtype=torch.float32, pin_memory=True)
    pinned = pinned_t.numpy()
    b.read_state(pinned)
    assert np.array_equal(pinned, state)
    state[:, 2:] *= 0.5
    pinned[:] = state
    a.write_state(np.ascontiguousarray(state))  # pageable: staged
    b.write_state(pinned)                       # page-locked: direct
    ra, rb = a.step(3)[1], b.step(3)[1]
    assert ra["substep_count"].tolist() == rb["substep_count"].tolist()
    assert np.array_equal(a.read_state(), b.read_state(pinned))
    assert np.array_equal(pinned, a.read_state())


def test_context_outlives_its_worlds_whatever_the_destroy_order():
    from bubblephysics_gb300.solver import Context
    c = Context(0)
    w = World(fixtures.pair_bounce_scene(), c)
    b = Batch(scenes.batched_worlds(4, seed=24), c, use_graph=False)
    c.close()              # released first: must stay alive for w and b
    assert w.step(1)[0] == N.OK
    assert b.step(1)[0] == N.OK
    w.close()
    b.close()              # the last user frees the context
