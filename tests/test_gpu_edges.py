"""Edge sizes on the GPU against the oracle, bit for bit:
- a batch of ragged worlds, including an empty world (walls only) and one-bubble worlds;
- worlds exactly at the team thresholds: 64 / 65 bubbles (group or block team at the default threshold), 512 / 513
  (one or two bubbles per thread of a 512-thread block), 4,096 / 4,097 (the largest block-team world and the smallest
  whole-GPU one).

Worlds without bodies keep every generated bubble, so the sizes are exact."""
import dataclasses

import numpy as np
import pytest

from bubblephysics_gb300 import _native as N
from bubblephysics_gb300 import scenes
from bubblephysics_gb300.solver import Batch, World
from oracle.oracle import OracleWorld
from test_gpu_config_sizes import same_bubbles, same_reports

pytestmark = pytest.mark.gpu


def world_of(n: int, seed: int) -> scenes.WorldSpec:
    rng = np.random.default_rng(1000 + seed)
    if n == 0:  # the walls of a small world without its bubbles
        spec = scenes.batched_world(rng, 8, world_index=seed, max_bodies=0)
        return dataclasses.replace(spec, bubbles=spec.bubbles[:0])
    spec = scenes.batched_world(rng, n, world_index=seed, max_bodies=0)
    assert spec.bubble_count == n
    return spec


RAGGED = [0, 1, 2, 31, 32, 33, 63, 64, 65, 127, 128, 129, 511, 512, 513, 1024]


@pytest.mark.parametrize("schedule", [dict(autotune=True), dict(threads_per_world=512, warp_world_max=64, group_width=64),
                                      dict(threads_per_world=256, warp_world_max=32, group_width=32)])
def test_ragged_batch_with_empty_and_tiny_worlds(ctx, schedule):
    specs = [world_of(n, i) for i, n in enumerate(RAGGED)]
    batch = Batch(specs, ctx, use_graph=True, **schedule)
    worlds = [OracleWorld(spec, 32) for spec in specs]
    for step in range(3):
        status, reps = batch.step(1)
        assert status == N.OK, step
        for w, cpu in enumerate(worlds):
            sc, rc = cpu.step(1)
            assert sc == N.OK, (w, step)
            same_reports(reps[w:w + 1], rc, f"world {w} ({RAGGED[w]} bubbles) step {step}")
            same_bubbles(batch.bubbles(w), cpu.bubbles(), f"world {w} ({RAGGED[w]} bubbles) step {step}")
    # the empty world: no live bubble, so no substep and no contact, as in the oracle
    assert reps[0]["substep_count"] == 0 and reps[0]["contact_count"] == 0


@pytest.mark.parametrize("n", [4096, 4097])
def test_single_world_at_the_whole_gpu_threshold(ctx, n):
    spec = world_of(n, 7)
    gpu, cpu = World(spec, ctx), OracleWorld(spec, 32)
    for step in range(2):
        sg, rg = gpu.step(1)
        sc, rc = cpu.step(1)
        assert sg == sc == N.OK, step
        same_reports(rg, rc, f"step {step}")
        assert np.array_equal(gpu.cells(), cpu.cells()), step
        assert np.array_equal(gpu.candidates(), cpu.candidates()), step
        assert np.array_equal(gpu.contacts(), cpu.contacts()), step
        same_bubbles(gpu.bubbles(), cpu.bubbles(), f"step {step}")
