"""Hit test on the GPU (bp_world_hit_test) against the oracle's restatement of nativeHitTest
(NativeGeometryKernels:501-541): identical answers for every query, contour edges included (the contours themselves
are bit-exact)."""
import numpy as np
import pytest

from bubblephysics_gb300 import scenes
from bubblephysics_gb300.solver import World
from oracle.oracle import OracleWorld
from test_hit_test_cpu import scene

pytestmark = pytest.mark.gpu


def check(spec, ctx, steps, queries):
    gpu, cpu = World(spec, ctx), OracleWorld(spec, 32)
    assert gpu.step(steps)[0] == cpu.step(steps)[0] == 0
    queries = np.asarray(queries, np.float64)
    g = gpu.hit_test(queries)
    c = cpu.hit_test(queries)
    for x, y in zip(g, c):
        assert np.array_equal(x, y)
    return g


def test_constructed_scene(ctx):
    g = check(scene(), ctx, 1, [(-5.0, 0.0), (100.0, 3.0), (200.0, 0.0), (50.0, 50.0), (10.0, 0.0)])
    assert g[0].tolist() == [5, 6, 900, 0, 50]


def test_plain_world_random_queries(ctx):
    spec = scenes.plain_world(seed=1)
    rng = np.random.default_rng(3)
    centres = spec.bubbles["center"].astype(np.float64)
    queries = np.concatenate([centres, rng.uniform((-50, -50), (425, 750), (2000, 2))])
    g = check(spec, ctx, 10, queries)
    assert g[2].sum() > 300


def test_batched_world_with_bodies_and_polygons(ctx):
    rng = np.random.default_rng(8)
    spec = scenes.batched_world(rng, 400, world_index=2)
    spec.bubbles["layer"] = rng.integers(0, 3, spec.bubble_count)
    lo, hi = spec.region[:2], spec.region[2:]
    queries = np.concatenate([rng.uniform(lo, hi, (3000, 2)), spec.bodies["position"].astype(np.float64)])
    g = check(spec, ctx, 4, queries)
    assert len(spec.bodies) > 0 and set(spec.bodies["id"].tolist()) & set(g[0].tolist())  # body centres hit bodies


@pytest.mark.parametrize("name", sorted(__import__("test_hit_test_cpu").HIT_CASES))
def test_reference_hit_test_cases_on_the_gpu(ctx, name):
    from test_hit_test_cpu import HIT_CASES, answers
    build, points, expected = HIT_CASES[name]
    spec = build()
    assert answers(spec, points, World(spec, ctx)) == expected
