"""The LBVH rigid broadphase on the GPU: Morton keys bit-exact with the oracle's restatement of the key rule, candidate
sets, contacts and states bit-exact with the oracle's brute-force loops (NativeGeometryKernels:279-290, 350-415), and
the tree path identical to the brute-force path of the same library on every team kind (warp, block, whole GPU)."""
import dataclasses

import numpy as np
import pytest

import fixtures
from bubblephysics_gb300 import _native as N
from bubblephysics_gb300 import scenes
from bubblephysics_gb300.solver import World
from oracle.oracle import OracleWorld
from test_gpu_golden import same

pytestmark = pytest.mark.gpu


def small_rigid_world(**kw):
    args = dict(seed=5, n=1500, bodies=400, side=1300.0)
    args.update(kw)
    return scenes.rigid_world(**args)


def with_flags(spec, flags, **kw):
    return dataclasses.replace(spec, flags=spec.flags | flags, **kw)


def test_rigid_world_keys_and_state_match_oracle(ctx):
    spec = small_rigid_world()
    leaves = len(spec.segments) + len(spec.bodies)
    assert leaves >= 128  # the automatic threshold picks the tree
    gpu, cpu = World(spec, ctx), OracleWorld(spec, 32)
    for _ in range(4):
        rep = same(gpu, cpu, 1)
        assert rep[0]["status"] == N.OK
        keys = gpu.rigid_keys()
        assert keys.size == leaves
        assert np.array_equal(keys, cpu.rigid_keys())
        assert np.array_equal(np.sort(keys & np.uint64(0xFFFFFFFF)), np.arange(leaves, dtype=np.uint64))
    assert rep[0]["body_candidate_count"] > 0


@pytest.mark.parametrize("path", [0, N.WORLD_FORCE_MULTI_CTA])
def test_tree_and_brute_force_paths_agree(ctx, path):
    base = small_rigid_world(seed=6)
    tree = World(with_flags(base, N.WORLD_RIGID_TREE | path), ctx)
    brute = World(with_flags(base, N.WORLD_NO_RIGID_TREE | path), ctx)
    for _ in range(3):
        st, rt = tree.step(2)
        sb, rb = brute.step(2)
        assert st == sb == N.OK
        for key in ("substep_count", "rebuild_count", "candidate_count", "body_candidate_count", "candidate_overflow",
                    "max_candidates_per_object", "contact_count", "limiter_object"):
            assert rt[key].tolist() == rb[key].tolist(), key
        bt, bb = tree.bubbles(), brute.bubbles()
        assert np.array_equal(bt["center"], bb["center"]) and np.array_equal(bt["velocity"], bb["velocity"])
        assert np.array_equal(tree.candidates(), brute.candidates())
        assert np.array_equal(tree.contacts(), brute.contacts())
    assert tree.rigid_keys().size == len(base.segments) + len(base.bodies)
    assert brute.rigid_keys().size == 0


def test_forced_tree_on_small_worlds_matches_oracle(ctx):
    """Worlds far below the automatic threshold (warp and block teams, a handful of leaves) with the tree forced."""
    rng = np.random.default_rng(31)
    done = 0
    for i, n in enumerate([24, 48, 150, 600] * 3):
        spec = scenes.batched_world(rng, n, world_index=i, max_bodies=32)
        if len(spec.bodies) == 0:
            continue
        spec = with_flags(spec, N.WORLD_RIGID_TREE)
        gpu, cpu = World(spec, ctx), OracleWorld(spec, 32)
        same(gpu, cpu, 6)
        assert np.array_equal(gpu.rigid_keys(), cpu.rigid_keys())
        done += 1
    assert done >= 4


def test_single_leaf_tree(ctx):
    spec = fixtures.segment_scene()
    spec = dataclasses.replace(spec, segments=spec.segments[:1], flags=spec.flags | N.WORLD_RIGID_TREE)
    gpu, cpu = World(spec, ctx), OracleWorld(spec, 32)
    same(gpu, cpu, 3)
    assert gpu.rigid_keys().tolist() == cpu.rigid_keys().tolist() == [0]


def test_body_row_overflow_through_tree(ctx):
    """Candidate limit 4: body rows overflow, so the tree pass hands them to the brute-force scan (first k bubbles
    in index order) and the adjacency filters by row membership."""
    spec = with_flags(small_rigid_world(seed=7), N.WORLD_RIGID_TREE, candidate_limit=4)
    gpu, cpu = World(spec, ctx), OracleWorld(spec, 32)
    rep = same(gpu, cpu, 2)
    assert rep[-1]["candidate_overflow"] > 0


def _violation(spec, ctx, bubble_id, where):
    spec = with_flags(spec, N.WORLD_INJECT_STATE, inject_object=int(bubble_id))
    gpu, cpu = World(spec, ctx), OracleWorld(spec, 32)
    gpu.set_injection(0, where)
    cpu.set_injection(0, where)
    return same(gpu, cpu, 1)[0]


@pytest.mark.parametrize("tree", [N.WORLD_RIGID_TREE, N.WORLD_NO_RIGID_TREE])
def test_assertion_inside_body_through_tree(ctx, tree):
    base = with_flags(small_rigid_world(seed=8), tree)
    circles = np.flatnonzero(base.bodies["kind"] == N.BODY_CIRCLE)
    body = base.bodies[circles[0]]
    rep = _violation(base, ctx, base.bubbles["id"][0], tuple(map(float, body["position"])))
    assert rep["status"] == N.E_CONTACT_VIOLATION and rep["violation_kind"] == N.VIOLATION_INSIDE_BODY
    assert rep["violation_objects"][1] == body["id"]


@pytest.mark.parametrize("tree", [N.WORLD_RIGID_TREE, N.WORLD_NO_RIGID_TREE])
def test_assertion_edge_crossing_through_tree(ctx, tree):
    base = with_flags(small_rigid_world(seed=9), tree)
    owners = base.segments["owner_id"]
    polygon = owners[owners >= 3_000_000][0]  # a static polygon's edges (the walls belong to owners 2,000,000 + k)
    edges = base.segments[owners == polygon]
    centroid = np.concatenate([edges["a"], edges["b"]]).mean(axis=0)
    rep = _violation(base, ctx, base.bubbles["id"][0], tuple(map(float, centroid)))
    assert rep["status"] == N.E_CONTACT_VIOLATION and rep["violation_kind"] == N.VIOLATION_EDGE_SIDE
