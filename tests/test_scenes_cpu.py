"""The synthetic workload generators: seeded and deterministic, ids sorted and unique, no bubble starting inside a
rigid body or static polygon, bounded samples that are prefixes of the full workload, and a serving pool whose worlds
do not depend on how it was generated (serially or in a process pool)."""
import numpy as np

from bubblephysics_gb300 import scenes


def same_world(a, b):
    return all(np.array_equal(getattr(a, f), getattr(b, f)) for f in
               ("bubbles", "segments", "bodies", "body_vertices", "body_triangles"))


def test_batched_worlds_sample_is_a_prefix():
    full = scenes.batched_worlds(12, seed=9)
    part = scenes.batched_worlds(12, seed=9, limit=4)
    assert len(part) == 4 and all(same_world(a, b) for a, b in zip(part, full[:4]))


def test_serving_pool_is_the_same_serial_or_per_world():
    pool = scenes.serving_worlds(6, seed=5)
    for w, spec in enumerate(pool):
        assert same_world(spec, scenes.serving_world((5, w, 16, 4096)))
        assert 0 < spec.bubble_count <= 4096


def test_rigid_world_places_bubbles_clear_of_every_obstacle():
    spec = scenes.rigid_world(seed=13, n=800, bodies=200, side=1100.0)
    b = spec.bubbles
    assert b.shape[0] == 800
    assert np.all(np.diff(b["id"]) > 0) and np.all(np.diff(spec.segments["id"]) > 0)
    assert len(set(spec.bodies["id"])) == len(spec.bodies)
    centers = b["center"].astype(np.float64)
    radii = b["radius"].astype(np.float64)
    # every bubble is more than r + 1 from every obstacle body (bounding circle)
    for body in spec.bodies:
        d = np.hypot(centers[:, 0] - body["position"][0], centers[:, 1] - body["position"][1])
        assert np.all(d > body["bounding_radius"] + radii + 1.0 - 1e-3)
    # and inside the walls
    assert np.all(centers.min(axis=1) > radii) and np.all(centers.max(axis=1) < 1100.0 - radii)
