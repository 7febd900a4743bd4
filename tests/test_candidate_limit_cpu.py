"""The candidate limit reaches the solver in its range, against SubstepSeamTests.swift:90-117, through the world API on a stand-in
device world that forwards to the oracle: the middle bubble of a 3 x 3 grid (radius 24, mass 1, spacing 50, K_c 229,
ForceScene's bubble) has 4 candidates within its bound margin; the default k = 128 keeps them all, k = 2 drops some
and counts the overflow."""
import pytest

from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import BubbleDescriptor, BubbleWorld, PhysicsMaterial, WorldConfiguration, WorldTransaction
from test_world_api_oracle_cpu import OracleBackedWorld


@pytest.fixture(autouse=True)
def oracle_backed(monkeypatch):
    monkeypatch.setattr(W, "World", OracleBackedWorld)
    monkeypatch.setattr(W, "default_context", lambda: None)


def overflow(limit=None):
    extra = {} if limit is None else {"candidate_limit": limit}
    world = BubbleWorld(WorldConfiguration((-2000.0, -2000.0, 2000.0, 2000.0), contours=False, **extra))
    tx = WorldTransaction().update_physics_material(1, PhysicsMaterial(229.0))
    for row in range(3):
        for column in range(3):
            tx = tx.add(BubbleDescriptor(1 + 3 * row + column, ((column - 1) * 50.0, (row - 1) * 50.0), 24.0, 1.0, 1))
    world.submit(tx)
    for _ in range(3):
        world.advance(1.0 / 60)
        assert world.diagnostics.last_advance_issue is None
    return world.diagnostics.contact_candidate_overflow, world.diagnostics.maximum_contact_candidates_per_object


def test_the_candidate_limit_shortens_the_candidate_row():
    full, maximum = overflow()
    assert full == 0 and maximum >= 4
    limited, _ = overflow(2)
    assert limited > 0


def test_the_solver_switches_are_clamped_to_their_ranges():
    """NativeMetalSubstepSurfaceTests.swift:21-63: k below 1 is 1 and above the capacity 128 is 128; a split
    multiplier below 1 is 1; values in range pass unchanged."""
    for limit, expected in ((8, 8), (0, 1), (-5, 1), (129, 128), (100_000, 128)):
        assert WorldConfiguration((0.0, 0.0, 1.0, 1.0), candidate_limit=limit).sanitized().candidate_limit == expected
    for split, expected in ((4.0, 4.0), (0.0, 1.0), (-3.0, 1.0)):
        cfg = WorldConfiguration((0.0, 0.0, 1.0, 1.0), substep_split_multiplier=split)
        assert cfg.sanitized().substep_split_multiplier == expected
    world = BubbleWorld(WorldConfiguration((-100.0, -100.0, 100.0, 100.0), candidate_limit=100_000))
    world.submit(WorldTransaction().update_physics_material(1, PhysicsMaterial(229.0))
                 .add(BubbleDescriptor(1, (0.0, 0.0), 5.0, 1.0, 1)))
    world.advance(1.0 / 60)
    assert world.diagnostics.last_advance_issue is None and world._spec(world._state)[0].candidate_limit == 128
