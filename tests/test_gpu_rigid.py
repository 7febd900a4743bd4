"""Rigid solver passes on the GPU against the oracle, bit for bit, through the C ABI (bp_rigid_predict,
bp_rigid_solve_joints, bp_rigid_finish on device buffers):
- jointed chains (every joint kind, damping, limits, motors, centroid offsets, speed limits) over 30 steps: 96 links
  (all rounds in one block, rotations cached in shared memory) and 1,024 links (two grid launches per round), and
  3 steps of 20,480 links;
- bodies flung at thin walls (rotation sampling, bisection stops, wall records, kinematic pass-through, filters,
  joint exclusions, the rotation budget) and the region policy (removed, wrapped);
- records that point outside their arrays: skipped and flagged on both sides."""
import numpy as np
import pytest

from bubblephysics_gb300 import _native as N
from bubblephysics_gb300 import scenes
from bubblephysics_gb300.rigid import ITERATIONS, RigidSolver
from oracle.oracle import OracleRigid

pytestmark = pytest.mark.gpu


def same_state(gpu, cpu, where):
    gb, cb = gpu.bodies(), cpu.bodies()
    for field in ("pose", "previous", "motion", "flags", "limits"):
        assert np.array_equal(gb[field], cb[field]), f"{where}: bodies.{field}"
    assert np.array_equal(gpu.joints()["state"], cpu.joints()["state"]), f"{where}: joint state"
    gw, cw = gpu.walls(), cpu.walls()
    assert np.array_equal(gw["participants"], cw["participants"]), f"{where}: walls"
    assert np.array_equal(gw["geometry"], cw["geometry"]) and np.array_equal(gw["extra"], cw["extra"]), where
    assert gpu.safety() == cpu.safety(), f"{where}: safety {gpu.safety()} != {cpu.safety()}"


def pair(scene, bubble_count=0):
    arrays = scene.joint_arrays(range(1, bubble_count + 1))
    return (RigidSolver(scene.bodies, scene.vertices, scene.segments, arrays, bubble_count),
            OracleRigid(scene.bodies, scene.vertices, scene.segments, arrays, bubble_count))


@pytest.mark.parametrize("chains,links,bubbles", [(8, 12, 0), (64, 16, 5)])  # one block; grid launches
def test_jointed_chains_match_the_oracle(ctx, chains, links, bubbles):
    scene = scenes.jointed_chains(seed=21 + chains, chains=chains, links=links)
    gpu, cpu = pair(scene, bubbles)
    for step in range(30):
        for side in (gpu, cpu):
            side.step(scene.dt, scene.region, ITERATIONS)
        same_state(gpu, cpu, f"step {step}")
    moved = gpu.bodies()["pose"][:, :2] - scene.bodies["pose"][:, :2]
    assert np.abs(moved).max() > 0.1


def test_large_world_joint_rounds(ctx):
    """20,480 jointed links: two grid launches per round, rotations and damping factors computed in place."""
    scene = scenes.jointed_chains(seed=5, chains=640, links=32)
    gpu, cpu = pair(scene)
    for step in range(3):
        for side in (gpu, cpu):
            side.predict(scene.dt)
            side.solve_joints(scene.dt, ITERATIONS, ITERATIONS)
        same_state(gpu, cpu, f"step {step}")


def test_single_rounds_equal_one_launch_of_all_rounds(ctx):
    scene = scenes.jointed_chains(seed=9, chains=8, links=8)
    fused, single = pair(scene)[0], pair(scene)[0]
    fused.solve_joints(scene.dt, ITERATIONS, ITERATIONS)
    for _ in range(ITERATIONS):
        single.solve_joints(scene.dt, 1, ITERATIONS)
    assert np.array_equal(fused.bodies()["pose"], single.bodies()["pose"])
    assert np.array_equal(fused.joints()["state"], single.joints()["state"])


def test_sweeps_walls_and_region_match_the_oracle(ctx):
    scene = scenes.rigid_sweeps()
    gpu, cpu = pair(scene)
    wall_records, region_results = 0, set()
    for step in range(6):
        for side in (gpu, cpu):
            side.predict(scene.dt)
        same_state(gpu, cpu, f"predict {step}")
        wall_records += int((gpu.walls()["participants"][:, 0] != 0).sum())
        for side in (gpu, cpu):
            side.finish(scene.region)
        same_state(gpu, cpu, f"finish {step}")
        region_results |= set(np.unique(gpu.bodies()["flags"][:, 2]).tolist())
    assert gpu.safety() & N.RIGID_SAFETY_ROTATION_BUDGET
    assert wall_records > 0  # the first step stops bodies at walls of static owners
    assert region_results == {0, 1, 2}  # wrapped once (then inside), removed every step


def test_records_outside_their_arrays_are_skipped_and_flagged(ctx):
    scene = scenes.jointed_chains(seed=3, chains=2, links=4)
    arrays = scene.joint_arrays()
    arrays.records[1]["ends"][1] = len(scene.bodies) + 7        # an end past the bodies
    arrays.ranges[2][1] = 50                                      # a reference list past the references
    bodies = scene.bodies.copy()
    bodies[0]["ranges"][0] = len(scene.vertices)                  # vertices past the vertex array
    gpu = RigidSolver(bodies, scene.vertices, scene.segments, arrays)
    cpu = OracleRigid(bodies, scene.vertices, scene.segments, arrays)
    for side in (gpu, cpu):
        side.step(scene.dt, scene.region, ITERATIONS)
    same_state(gpu, cpu, "invalid records")
    assert gpu.safety() & N.RIGID_SAFETY_INVALID


@pytest.mark.parametrize("row_width", [32, 8])  # 8: the floors' rows overflow and keep their smallest keys
def test_pile_whole_rigid_step_matches_the_oracle(ctx, row_width):
    """Boxes, circles and capsules dropped on static floors: body-pair rows, CCD, contact rounds with friction and
    restitution, joint rounds and the wall guard, 25 steps of the reference's whole rigid step."""
    scene = scenes.rigid_pile(count=192)
    arrays = scene.joint_arrays()
    gpu = RigidSolver(scene.bodies, scene.vertices, scene.segments, arrays, triangles=scene.triangles,
                      row_width=row_width)
    cpu = OracleRigid(scene.bodies, scene.vertices, scene.segments, arrays, triangles=scene.triangles,
                      row_width=row_width)
    for step in range(25):
        for side in (gpu, cpu):
            side.step(scene.dt, scene.region)
        same_state(gpu, cpu, f"step {step}")
        (rows_g, counts_g), (rows_c, counts_c) = gpu.candidates(), cpu.candidates()
        assert np.array_equal(counts_g, counts_c), f"step {step}: row counts"
        for i, n in enumerate(counts_g[:, 0]):
            assert np.array_equal(rows_g[i, :n]["participants"], rows_c[i, :n]["participants"]), (step, i)
            assert np.array_equal(rows_g[i, :n]["metadata"], rows_c[i, :n]["metadata"]), (step, i)
        assert np.array_equal(gpu.overflow(), cpu.overflow_counts()), f"step {step}: overflow"
    assert (rows_g["metadata"][:, :, 3] != 0).any()  # contacts carried normal impulses
