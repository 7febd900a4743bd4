"""What each motion role does in a step, through the world API on a stand-in device world that forwards to the oracle,
against NativeMetalMotionRoleTests.swift:9-182. The scene is the reference test's: a bubble of radius 1 and mass 1 at
the origin (band stiffness 60) in a region of 100 x 100, K_c 1000 (stiff) or 229 (soft), and a static wall 0.25 thick
from y = -10 to 10 at a chosen x. The cases on dynamic rigid bodies (a motor torque turning a polygon) need the rigid
solver, which is not built here."""

import pytest

import clr
from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (BubbleDescriptor, BubbleDrivePolicy, BubbleWorld, Circle, ForceFieldDescriptor,
                                       MotionRole as M, MotorDrive, ObjectFilter, ParameterTransition, PathDrive,
                                       PhysicsMaterial, Polygon, RigidBodyDescriptor, TransactionRejectionReason as R,
                                       WorldConfiguration, WorldTransaction)
from test_world_api_oracle_cpu import OracleBackedWorld

BALL, WALL = 1, 2
DT = 1.0 / 60
STIFF, SOFT = 1000.0, 229.0


@pytest.fixture(autouse=True)
def oracle_backed(monkeypatch):
    monkeypatch.setattr(W, "World", OracleBackedWorld)
    monkeypatch.setattr(W, "default_context", lambda: None)


def initial(commands=None, role=M.DYNAMIC, stiffness=STIFF, wall_at=None, damping=0.0, at=(0.0, 0.0)):
    """The reference test's `initial` followed by `commands` in the same step's batch; returns the world after it."""
    world = BubbleWorld(WorldConfiguration((-50.0, -50.0, 50.0, 50.0)))
    tx = WorldTransaction().update_physics_material("m", PhysicsMaterial(stiffness, damping)) \
        .add(BubbleDescriptor(BALL, at, 1.0, 1.0, "m", motion_role=role, drive_policy=BubbleDrivePolicy(60.0)))
    if wall_at is not None:
        x = wall_at
        tx = tx.add(RigidBodyDescriptor(WALL, Polygon(((x, -10.0), (x + 0.25, -10.0), (x + 0.25, 10.0), (x, 10.0))),
                                        (0.0, 0.0)))
    world.submit(tx)
    if commands is not None:
        world.submit(commands)
    return world


def step(world, commands=None):
    if commands is not None:
        world.submit(commands)
    frame = world.advance(DT)
    assert world.diagnostics.last_advance_issue is None, world.diagnostics.last_rejection_reason
    return frame


def test_blocked_player_drive_reports_the_achieved_point_and_the_blocker_without_teleporting():
    """NativeMetalMotionRoleTests.swift:37-57: the band (K 60) presses the bubble into the wall at x = 2 with about
    400; the centre never comes within 0.1 of the wall's face and, damped by gamma 5, rests at the fixed point
    x = 2 - d(F), F = 60 (8 - x), within 0.02; the feedback names the wall, a deviation above 6 and the position."""
    world = initial(WorldTransaction().begin_player_drive(BALL, (8.0, 0.0)), wall_at=2.0, damping=5.0)
    frame = step(world)
    for _ in range(200):
        frame = step(world)
        assert frame.objects[BALL].position[0] < 1.9
    rest = frame.objects[BALL].position[0]
    equilibrium = 1.0
    for _ in range(60):
        equilibrium = 2 - clr.equilibrium_distance(60 * (8 - equilibrium), STIFF, 1.0)
    assert abs(rest - equilibrium) <= 0.02, (rest, equilibrium)
    feedback = frame.drive_feedback[0]
    assert feedback.blocking_contact.object_id == WALL
    assert feedback.deviation[0] > 6.0
    assert feedback.achieved_point == tuple(map(float, frame.objects[BALL].position))


@pytest.mark.parametrize("role", [M.DYNAMIC, M.MOTOR_DRIVEN, M.PATH_DRIVEN, M.PLAYER_DRIVEN, M.STATIC])
def test_dynamic_motor_and_band_driven_bubbles_feel_fields_while_path_and_static_do_not(role):
    """NativeMetalMotionRoleTests.swift:59-74: a directional field (12, 0) over a circle of radius 20 and the global
    force (0, 6) give the mass-1 bubble (0.2, 0.1) in one step when it is dynamic, motor-driven or held by the band at
    its own position; a path-driven or static bubble stays at rest."""
    field = ForceFieldDescriptor(3, (0.0, 0.0), "directional", Circle(20.0), force=(12.0, 0.0))
    commands = WorldTransaction().add(field).set_global_force((0.0, 6.0))
    if role == M.PLAYER_DRIVEN:
        commands = commands.begin_player_drive(BALL, (0.0, 0.0))
    world = initial(commands, role=role)
    velocity = step(world).objects[BALL].velocity
    if role in (M.DYNAMIC, M.MOTOR_DRIVEN, M.PLAYER_DRIVEN):
        assert abs(velocity[0] - 0.2) <= 1e-3 and abs(velocity[1] - 0.1) <= 1e-3, velocity
    else:
        assert tuple(velocity) == (0.0, 0.0)


def test_path_driven_bubble_stops_at_a_blocker_it_cannot_pass():
    """NativeMetalMotionRoleTests.swift:76-91: the path pushes the bubble into the wall at 6 units/s until the contact
    brakes it to a stop; the drive then reports itself stopped by the wall, the bubble stands at the wall's face with
    a dent below 0.1 % of its radius, and it stays there."""
    world = initial(WorldTransaction().set_path_drive(BALL, PathDrive(((8.0, 0.0), (8.0, 8.0)), 6.0)),
                    wall_at=2.0, damping=5.0)
    for _ in range(61):
        frame = step(world)
    feedback = frame.drive_feedback[0]
    assert feedback.is_stopped
    assert feedback.blocking_contact.object_id == WALL
    assert feedback.achieved_point[0] <= 1.001
    position = feedback.achieved_point
    for _ in range(5):
        frame = step(world)
    x = frame.objects[BALL].position[0]
    assert abs(x - position[0]) <= 1e-3 and x <= position[0]


def test_player_drive_after_a_stopped_path_reports_only_the_current_drive():
    """NativeMetalMotionRoleTests.swift:93-107."""
    world = initial(WorldTransaction().set_path_drive(BALL, PathDrive(((8.0, 0.0),), 6.0)), wall_at=2.0, damping=5.0)
    for _ in range(61):
        frame = step(world)
    assert frame.drive_feedback[0].is_stopped
    assert frame.drive_feedback[0].blocking_contact.object_id == WALL
    frame = step(world, WorldTransaction().begin_player_drive(BALL, (-8.0, 0.0)))
    feedback = frame.drive_feedback[0]
    assert world._state.bubbles[BALL].desc.motion_role == M.PLAYER_DRIVEN
    assert feedback.target == (-8.0, 0.0)
    assert not feedback.is_stopped
    assert feedback.blocking_contact is None


def test_grab_and_release_keep_the_collision_radius_at_the_target_radius():
    """NativeMetalMotionRoleTests.swift:109-124: a soft bubble dented by the wall at x = 0.7 keeps its collision
    radius at the target radius while grabbed and after release."""
    world = initial(stiffness=SOFT, wall_at=0.7)
    assert step(world).objects[BALL].effective_radius < 0.99
    step(world, WorldTransaction().begin_player_drive(BALL, (-3.0, 0.0)))
    assert world._state.bubbles[BALL].desc.radius == 1.0
    for _ in range(20):
        step(world)
        assert world._state.bubbles[BALL].desc.radius == 1.0
    step(world, WorldTransaction().end_player_drive(BALL))
    assert world._state.bubbles[BALL].desc.radius == 1.0


def test_motor_force_and_transitions_advance_on_simulation_time():
    """NativeMetalMotionRoleTests.swift:126-140: after one step of 1/60 s the global force, the radius and the
    material's damping have gone 1/60 of the way to their targets, the motor's force 6 has given the bubble 0.1, and
    a transition of zero duration replaces the running one at once."""
    commands = WorldTransaction().set_motor_drive(BALL, MotorDrive((6.0, 0.0))) \
        .start_transition(ParameterTransition(("globalForce",), (0.0, 12.0), 1.0)) \
        .start_transition(ParameterTransition(("bubbleRadius", BALL), 2.0, 1.0)) \
        .start_transition(ParameterTransition(("physicsMaterial", "m", "damping"), 0.6, 1.0))
    world = initial(commands)
    frame = step(world)
    assert abs(world.global_force[1] - 0.2) <= 1e-4
    assert abs(world._state.bubbles[BALL].desc.radius - (1 + 1.0 / 60)) <= 1e-4
    assert abs(world.physics_materials["m"].damping - 0.01) <= 1e-4
    assert frame.objects[BALL].velocity[0] > 0.099
    step(world, WorldTransaction().start_transition(ParameterTransition(("globalForce",), (0.0, -12.0), 0.0)))
    assert tuple(world.global_force) == (0.0, -12.0)


def test_a_body_cannot_be_grabbed():
    """NativeMetalMotionRoleTests.swift:142-152: a player drive on a rigid body is refused with
    incompatibleObjectKind and leaves its role as it was."""
    world = initial(wall_at=2.0)
    step(world)
    token = world.submit(WorldTransaction().begin_player_drive(WALL, (8.0, 0.0)))
    frame = world.advance(DT)
    rejected = [e for e in frame.events if e.kind == "transactionRejected" and e.token == token]
    assert len(rejected) == 1 and rejected[0].rejection.reason == R.INCOMPATIBLE_OBJECT_KIND
    assert rejected[0].rejection.operation_index == 0
    assert world._state.bodies[WALL].desc.motion_role == M.STATIC


@pytest.mark.parametrize("kind, expected", [("radial", (-0.1, 0.0)), ("vortex", (0.0, 0.1))])
def test_radial_and_vortex_fields_act_through_their_falloff(kind, expected):
    """NativeMetalMotionRoleTests.swift:162-173: a bubble at (5, 0) in a field of radius 10 about the origin with
    falloff 1 (radial strength -12, vortex 12) and a filter naming it gains `expected` in one step."""
    strength = -12.0 if kind == "radial" else 12.0
    field = ForceFieldDescriptor(3, (0.0, 0.0), kind, Circle(10.0), strength=strength, falloff=1.0,
                                 filter=ObjectFilter(frozenset({BALL})))
    world = initial(WorldTransaction().add(field), at=(5.0, 0.0))
    velocity = step(world).objects[BALL].velocity
    assert abs(velocity[0] - expected[0]) <= 1e-4 and abs(velocity[1] - expected[1]) <= 1e-4, velocity


def test_a_field_whose_filter_takes_nothing_has_no_effect():
    """NativeMetalMotionRoleTests.swift:174-180."""
    field = ForceFieldDescriptor(3, (0.0, 0.0), "directional", Circle(10.0), force=(100.0, 100.0),
                                 filter=ObjectFilter(frozenset()))
    world = initial(WorldTransaction().add(field))
    assert tuple(step(world).objects[BALL].velocity) == (0.0, 0.0)
