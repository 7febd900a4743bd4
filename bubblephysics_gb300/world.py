"""The reference's public world API for the bubble path, over this library's C ABI.

Shapes follow Sources/BubblePhysicsPublic: BubbleWorld (BubbleWorld.swift:10-420) owns the world and a queue of
transactions and publishes only completed steps; WorldTransaction (Model/WorldTransaction.swift:93-123) is a value
builder whose operations apply in order at the next step boundary; WorldFrame (Model/WorldFrame.swift:130-150) is the
last complete state with the receipts and events of the steps that produced it; advance(by:) runs a fixed-step clock
(Sources/BubblePhysicsRuntime/FixedStepDriver.swift: backlog capped by maximum_backlog, at most 8 steps per call, time
taken off only after a whole step). Contact events are compacted from the end-of-step contact records the way
NativePublicWorld.contactTransitions (NativePublicWorld.swift:340-391) does: a pair begins when it has contact now and
had none after the previous step, ends when it had contact and has none now (or one of its objects left), pairs sorted
by (smaller id, larger id) as unsigned 64-bit ids, only for pairs with an object that asked for contact events.

Kept for the bubble path: bubbles (dynamic or static, remove or wrap at the region), static circles / capsules /
polygons (polygons become one-sided edges like NativePublicWorld.step), kinematic bodies with a constant drive,
sensors (circle or polygon; enteredSensor / exitedSensor events of bubbles), physics materials, global force, impulses
and motion-role changes; each published bubble state carries its contour's effective radius and bounds
(bp_world_contours) and hit_test answers on the published state (bp_world_hit_test). Operations of the reference
outside this path (merges, splits, force fields, drives other than kinematic, render state) are rejected with
TransactionRejectionReason.UNSUPPORTED_OPERATION naming the operation, so a caller sees what is missing. Joints are
staged with the reference's checks (duplicateJointID, jointNotFound, unsupportedJointBody, ...); one can only be
kept next to a dynamic rigid body, which this world rejects at the end of the transaction, so none survives a step. The world
steps on the GPU (World, bp_world_step); there is no CPU fallback.
"""
from __future__ import annotations

import math
import sys
import weakref
from dataclasses import dataclass, field, replace
from enum import Enum

import numpy as np

from . import _native as N
from .queries import QueryIndex, RaycastHit, shape_box
from .solver import Context, World, default_context, static_polygon_edges
from .spec import WorldSpec


# ---------------------------------------------------------------------------------------------------------------------
# Model (Sources/BubblePhysicsPublic/Model)
# ---------------------------------------------------------------------------------------------------------------------
@dataclass(frozen=True)
class CollisionFilter:
    category: int = 1
    mask: int = 0xFFFFFFFF

    def accepts(self, other: "CollisionFilter") -> bool:
        """Two objects collide when each one's category is in the other's mask (CollisionFilter.collides(with:))."""
        return bool(self.category & other.mask) and bool(other.category & self.mask)

    collides_with = accepts


@dataclass(frozen=True)
class ObjectFilter:
    """The objects a sensor watches (ObjectFilter of the reference): None = every object, an empty set = none."""
    object_ids: frozenset | None = None

    def takes(self, object_id: int) -> bool:
        return self.object_ids is None or object_id in self.object_ids


@dataclass(frozen=True)
class PhysicsMaterial:
    """Contact stiffness K_c and damping gamma of a bubble material (PhysicsMaterial, Model/Resources.swift)."""
    contact_stiffness: float
    damping: float = 0.0


class MotionRole(Enum):
    DYNAMIC = "dynamic"
    STATIC = "static"
    KINEMATIC = "kinematic"
    MOTOR_DRIVEN = "motorDriven"
    PLAYER_DRIVEN = "playerDriven"
    PATH_DRIVEN = "pathDriven"


# Roles that move a body under forces (the rigid solver's bodies): the reference refuses them next to bubbles
DYNAMIC_ROLES = (MotionRole.DYNAMIC, MotionRole.MOTOR_DRIVEN, MotionRole.PLAYER_DRIVEN, MotionRole.PATH_DRIVEN)


class RegionExitPolicy(Enum):
    REMOVE = "remove"
    WRAP = "wrap"


class EventInterest(Enum):
    """The events an object asks for (EventInterest, Model/Identifiers.swift:27-41); none by default. Sensors report
    entries and exits through their own `reports_enter` / `reports_exit`."""
    CONTACT = "contact"
    DRIVE_BLOCKED = "driveBlocked"
    DID_EXIT_SIMULATION_REGION = "didExitSimulationRegion"
    DID_WRAP = "didWrap"
    DID_ADD = "didAdd"
    DID_REMOVE = "didRemove"
    DID_REPLACE = "didReplace"


@dataclass(frozen=True)
class BubbleDescriptor:
    id: int
    position: tuple
    radius: float
    mass: float
    physics_material_id: str
    velocity: tuple = (0.0, 0.0)
    motion_role: MotionRole = MotionRole.DYNAMIC
    region_exit_policy: RegionExitPolicy = RegionExitPolicy.REMOVE
    filter: CollisionFilter = CollisionFilter()
    event_interest: frozenset = frozenset()
    layer: int = 0
    drive_policy: "BubbleDrivePolicy | None" = None

    def __post_init__(self):  # BubbleDescriptor.init, Model/Objects.swift:133-160
        if not all(math.isfinite(float(v)) for v in (*self.position, *self.velocity)):
            raise ValueError("bubble position and velocity must be finite")
        if not (math.isfinite(self.radius) and self.radius > 0):
            raise ValueError("bubble.targetRadius must be finite and positive")
        if not (math.isfinite(self.mass) and self.mass > 0):
            raise ValueError("bubble.mass must be finite and positive")


@dataclass(frozen=True)
class BubbleDrivePolicy:
    """How a bubble can be grabbed by the band (BubbleDrivePolicy): F = K_band (target - x), its magnitude clamped to
    maximum_force (None: no limit)."""
    band_stiffness: float
    maximum_force: float | None = None

    def __post_init__(self):  # Model/Motion.swift:15-21
        if not (math.isfinite(self.band_stiffness) and self.band_stiffness > 0):
            raise ValueError("drive.bandStiffness out of range")
        if self.maximum_force is not None and not (math.isfinite(self.maximum_force) and self.maximum_force > 0):
            raise ValueError("drive.maximumForce out of range")


@dataclass(frozen=True)
class MotorDrive:
    """A constant force and torque on a motor-driven bubble (MotorDrive)."""
    force: tuple = (0.0, 0.0)
    torque: float = 0.0

    def __post_init__(self):  # Model/Motion.swift:41-43
        if not all(math.isfinite(float(v)) for v in self.force):
            raise ValueError("motor.force must be finite")
        if not math.isfinite(float(self.torque)):
            raise ValueError("motor.torque must be finite")


@dataclass(frozen=True)
class PathDrive:
    """A path a path-driven bubble follows at `speed` (PathDrive, Model/Motion.swift:26-35): its velocity is set at the
    start of every step towards the current point, forces and damping do not act on it, contacts do."""
    points: tuple
    speed: float

    def __post_init__(self):
        points = tuple((float(x), float(y)) for x, y in self.points)
        if not points:
            raise ValueError("path.points must not be empty")
        if not all(math.isfinite(v) for p in points for v in p):
            raise ValueError("path.point must be finite")
        if not (math.isfinite(self.speed) and self.speed > 0):
            raise ValueError("path.speed must be finite and positive")
        object.__setattr__(self, "points", points)


@dataclass(frozen=True)
class KinematicDrive:
    """The motion imposed on a kinematic body (KinematicDrive, Model/Motion.swift:74-79): `KinematicDrive.velocity`
    (a constant linear and angular velocity, tracked as an exact pose), `KinematicDrive.path` (a PathDrive, never
    blocked) or `KinematicDrive.target` (a pose reached in one step). Forces and contacts never move the body."""
    kind: str
    linear: tuple = (0.0, 0.0)
    angular: float = 0.0
    path_drive: PathDrive | None = None
    target_position: tuple = (0.0, 0.0)
    target_rotation: float = 0.0

    @staticmethod
    def velocity(linear, angular: float = 0.0) -> "KinematicDrive":
        return KinematicDrive("velocity", linear=tuple(float(v) for v in linear), angular=float(angular))

    @staticmethod
    def path(path: PathDrive) -> "KinematicDrive":
        return KinematicDrive("path", path_drive=path)

    @staticmethod
    def target(position, rotation: float = 0.0) -> "KinematicDrive":
        return KinematicDrive("target", target_position=tuple(float(v) for v in position), target_rotation=float(rotation))

    def values(self) -> tuple:
        return (*self.linear, self.angular, *self.target_position, self.target_rotation)


@dataclass(frozen=True)
class DriveBlockingContact:
    object_id: int
    point: tuple
    normal: tuple        # from the obstacle to the driven bubble


@dataclass(frozen=True)
class DriveFeedback:
    """The running result of a player drive (DriveFeedback): its target, where the bubble got, and the first contact
    standing against the drive."""
    object_id: int
    player_drive_id: int | None
    target: tuple
    achieved_point: tuple
    blocking_contact: DriveBlockingContact | None = None
    is_stopped: bool = False

    @property
    def deviation(self) -> tuple:
        """target - achieved point (DriveFeedback.deviation)."""
        return (self.target[0] - self.achieved_point[0], self.target[1] - self.achieved_point[1])


@dataclass(frozen=True)
class ForceFieldDescriptor:
    """A force field (ForceFieldDescriptor): `kind` "directional" (the constant `force`, turned by `angle`), "radial"
    or "vortex" (`strength` with `falloff`) over a circle or polygon range about `position`, acting on the bubbles its
    filter takes."""
    id: int
    position: tuple
    kind: str
    shape: object
    angle: float = 0.0
    force: tuple = (0.0, 0.0)
    strength: float = 0.0
    falloff: float = 0.0
    filter: "ObjectFilter" = None
    event_interest: frozenset = frozenset()

    def __post_init__(self):  # ForceFieldDescriptor.init and ForceField's parameters, Model/Objects.swift:321-340
        if not all(math.isfinite(float(v)) for v in (*self.position, self.angle, *self.force, self.strength)):
            raise ValueError("field position, rotation and parameters must be finite")
        if not (math.isfinite(self.falloff) and self.falloff >= 0):
            raise ValueError("field.falloff must be finite and non-negative")


@dataclass(frozen=True)
class ParameterTransition:
    """A value moved over time (ParameterTransition): `target` is ("globalForce",), ("bubbleRadius", id) or
    ("physicsMaterial", material id, "contactStiffness" | "damping"); `value` a float or, for the global force, a pair;
    `curve` "linear", "easeIn", "easeOut", "easeInOut" or ("cubicBezier", x1, y1, x2, y2)."""
    target: tuple
    value: object
    duration: float
    curve: object = "linear"


def transition_curve(curve, t):
    """Progress along a transition curve (MotionControllers.curve), in float."""
    t = np.float32(t)
    one = np.float32(1)
    if curve == "linear":
        return t
    if curve == "easeIn":
        return t * t
    if curve == "easeOut":
        return one - (one - t) * (one - t)
    if curve == "easeInOut":
        return t * t * (np.float32(3) - np.float32(2) * t)
    _, x1, y1, x2, y2 = curve

    def bezier(u, a, b):
        v = one - u
        return np.float32(3) * v * v * u * np.float32(a) + np.float32(3) * v * u * u * np.float32(b) + u * u * u
    low, high = np.float32(0), one
    for _ in range(24):
        middle = (low + high) / np.float32(2)
        if bezier(middle, x1, x2) < t:
            low = middle
        else:
            high = middle
    return one if t == 1 else bezier((low + high) / np.float32(2), y1, y2)


@dataclass(frozen=True)
class Circle:
    radius: float

    def __post_init__(self):  # RangeGeometry.circle / RigidShape.circle: a finite, positive radius
        if not (math.isfinite(self.radius) and self.radius > 0):
            raise ValueError("circle.radius must be finite and positive")


@dataclass(frozen=True)
class Capsule:
    half_length: float
    radius: float

    def __post_init__(self):
        if not (math.isfinite(self.half_length) and self.half_length > 0 and math.isfinite(self.radius) and self.radius > 0):
            raise ValueError("capsule.halfLength and capsule.radius must be finite and positive")


@dataclass(frozen=True)
class Polygon:
    """A simple polygon (PolygonGeometry, Model/Objects.swift:18-73), local to the object's position, in either
    orientation, convex or not: a repeated first vertex at the end is dropped; fewer than three vertices, a zero-length
    or doubling-back edge, edges that cross or touch and a zero area are refused, all in double."""
    points: tuple

    def __post_init__(self):
        ring = [(float(np.float32(x)), float(np.float32(y))) for x, y in self.points]
        if not all(math.isfinite(v) for p in ring for v in p):
            raise ValueError("polygon.vertex must be finite")
        if len(ring) > 1 and ring[0] == ring[-1]:
            ring.pop()
        if len(ring) < 3:
            raise ValueError("a polygon needs three vertices")
        n = len(ring)
        for i in range(n):
            a, b, c = ring[i], ring[(i + 1) % n], ring[(i + 2) % n]
            if a == b:
                raise ValueError("degenerate polygon: a zero-length edge")
            if _cross3(a, b, c) == 0 and (b[0] - a[0]) * (c[0] - b[0]) + (b[1] - a[1]) * (c[1] - b[1]) < 0:
                raise ValueError("degenerate polygon: an edge doubles back")
            for j in range(i + 2, n):
                if i == 0 and j == n - 1:
                    continue
                if _segments_touch(a, b, ring[j], ring[(j + 1) % n]):
                    raise ValueError("self-intersecting polygon")
        if sum(_cross3(ring[0], ring[k], ring[k + 1]) for k in range(1, n - 1)) == 0:
            raise ValueError("degenerate polygon: zero area")
        object.__setattr__(self, "points", tuple(ring))


def _cross3(a, b, c) -> float:
    return (b[0] - a[0]) * (c[1] - a[1]) - (b[1] - a[1]) * (c[0] - a[0])


def _segments_touch(a, b, c, d) -> bool:
    """Whether segments ab and cd share a point (crossing, touching or overlapping), in double."""
    def within(p, u, v):
        return min(u[0], v[0]) <= p[0] <= max(u[0], v[0]) and min(u[1], v[1]) <= p[1] <= max(u[1], v[1])
    abc, abd, cda, cdb = _cross3(a, b, c), _cross3(a, b, d), _cross3(c, d, a), _cross3(c, d, b)
    if (abc == 0 and within(c, a, b)) or (abd == 0 and within(d, a, b)) or \
            (cda == 0 and within(a, c, d)) or (cdb == 0 and within(b, c, d)):
        return True
    return ((abc > 0 > abd) or (abc < 0 < abd)) and ((cda > 0 > cdb) or (cda < 0 < cdb))


def polygon_triangles(points) -> tuple[np.ndarray, np.ndarray]:
    """A polygon body's device vertices (counter-clockwise, as the device's inside test and edge normals take them)
    and triangles: a fan when the polygon is convex, ear clipping otherwise."""
    local = np.asarray(points, np.float32)
    twice = sum(_cross3(local[0], local[k], local[k + 1]) for k in range(1, len(local) - 1))
    if twice < 0:
        local = local[::-1].copy()
    n = len(local)
    if all(_cross3(local[k], local[(k + 1) % n], local[(k + 2) % n]) >= 0 for k in range(n)):
        return local, np.array([[0, k, k + 1] for k in range(1, n - 1)], np.uint32)
    left, tris = list(range(n)), []
    while len(left) > 3:
        for k in range(len(left)):
            i, j, m = left[k - 1], left[k], left[(k + 1) % len(left)]
            if _cross3(local[i], local[j], local[m]) <= 0:
                continue
            others = [q for q in left if q not in (i, j, m)]
            if any(_cross3(local[i], local[j], local[q]) >= 0 and _cross3(local[j], local[m], local[q]) >= 0 and
                   _cross3(local[m], local[i], local[q]) >= 0 for q in others):
                continue
            tris.append([i, j, m])
            left.pop(k)
            break
        else:
            break  # only collinear vertices are left
    if len(left) == 3:
        tris.append(left)
    return local, np.array(tris, np.uint32).reshape(-1, 3)


@dataclass(frozen=True)
class RigidBodyDescriptor:
    id: int
    shape: object
    position: tuple
    angle: float = 0.0
    motion_role: MotionRole = MotionRole.STATIC
    velocity: tuple = (0.0, 0.0)          # kinematic drive
    angular_velocity: float = 0.0
    filter: CollisionFilter = CollisionFilter()
    event_interest: frozenset = frozenset()
    layer: int = 0

    def __post_init__(self):  # RigidBodyDescriptor.init: a finite pose
        if not all(math.isfinite(float(v)) for v in (*self.position, self.angle, *self.velocity, self.angular_velocity)):
            raise ValueError("body position, rotation and velocity must be finite")


@dataclass(frozen=True)
class SensorDescriptor:
    """A sensor (circle or polygon, local points about `position`, rotated by `angle`) reporting the bubbles and bodies
    that enter or leave it (SensorDescriptor of the reference; enteredSensor / exitedSensor events). Bodies are the
    circles, capsules and kinematic polygons; a static polygon, held by the device world as one-sided edges, is not
    reported."""
    id: int
    shape: object
    position: tuple
    angle: float = 0.0
    filter: ObjectFilter = ObjectFilter()
    reports_enter: bool = True
    reports_exit: bool = True
    event_interest: frozenset = frozenset()  # didAdd / didRemove / didReplace of the sensor itself

    def __post_init__(self):
        if not all(math.isfinite(float(v)) for v in (*self.position, self.angle)):
            raise ValueError("sensor position and rotation must be finite")


@dataclass(frozen=True)
class WorldConfiguration:
    """WorldConfiguration (Model/WorldConfiguration.swift:39-66) plus the solver switches of the path."""
    simulation_region: tuple                 # (min x, min y, max x, max y)
    fixed_time_step: float = 1.0 / 60.0
    global_force: tuple = (0.0, 0.0)
    maximum_backlog: float = 0.25
    maximum_steps_per_advance: int = 8
    gravity: tuple = (0.0, 0.0)              # acceleration on force-driven bubbles (0: the reference's behaviour)
    candidate_limit: int = 128
    substep_split_multiplier: float = 1.0    # NativeMetalConfiguration.substepSplitMultiplier
    event_buffer_capacity: int = 1024        # WorldConfiguration.eventBufferCapacity: step events per step
    contours: bool = True                    # publish the contours' effective radius and bounds with each bubble
    automatic_pause: bool = True             # WorldConfiguration.automaticPause: pause in the background
    max_contour_segment_length: float = 8.0  # ReferenceConfiguration.maxContourSegmentLength
    contour_surface_tension: float = 20.0    # ReferenceConfiguration.contourSurfaceTension
    position_tolerance: float = 1e-4         # ReferenceConfiguration.positionTolerance (contour clearance)

    def __post_init__(self):
        if not (math.isfinite(self.fixed_time_step) and self.fixed_time_step > 0):
            raise ValueError("fixedTimeStep must be finite and positive")
        if not (math.isfinite(self.maximum_backlog) and self.maximum_backlog > 0):
            raise ValueError("maximumBacklog must be finite and positive")
        if not self.event_buffer_capacity > 0:
            raise ValueError("eventBufferCapacity must be positive")

    def sanitized(self) -> "WorldConfiguration":
        """The solver switches in their ranges (NativeMetalConfiguration.sanitized): k within 1...128, a split multiplier
        below 1 (or not finite) is 1."""
        split = self.substep_split_multiplier
        return replace(self, candidate_limit=min(128, max(1, int(self.candidate_limit))),
                       substep_split_multiplier=split if math.isfinite(split) and split >= 1 else 1.0)


class TransactionRejectionReason(Enum):
    OBJECT_NOT_FOUND = "objectNotFound"
    DUPLICATE_OBJECT_ID = "duplicateObjectID"
    REPLACEMENT_ID_MISMATCH = "replacementIDMismatch"
    PHYSICS_MATERIAL_NOT_FOUND = "physicsMaterialNotFound"
    INCOMPATIBLE_OBJECT_KIND = "incompatibleObjectKind"
    INVALID_VALUE = "invalidValue"
    INVALID_PLACEMENT = "invalidPlacement"
    UNSUPPORTED_OPERATION = "unsupportedOperation"
    UNSUPPORTED_MOTION_ROLE = "unsupportedMotionRole"        # detail: (object id, role)
    INCOMPATIBLE_MOTION_ROLE = "incompatibleMotionRole"      # detail: object id
    DRIVE_ALREADY_ACTIVE = "driveAlreadyActive"              # detail: object id
    DRIVE_NOT_ACTIVE = "driveNotActive"                      # detail: object id
    INCOMPATIBLE_TRANSITION_VALUE = "incompatibleTransitionValue"
    UNSUPPORTED_BUBBLE_WITH_DYNAMIC_RIGID_BODY = "unsupportedBubbleWithDynamicRigidBody"
    DUPLICATE_JOINT_ID = "duplicateJointID"                  # detail: joint id
    JOINT_NOT_FOUND = "jointNotFound"                        # detail: joint id
    UNSUPPORTED_JOINT_BODY = "unsupportedJointBody"          # detail: joint id


@dataclass(frozen=True)
class TransactionRejection:
    operation_index: int
    reason: TransactionRejectionReason
    detail: object = None


@dataclass(frozen=True)
class TransactionReceipt:
    token: int
    created_object_ids: tuple
    removed_object_ids: tuple
    replaced_object_ids: tuple
    removed_joint_ids: tuple = ()   # ascending: removed by remove_joint or with a body they joined


@dataclass(frozen=True)
class ObjectState:
    kind: str                 # "bubble", "polygon", "circle", "capsule"
    position: tuple
    velocity: tuple
    rotation: float
    angular_velocity: float
    bounds: tuple             # (min x, min y, max x, max y); a bubble's covers its deformed contour
    effective_radius: float | None = None  # bubble: the contour's smallest distance from the centre


@dataclass(frozen=True)
class WorldEvent:
    """kind: transactionRejected, didAdd, didRemove, didReplace, didExitSimulationRegion, didWrap, contactBegan,
    contactEnded, enteredSensor, exitedSensor (objects = (sensor, bubble or body)), driveBlocked (objects = (bubble,
    obstacle))."""
    kind: str
    objects: tuple = ()
    point: tuple | None = None
    normal: tuple | None = None
    impulse: float | None = None
    token: int | None = None
    rejection: TransactionRejection | None = None


@dataclass(frozen=True)
class WorldEventOverflow:
    """The step events that did not fit the event buffer (WorldEventOverflow)."""
    dropped_count: int = 0


@dataclass(frozen=True)
class WorldFrame:
    step_index: int = 0
    simulation_time: float = 0.0
    transaction_receipts: tuple = ()
    events: tuple = ()
    objects: dict = field(default_factory=dict)
    drive_feedback: tuple = ()                   # DriveFeedback of every active player drive, ascending by id
    event_overflow: WorldEventOverflow = WorldEventOverflow()


class WorldFailureReason(Enum):
    SUBSTEP_LIMIT_EXCEEDED = "substepLimitExceeded"
    NON_FINITE_VALUES = "nonFiniteValues"
    CONTACT_VIOLATION = "contactViolation"
    COMMAND_EXECUTION_FAILED = "commandExecutionFailed"


class WorldRejectionReason(str, Enum):
    """Why a step was rejected without ending the world (WorldRejectionReason): the queue and the time stay for a
    retry."""
    SOLVER_GUARD = "solverGuard"
    INVALID_FRAME = "invalidFrame"
    INVALID_SNAPSHOT = "invalidSnapshot"
    FRAME_IN_FLIGHT = "frameInFlight"
    UNEXPECTED = "unexpected"


class AdvanceIssue(str, Enum):
    """Why an advance published nothing new (WorldAdvanceIssue of the reference)."""
    WORLD_FAILED = "worldFailed"
    INVALID_TIME_DELTA = "invalidTimeDelta"
    TIME_ACCUMULATOR_OVERFLOW = "timeAccumulatorOverflow"
    STEP_FAILED = "stepFailed"


@dataclass
class WorldDiagnostics:
    backlog_seconds: float = 0.0
    discarded_backlog_seconds: float = 0.0
    consecutive_backlogged_advances: int = 0
    last_advance_issue: AdvanceIssue | None = None
    last_rejection_reason: WorldRejectionReason | None = None
    steps_in_last_advance: int = 0
    last_step_substeps: int = 0            # NativeMetalFrameTelemetry.substepCount of the last completed step
    last_step_rebuilds: int = 0            # its grid rebuilds
    pending_transaction_count: int = 0
    is_paused: bool = False
    contact_candidate_overflow: int = 0
    maximum_contact_candidates_per_object: int = 0
    failure_reason: WorldFailureReason | None = None
    failure_detail: dict | None = None


# ---------------------------------------------------------------------------------------------------------------------
# Transactions (value builder: every method returns a copy)
# ---------------------------------------------------------------------------------------------------------------------
@dataclass(frozen=True)
class WorldTransaction:
    operations: tuple = ()

    def _with(self, *op) -> "WorldTransaction":
        return WorldTransaction(self.operations + (op,))

    def add(self, obj) -> "WorldTransaction":
        return self._with("add", obj)

    def remove(self, object_id: int) -> "WorldTransaction":
        return self._with("remove", object_id)

    def add_joint(self, joint) -> "WorldTransaction":
        """`joint` is a rigid.Joint (WorldTransaction.addJoint, Model/WorldTransaction.swift:121)."""
        return self._with("addJoint", joint)

    def remove_joint(self, joint_id: int) -> "WorldTransaction":
        return self._with("removeJoint", joint_id)

    def replace(self, object_id: int, obj) -> "WorldTransaction":
        return self._with("replace", object_id, obj)

    def update_physics_material(self, material_id: str, material: PhysicsMaterial) -> "WorldTransaction":
        return self._with("updatePhysicsMaterial", material_id, material)

    def set_motion(self, object_id: int, role: MotionRole) -> "WorldTransaction":
        return self._with("setMotion", object_id, role)

    def update_render_material(self, material_id, material=None) -> "WorldTransaction":
        """Accepted and kept for the renderer, which is not part of this path; it takes its place in the operation
        order like the reference's."""
        return self._with("updateRenderMaterial", material_id, material)

    def set_global_force(self, force) -> "WorldTransaction":
        return self._with("setGlobalForce", tuple(float(v) for v in force))

    def apply_impulse(self, object_id: int, impulse) -> "WorldTransaction":
        return self._with("applyImpulse", object_id, tuple(float(v) for v in impulse))

    def set_motor_drive(self, object_id: int, drive: "MotorDrive") -> "WorldTransaction":
        return self._with("setMotorDrive", object_id, drive)

    def set_path_drive(self, object_id: int, drive: PathDrive) -> "WorldTransaction":
        return self._with("setPathDrive", object_id, drive)

    def begin_player_drive(self, object_id: int, target) -> "WorldTransaction":
        return self._with("beginPlayerDrive", object_id, tuple(float(v) for v in target))

    def update_player_drive(self, object_id: int, target) -> "WorldTransaction":
        return self._with("updatePlayerDrive", object_id, tuple(float(v) for v in target))

    def end_player_drive(self, object_id: int) -> "WorldTransaction":
        return self._with("endPlayerDrive", object_id)

    def start_transition(self, transition: ParameterTransition) -> "WorldTransaction":
        return self._with("startTransition", transition)

    def set_layer(self, object_id: int, layer: int) -> "WorldTransaction":
        return self._with("setLayer", object_id, int(layer))

    def set_kinematic_drive(self, object_id: int, drive, angular_velocity: float = 0.0) -> "WorldTransaction":
        """`drive` is a KinematicDrive, or a linear velocity (with `angular_velocity`) for KinematicDrive.velocity."""
        if not isinstance(drive, KinematicDrive):
            drive = KinematicDrive.velocity(drive, angular_velocity)
        return self._with("setKinematicDrive", object_id, drive)

    def operation(self, name: str, *args) -> "WorldTransaction":
        """Any other operation of the reference's transaction (merges, splits, joints, sensors, ...): recorded, and
        rejected at the step boundary as unsupported by this backend."""
        return self._with(name, *args)


# ---------------------------------------------------------------------------------------------------------------------
# Runtime state and staging
# ---------------------------------------------------------------------------------------------------------------------
@dataclass
class _Bubble:
    desc: BubbleDescriptor
    position: np.ndarray
    velocity: np.ndarray
    rotation: float = 0.0
    angular_velocity: float = 0.0
    motor: MotorDrive | None = None            # motor-driven
    drive_target: tuple | None = None          # player-driven: the band's target
    drive_id: int | None = None
    motion_before_drive: "MotionRole | None" = None
    path: PathDrive | None = None              # path-driven: the path, the point it heads for, and the stop
    path_index: int = 0
    path_stopped: bool = False
    path_blocker: "DriveBlockingContact | None" = None


@dataclass
class _Body:
    desc: RigidBodyDescriptor
    position: np.ndarray
    angle: float
    drive: KinematicDrive | None = None        # kinematic: the drive, this step's velocity, the exact pose it tracks
    velocity: np.ndarray = field(default_factory=lambda: np.zeros(2, np.float32))
    angular_velocity: float = 0.0
    exact: tuple | None = None
    path_index: int = 0

    @staticmethod
    def of(desc: RigidBodyDescriptor) -> "_Body":
        """A body as added: a kinematic descriptor's velocity is its first drive."""
        drive = None
        if desc.motion_role == MotionRole.KINEMATIC and any(v != 0 for v in (*desc.velocity, desc.angular_velocity)):
            drive = KinematicDrive.velocity(desc.velocity, desc.angular_velocity)
        return _Body(desc, np.asarray(desc.position, np.float32).copy(), float(desc.angle), drive)


@dataclass
class _State:
    materials: dict = field(default_factory=dict)
    bubbles: dict = field(default_factory=dict)   # id -> _Bubble
    bodies: dict = field(default_factory=dict)    # id -> _Body
    global_force: tuple = (0.0, 0.0)
    sensors: dict = field(default_factory=dict)   # id -> SensorDescriptor
    fixed_time_step: float = 1.0 / 60.0          # for the band's stability bound
    next_drive_id: int = 1
    transitions: dict = field(default_factory=dict)          # target -> ParameterTransition
    transition_progress: dict = field(default_factory=dict)  # target -> (initial value, elapsed seconds)
    fields: dict = field(default_factory=dict)               # id -> ForceFieldDescriptor
    joints: dict = field(default_factory=dict)               # joint id -> rigid.Joint

    def copy(self) -> "_State":
        return _State(dict(self.materials),
                      {k: replace(v, position=v.position.copy(), velocity=v.velocity.copy()) for k, v in self.bubbles.items()},
                      {k: replace(v, position=v.position.copy(), velocity=v.velocity.copy()) for k, v in self.bodies.items()},
                      self.global_force, dict(self.sensors), self.fixed_time_step, self.next_drive_id,
                      dict(self.transitions), dict(self.transition_progress), dict(self.fields), dict(self.joints))


def _finite(*values) -> bool:
    return all(math.isfinite(float(v)) for v in values)


class PlacementIssue(str, Enum):
    """Why a bubble's centre cannot stand at a point (PlacementIssue of the reference), in the order they are checked."""
    OUTSIDE_REGION = "outsideRegion"
    INSIDE_RIGID_BODY = "insideRigidBody"
    COINCIDENT_CENTER = "coincidentCenter"


_F = np.float32
POSITION_TOLERANCE = _F(1e-4)  # PlacementGeometry.positionTolerance
MAXIMUM_DRIVE_MAGNITUDE = 1e6   # TransactionStager.maximumDriveMagnitude: larger finite drives overflow float in a step


def _body_shape(body: _Body):
    """The body's shape in the world at its pose, in float: ("circle", c, r), ("capsule", a, b, r) or ("polygon", ring)."""
    c, s = _F(math.cos(body.angle)), _F(math.sin(body.angle))
    px, py = _F(body.position[0]), _F(body.position[1])

    def world(x, y):
        x, y = _F(x), _F(y)
        return np.array([px + x * c - y * s, py + x * s + y * c], np.float32)
    shape = body.desc.shape
    if isinstance(shape, Circle):
        return ("circle", np.array([px, py], np.float32), _F(shape.radius))
    if isinstance(shape, Capsule):
        return ("capsule", world(-shape.half_length, 0.0), world(shape.half_length, 0.0), _F(shape.radius))
    return ("polygon", [world(x, y) for x, y in shape.points])


def _distance_to_segment(p, a, b):
    e = b - a
    sq = _F(e[0] * e[0] + e[1] * e[1])
    t = max(_F(0), min(_F(1), _F((p[0] - a[0]) * e[0] + (p[1] - a[1]) * e[1]) / sq)) if sq > 0 else _F(0)
    d = p - (a + e * t)
    return _F(math.sqrt(float(d[0] * d[0] + d[1] * d[1])))


def _contains_including_boundary(shape, p) -> bool:
    """Point-in-shape with the boundary inside (PlacementGeometry.containsIncludingBoundary): circles and capsules by
    distance (<=), polygons by an exact on-edge test, then the crossing parity."""
    if shape[0] == "circle":
        d = p - shape[1]
        return bool(d[0] * d[0] + d[1] * d[1] <= shape[2] * shape[2])
    if shape[0] == "capsule":
        return bool(_distance_to_segment(p, shape[1], shape[2]) <= shape[3])
    ring = shape[1]
    j = len(ring) - 1
    for i in range(len(ring)):
        a, b = ring[i], ring[j]
        j = i
        cross = (b[0] - a[0]) * (p[1] - a[1]) - (b[1] - a[1]) * (p[0] - a[0])
        if cross == 0 and min(a[0], b[0]) <= p[0] <= max(a[0], b[0]) and min(a[1], b[1]) <= p[1] <= max(a[1], b[1]):
            return True
    inside = False
    j = len(ring) - 1
    for i in range(len(ring)):
        a, b = ring[i], ring[j]
        if (a[1] > p[1]) != (b[1] > p[1]) and p[0] <= (b[0] - a[0]) * (p[1] - a[1]) / (b[1] - a[1]) + a[0]:
            inside = not inside
        j = i
    return inside


def placement_issue(point, radius: float, filt: CollisionFilter, state: _State, region,
                    excluding=frozenset()) -> PlacementIssue | None:
    """The first reason a bubble's centre cannot stand at `point` (PlacementGeometry.issue): outside the region
    (whatever its exit policy), inside a body it collides with (boundary included), or within the coincident-centre
    tolerance max(1e-4 min(r, r_other), 1e-4) of a bubble it collides with. Excluded ids take no part."""
    p = np.asarray(point, np.float32)
    if not (region[0] <= p[0] <= region[2] and region[1] <= p[1] <= region[3]):
        return PlacementIssue.OUTSIDE_REGION
    for oid, body in state.bodies.items():
        if oid not in excluding and filt.accepts(body.desc.filter) and _contains_including_boundary(_body_shape(body), p):
            return PlacementIssue.INSIDE_RIGID_BODY
    for oid, other in state.bubbles.items():
        if oid in excluding or not filt.accepts(other.desc.filter):
            continue
        tolerance = max(_F(1e-4) * min(_F(radius), _F(other.desc.radius)), POSITION_TOLERANCE)
        d = p - np.asarray(other.position, np.float32)
        if _F(math.sqrt(float(d[0] * d[0] + d[1] * d[1]))) < tolerance:
            return PlacementIssue.COINCIDENT_CENTER
    return None


def _not_physical(state: _State, oid: int):
    """The rejection for an id that names no bubble or body: a sensor or a force field has no motion
    (TransactionStager.physicalObject), anything else is not found."""
    if oid in state.sensors or oid in state.fields:
        return TransactionRejectionReason.INCOMPATIBLE_OBJECT_KIND, oid
    return TransactionRejectionReason.OBJECT_NOT_FOUND


def _set_bubble_motion(b: _Bubble, oid: int, role: MotionRole):
    """setMotion of a bubble (TransactionStager.swift:268-281): the player-driven role needs a running player drive;
    leaving a role drops its drive (the band, the path, the motor)."""
    if role == MotionRole.KINEMATIC:
        return TransactionRejectionReason.UNSUPPORTED_MOTION_ROLE, (oid, role)
    if role == MotionRole.PLAYER_DRIVEN and b.drive_target is None:
        return TransactionRejectionReason.DRIVE_NOT_ACTIVE, oid
    b.desc = replace(b.desc, motion_role=role)
    if role != MotionRole.PLAYER_DRIVEN:
        b.drive_target = b.drive_id = b.motion_before_drive = None
    if role != MotionRole.PATH_DRIVEN:
        b.path, b.path_index, b.path_stopped, b.path_blocker = None, 0, False, None
    if role != MotionRole.MOTOR_DRIVEN:
        b.motor = None
    if role == MotionRole.STATIC:
        b.velocity[:] = 0
    return None


STATIC_OUTSIDE = "staticGeometryOutsideSimulationRegion"


def _circle_inside(center, radius, region) -> bool:
    x, y, r = float(np.float32(center[0])), float(np.float32(center[1])), float(np.float32(radius))
    return x - r >= region[0] and x + r <= region[2] and y - r >= region[1] and y + r <= region[3]


def _range_inside(shape, position, angle, region) -> bool:
    """A circle or polygon range about `position`, turned by `angle`, lies in the region (WorldConfiguration.swift:
    95-119, in double)."""
    if isinstance(shape, Circle):
        return _circle_inside(position, shape.radius, region)
    c, s = math.cos(float(np.float32(angle))), math.sin(float(np.float32(angle)))
    px, py = float(np.float32(position[0])), float(np.float32(position[1]))
    for vx, vy in shape.points:
        vx, vy = float(np.float32(vx)), float(np.float32(vy))
        x, y = px + vx * c - vy * s, py + vx * s + vy * c
        if not (region[0] <= x <= region[2] and region[1] <= y <= region[3]):
            return False
    return True


def static_geometry_inside(obj, region, state: _State | None = None, role=None, position=None, angle=None) -> bool:
    """WorldConfiguration.validate for this path: a static bubble (at the largest radius a scheduled transition takes
    it to), a static body, a sensor and a force field lie wholly in the simulation region; other roles are not held
    to it. `role`, `position` and `angle` give the object's runtime values when they differ from its descriptor."""
    role = role or getattr(obj, "motion_role", None)
    position = obj.position if position is None else position
    if isinstance(obj, (SensorDescriptor, ForceFieldDescriptor)):
        return _range_inside(obj.shape, position, obj.angle, region)
    if role != MotionRole.STATIC:
        return True
    if isinstance(obj, BubbleDescriptor):
        radius = float(np.float32(obj.radius))
        scheduled = state.transitions.get(("bubbleRadius", obj.id)) if state is not None else None
        if scheduled is not None:
            radius = max(radius, float(np.float32(scheduled.value)))
        return _circle_inside(position, radius, region)
    angle = obj.angle if angle is None else angle
    shape = obj.shape
    if isinstance(shape, Capsule):  # the axis' two ends, each with a circle of the radius
        rot = np.float32(angle)
        axis = np.array([np.cos(rot), np.sin(rot)], np.float32) * np.float32(shape.half_length)
        p = np.asarray(position, np.float32)
        return _circle_inside(p + axis, shape.radius, region) and _circle_inside(p - axis, shape.radius, region)
    return _range_inside(shape, position, angle, region)


def _validate_bubble(desc: BubbleDescriptor, state: _State, region):
    if desc.physics_material_id not in state.materials:
        return TransactionRejectionReason.PHYSICS_MATERIAL_NOT_FOUND
    if not (_finite(*desc.position, *desc.velocity, desc.radius, desc.mass) and desc.radius > 0 and desc.mass > 0):
        return TransactionRejectionReason.INVALID_VALUE
    if desc.motion_role == MotionRole.KINEMATIC:  # kinematic bubbles do not exist (TransactionStager.swift:510-513)
        return TransactionRejectionReason.UNSUPPORTED_MOTION_ROLE, (desc.id, desc.motion_role)
    policy = desc.drive_policy
    if policy is not None:
        if not (_finite(policy.band_stiffness) and policy.band_stiffness > 0):
            return TransactionRejectionReason.INVALID_VALUE, "drive.bandStiffness"
        if policy.maximum_force is not None and not (_finite(policy.maximum_force) and policy.maximum_force > 0):
            return TransactionRejectionReason.INVALID_VALUE, "drive.maximumForce"
        # the band stays stable while omega_band dt <= 1/4: K_band <= m / (16 dt^2), in the world's float step
        step = float(np.float32(state.fixed_time_step))
        if not float(np.float32(policy.band_stiffness)) * 16 * step * step <= float(np.float32(desc.mass)):
            return TransactionRejectionReason.INVALID_VALUE, "drive.bandStiffness"
    if not static_geometry_inside(desc, region, state):
        return TransactionRejectionReason.INVALID_VALUE, STATIC_OUTSIDE
    issue = placement_issue(desc.position, desc.radius, desc.filter, state, region, frozenset({desc.id}))
    if issue is not None:
        return TransactionRejectionReason.INVALID_PLACEMENT, (desc.id, issue)
    return None


def _validate_body(desc: RigidBodyDescriptor, state: _State, region) -> TransactionRejectionReason | None:
    shape = desc.shape
    sizes = {Circle: lambda s: (s.radius,), Capsule: lambda s: (s.half_length, s.radius)}.get(type(shape))
    if sizes is not None:
        if not (_finite(*sizes(shape)) and min(sizes(shape)) > 0):
            return TransactionRejectionReason.INVALID_VALUE
    elif isinstance(shape, Polygon):
        if len(shape.points) < 3 or not _finite(*np.ravel(shape.points)):
            return TransactionRejectionReason.INVALID_VALUE
    else:
        return TransactionRejectionReason.INVALID_VALUE
    if not _finite(*desc.position, desc.angle, *desc.velocity, desc.angular_velocity):
        return TransactionRejectionReason.INVALID_VALUE
    if not static_geometry_inside(desc, region):
        return TransactionRejectionReason.INVALID_VALUE, STATIC_OUTSIDE
    # a body may not cover the centre of a bubble it collides with; the smallest such id is named
    # (PlacementGeometry.bubbleInside)
    shape = _body_shape(_Body(desc, np.asarray(desc.position, np.float64), float(desc.angle)))
    inside = [oid for oid, b in state.bubbles.items()
              if b.desc.filter.accepts(desc.filter) and _contains_including_boundary(shape, np.asarray(b.position, np.float32))]
    if inside:
        return TransactionRejectionReason.INVALID_PLACEMENT, (min(inside, key=lambda v: v & 0xFFFFFFFFFFFFFFFF),
                                                             PlacementIssue.INSIDE_RIGID_BODY)
    return None


def _add_joint(joint, state: _State):
    """TransactionStager.add(_ joint:) (TransactionStager.swift:444-470) with the Joint initialiser's checks
    (Model/Joints.swift:56-66): a new id; finite anchors and reference angle; two different objects; distance length,
    softness and damping not negative; every drive-like value within 1e6; ends that are bubbles or rigid bodies; and
    at least one movable rigid body (dynamic, motor- or player-driven) and no bubble or path-driven end
    (jointBodiesAreSupported). Returns the rejection or None (the joint is then kept)."""
    if joint.id in state.joints:
        return TransactionRejectionReason.DUPLICATE_JOINT_ID, joint.id
    if joint.body_b is not None and joint.body_b == joint.body_a:
        return TransactionRejectionReason.INVALID_VALUE, "joint.bodies"
    checks = [("joint.anchorA", tuple(joint.anchor_a)), ("joint.anchorB", tuple(joint.anchor_b)),
              ("joint.referenceAngle", (joint.reference_angle,))]
    if joint.kind == "distance":
        checks += [("joint.length", (joint.length,)), ("joint.softness", (joint.softness,)),
                   ("joint.damping", (joint.damping,))]
        for name, value in (("joint.length", joint.length), ("joint.softness", joint.softness),
                            ("joint.damping", joint.damping)):
            if _finite(value) and value < 0:
                return TransactionRejectionReason.INVALID_VALUE, name
    elif joint.kind == "hinge":
        if joint.limits is not None:
            checks += [("hinge.lower", (joint.limits[0],)), ("hinge.upper", (joint.limits[1],))]
        if joint.motor is not None:
            checks += [("hinge.motor.targetAngularVelocity", (joint.motor[0],))]
    elif joint.kind != "weld":
        return TransactionRejectionReason.INVALID_VALUE, "joint.kind"
    for name, values in checks:
        if not _finite(*values) or any(abs(float(np.float32(v))) > MAXIMUM_DRIVE_MAGNITUDE for v in values):
            return TransactionRejectionReason.INVALID_VALUE, name
    ends = [joint.body_a] + ([joint.body_b] if joint.body_b is not None else [])
    for oid in ends:
        if oid in state.sensors or oid in state.fields:
            return TransactionRejectionReason.INCOMPATIBLE_OBJECT_KIND, oid
        if oid not in state.bubbles and oid not in state.bodies:
            return TransactionRejectionReason.OBJECT_NOT_FOUND, oid
    movable = False
    for oid in ends:
        if oid in state.bubbles:  # no joints with bubbles in the v4 engine
            return TransactionRejectionReason.UNSUPPORTED_JOINT_BODY, joint.id
        role = state.bodies[oid].desc.motion_role
        if role == MotionRole.PATH_DRIVEN:
            return TransactionRejectionReason.UNSUPPORTED_JOINT_BODY, joint.id
        movable = movable or role in (MotionRole.DYNAMIC, MotionRole.MOTOR_DRIVEN, MotionRole.PLAYER_DRIVEN)
    if not movable:
        return TransactionRejectionReason.UNSUPPORTED_JOINT_BODY, joint.id
    state.joints[joint.id] = joint
    return None


def _apply(op, state: _State, region) -> tuple[TransactionRejectionReason | None, dict]:
    """Applies one operation to `state` (a staging copy); returns (rejection reason, {created, removed, replaced})."""
    kind, args = op[0], op[1:]
    touched = {"created": [], "removed": [], "replaced": [], "removed_joints": []}
    if kind in ("add", "replace"):
        obj = args[-1]
        if kind == "replace":
            oid = args[0]
            if oid not in state.bubbles and oid not in state.bodies and oid not in state.sensors and \
                    oid not in state.fields:
                return TransactionRejectionReason.OBJECT_NOT_FOUND, touched
            if obj.id != oid:
                return TransactionRejectionReason.REPLACEMENT_ID_MISMATCH, touched
            state.bubbles.pop(oid, None)
            state.bodies.pop(oid, None)
            state.sensors.pop(oid, None)
            state.fields.pop(oid, None)
        elif obj.id in state.bubbles or obj.id in state.bodies or obj.id in state.sensors or obj.id in state.fields:
            return TransactionRejectionReason.DUPLICATE_OBJECT_ID, touched
        if isinstance(obj, BubbleDescriptor):
            reason = _validate_bubble(obj, state, region)
            if reason:
                return reason, touched
            state.bubbles[obj.id] = _Bubble(obj, np.asarray(obj.position, np.float32).copy(),
                                            np.asarray(obj.velocity, np.float32).copy())
        elif isinstance(obj, RigidBodyDescriptor):
            reason = _validate_body(obj, state, region)
            if reason:
                return reason, touched
            state.bodies[obj.id] = _Body.of(obj)
        elif isinstance(obj, ForceFieldDescriptor):
            shape = obj.shape
            ok = obj.kind in ("directional", "radial", "vortex") and \
                _finite(*obj.position, obj.angle, *obj.force, obj.strength, obj.falloff) and obj.falloff >= 0 and (
                    (isinstance(shape, Circle) and _finite(shape.radius) and shape.radius > 0) or
                    (isinstance(shape, Polygon) and len(shape.points) >= 3 and _finite(*np.ravel(shape.points))))
            if not ok:
                return TransactionRejectionReason.INVALID_VALUE, touched
            if not static_geometry_inside(obj, region):
                return (TransactionRejectionReason.INVALID_VALUE, STATIC_OUTSIDE), touched
            state.fields[obj.id] = obj
        elif isinstance(obj, SensorDescriptor):
            shape = obj.shape
            ok = _finite(*obj.position, obj.angle) and (
                (isinstance(shape, Circle) and _finite(shape.radius) and shape.radius > 0) or
                (isinstance(shape, Polygon) and len(shape.points) >= 3 and _finite(*np.ravel(shape.points))))
            if not ok:
                return TransactionRejectionReason.INVALID_VALUE, touched
            if not static_geometry_inside(obj, region):
                return (TransactionRejectionReason.INVALID_VALUE, STATIC_OUTSIDE), touched
            state.sensors[obj.id] = obj
        else:
            return TransactionRejectionReason.UNSUPPORTED_OPERATION, touched
        touched["replaced" if kind == "replace" else "created"].append(obj.id)
        return None, touched
    if kind == "remove":
        oid = args[0]
        if state.bubbles.pop(oid, None) is None and state.bodies.pop(oid, None) is None and \
                state.sensors.pop(oid, None) is None and state.fields.pop(oid, None) is None:
            return TransactionRejectionReason.OBJECT_NOT_FOUND, touched
        touched["removed"].append(oid)
        # removing an object removes its joints (TransactionStager.removeJoints, TransactionStager.swift:437-443)
        for jid in [j for j, joint in state.joints.items() if oid in (joint.body_a, joint.body_b)]:
            del state.joints[jid]
            touched["removed_joints"].append(jid)
        return None, touched
    if kind == "addJoint":
        return _add_joint(args[0], state), touched
    if kind == "removeJoint":  # TransactionStager.swift:370-373
        jid = args[0]
        if jid not in state.joints:
            return (TransactionRejectionReason.JOINT_NOT_FOUND, jid), touched
        del state.joints[jid]
        touched["removed_joints"].append(jid)
        return None, touched
    if kind == "updatePhysicsMaterial":
        mid, material = args
        if not (_finite(material.contact_stiffness, material.damping) and material.contact_stiffness >= 0 and
                material.damping >= 0):
            return TransactionRejectionReason.INVALID_VALUE, touched
        state.materials[mid] = material
        return None, touched
    if kind == "updateRenderMaterial":
        return None, touched
    if kind == "setMotion":
        oid, role = args
        b = state.bubbles.get(oid)
        if b is None:
            body = state.bodies.get(oid)
            if body is None:
                return _not_physical(state, oid), touched
            if role == MotionRole.STATIC and not static_geometry_inside(body.desc, region, role=role,
                                                                         position=body.position, angle=body.angle):
                return (TransactionRejectionReason.INVALID_VALUE, STATIC_OUTSIDE), touched
            if role != MotionRole.KINEMATIC:  # leaving the kinematic role discards the drive
                body.desc = replace(body.desc, motion_role=role, velocity=(0.0, 0.0), angular_velocity=0.0)
                body.drive, body.exact, body.path_index = None, None, 0
                body.velocity, body.angular_velocity = np.zeros(2, np.float32), 0.0
            else:
                body.desc = replace(body.desc, motion_role=role)
            return None, touched
        if role == MotionRole.STATIC and not static_geometry_inside(b.desc, region, state, role, b.position):
            return (TransactionRejectionReason.INVALID_VALUE, STATIC_OUTSIDE), touched
        return _set_bubble_motion(b, oid, role), touched
    if kind == "setPathDrive":
        oid, drive = args
        b = state.bubbles.get(oid)
        if b is None:
            return (_not_physical(state, oid) if oid not in state.bodies else
                    (TransactionRejectionReason.UNSUPPORTED_MOTION_ROLE, (oid, MotionRole.PATH_DRIVEN))), touched
        _set_bubble_motion(b, oid, MotionRole.PATH_DRIVEN)
        b.path, b.path_index, b.path_stopped, b.path_blocker = drive, 0, False, None
        return None, touched
    if kind == "setGlobalForce":
        if not _finite(*args[0]):
            return TransactionRejectionReason.INVALID_VALUE, touched
        state.global_force = args[0]
        return None, touched
    if kind == "applyImpulse":  # TransactionStager.swift:312-324
        oid, impulse = args
        if not _finite(*impulse):
            return (TransactionRejectionReason.INVALID_VALUE, "impulse"), touched
        b = state.bubbles.get(oid)
        if b is None:
            if oid in state.bodies:  # static and kinematic bodies take no impulse
                return (TransactionRejectionReason.INCOMPATIBLE_MOTION_ROLE, oid), touched
            return (TransactionRejectionReason.INCOMPATIBLE_OBJECT_KIND, oid) if oid in state.sensors or \
                oid in state.fields else TransactionRejectionReason.OBJECT_NOT_FOUND, touched
        if b.desc.motion_role not in (MotionRole.DYNAMIC, MotionRole.MOTOR_DRIVEN):
            return (TransactionRejectionReason.INCOMPATIBLE_MOTION_ROLE, oid), touched
        mass = float(np.float32(b.desc.mass))
        velocity = np.array([float(b.velocity[k]) + float(np.float32(impulse[k])) / mass for k in range(2)])
        if not np.isfinite(velocity.astype(np.float32)).all():
            return (TransactionRejectionReason.INVALID_VALUE, "velocityAfterImpulse"), touched
        b.velocity = velocity.astype(np.float32)
        return None, touched
    if kind == "setLayer":
        oid, layer = args
        if not (-2 ** 31 <= layer < 2 ** 31) and (oid in state.bubbles or oid in state.bodies):  # Int32
            return TransactionRejectionReason.INVALID_VALUE, touched
        if oid in state.bubbles:
            state.bubbles[oid].desc = replace(state.bubbles[oid].desc, layer=layer)
        elif oid in state.bodies:
            state.bodies[oid].desc = replace(state.bodies[oid].desc, layer=layer)
        else:
            return TransactionRejectionReason.OBJECT_NOT_FOUND if oid not in state.sensors else \
                TransactionRejectionReason.INCOMPATIBLE_OBJECT_KIND, touched
        return None, touched
    if kind == "startTransition":
        tr = args[0]
        if not math.isfinite(tr.duration) or tr.duration < 0:
            return (TransactionRejectionReason.INVALID_VALUE, "transition.duration"), touched
        curve = tr.curve  # TransactionStager.swift:576-614
        if not (curve in ("linear", "easeIn", "easeOut", "easeInOut") or
                (isinstance(curve, tuple) and len(curve) == 5 and curve[0] == "cubicBezier" and _finite(*curve[1:]) and
                 all(0 <= v <= 1 for v in curve[1:]) and curve[1] <= curve[3])):
            return (TransactionRejectionReason.INVALID_VALUE, "transition.curve"), touched
        target = tr.target
        vector = isinstance(tr.value, (tuple, list))
        if target[0] == "globalForce" and vector:
            if not _finite(*tr.value):
                return (TransactionRejectionReason.INVALID_VALUE, "transition.globalForce"), touched
        elif target[0] == "physicsMaterial" and len(target) == 3 and not vector:
            if target[1] not in state.materials:
                return TransactionRejectionReason.PHYSICS_MATERIAL_NOT_FOUND, touched
            if not (_finite(tr.value) and tr.value >= 0):
                return (TransactionRejectionReason.INVALID_VALUE, "transition.material"), touched
            # K_c belongs to bubble materials only; friction and restitution to rigid ones, which this path has not
            if target[2] not in ("contactStiffness", "damping") or (target[2] == "contactStiffness" and not tr.value > 0):
                return (TransactionRejectionReason.INVALID_VALUE, "transition.material"), touched
        elif target[0] == "bubbleRadius" and not vector:
            b = state.bubbles.get(target[1])
            if b is None:
                return (TransactionRejectionReason.INCOMPATIBLE_OBJECT_KIND, target[1]) if target[1] in state.bodies or \
                    target[1] in state.sensors or target[1] in state.fields else \
                    TransactionRejectionReason.OBJECT_NOT_FOUND, touched
            if not (_finite(tr.value) and tr.value > 0):
                return (TransactionRejectionReason.INVALID_VALUE, "transition.radius"), touched
            if b.desc.motion_role == MotionRole.STATIC and \
                    not _circle_inside(b.position, tr.value, region):
                return (TransactionRejectionReason.INVALID_VALUE, STATIC_OUTSIDE), touched
        else:
            return TransactionRejectionReason.INCOMPATIBLE_TRANSITION_VALUE, touched
        state.transitions[target] = tr
        state.transition_progress.pop(target, None)
        return None, touched
    if kind == "setMotorDrive":
        oid, drive = args
        values = (*drive.force, drive.torque)
        if not _finite(*values):
            return TransactionRejectionReason.INVALID_VALUE, touched
        if any(abs(v) > MAXIMUM_DRIVE_MAGNITUDE for v in values):
            return (TransactionRejectionReason.INVALID_VALUE, "motor.force" if max(map(abs, drive.force)) >
                    MAXIMUM_DRIVE_MAGNITUDE else "motor.torque"), touched
        b = state.bubbles.get(oid)
        if b is None:
            return (_not_physical(state, oid) if oid not in state.bodies else
                    (TransactionRejectionReason.UNSUPPORTED_MOTION_ROLE, (oid, MotionRole.MOTOR_DRIVEN))), touched
        _set_bubble_motion(b, oid, MotionRole.MOTOR_DRIVEN)
        b.motor = drive
        return None, touched
    if kind in ("beginPlayerDrive", "updatePlayerDrive"):
        oid, target = args
        if not _finite(*target):
            return TransactionRejectionReason.INVALID_VALUE, touched
        b = state.bubbles.get(oid)
        if b is None:
            return _not_physical(state, oid) if oid not in state.bodies else \
                (TransactionRejectionReason.INCOMPATIBLE_OBJECT_KIND, oid), touched
        if kind == "beginPlayerDrive" and b.desc.drive_policy is None:
            return (TransactionRejectionReason.INCOMPATIBLE_OBJECT_KIND, oid), touched
        if b.desc.drive_policy is not None and any(abs(v) > MAXIMUM_DRIVE_MAGNITUDE for v in target):
            return (TransactionRejectionReason.INVALID_VALUE, "playerDrive.target"), touched
        if kind == "beginPlayerDrive":
            if b.drive_target is not None:
                return (TransactionRejectionReason.DRIVE_ALREADY_ACTIVE, oid), touched
            # a bubble added in the player-driven role goes back to dynamic (TransactionStager.swift:330)
            b.motion_before_drive = MotionRole.DYNAMIC if b.desc.motion_role == MotionRole.PLAYER_DRIVEN else \
                b.desc.motion_role
            b.desc = replace(b.desc, motion_role=MotionRole.PLAYER_DRIVEN)
            b.drive_id = state.next_drive_id
            state.next_drive_id += 1
        elif b.drive_target is None:
            return (TransactionRejectionReason.DRIVE_NOT_ACTIVE, oid), touched
        b.drive_target = tuple(float(v) for v in target)
        return None, touched
    if kind == "endPlayerDrive":
        oid = args[0]
        b = state.bubbles.get(oid)
        if b is None:
            return _not_physical(state, oid) if oid not in state.bodies else \
                (TransactionRejectionReason.DRIVE_NOT_ACTIVE, oid), touched
        if b.drive_target is None:
            return (TransactionRejectionReason.DRIVE_NOT_ACTIVE, oid), touched
        b.desc = replace(b.desc, motion_role=b.motion_before_drive or MotionRole.DYNAMIC)
        b.drive_target = b.drive_id = b.motion_before_drive = None
        return None, touched
    if kind == "setKinematicDrive":
        oid, drive = args
        body = state.bodies.get(oid)
        if body is None and oid not in state.bubbles:
            return TransactionRejectionReason.OBJECT_NOT_FOUND, touched
        if body is None or body.desc.motion_role != MotionRole.KINEMATIC:
            return (TransactionRejectionReason.INCOMPATIBLE_MOTION_ROLE, oid), touched
        names = {"velocity": (("kinematicDrive.linear", drive.linear), ("kinematicDrive.angular", (drive.angular,))),
                 "target": (("kinematicDrive.position", drive.target_position),
                            ("kinematicDrive.rotation", (drive.target_rotation,)))}.get(drive.kind, ())
        for name, values in names:  # TransactionStager.swift:293-302: finite and within 1e6
            if not _finite(*values) or any(abs(float(np.float32(v))) > MAXIMUM_DRIVE_MAGNITUDE for v in values):
                return (TransactionRejectionReason.INVALID_VALUE, name), touched
        if drive.kind == "velocity":
            body.desc = replace(body.desc, velocity=drive.linear, angular_velocity=drive.angular)
        body.drive, body.exact, body.path_index = drive, None, 0
        return None, touched
    return TransactionRejectionReason.UNSUPPORTED_OPERATION, touched


def stage(pending: list, state: _State, region) -> tuple[_State, list, list]:
    """TransactionStager.stageBatch for this path: each transaction applies atomically (all operations or none) in
    submission order against the state left by the previous ones. Returns (new state, receipts, events)."""
    receipts, events = [], []
    current = state
    for token, tx in pending:
        trial = current.copy()
        created, removed, replaced_ids, removed_joints = [], [], [], []
        rejection = None
        tx_events = []
        for index, op in enumerate(tx.operations):
            # the events of an operation follow the interests of the objects it touches, in operation order
            before = _interest_of(trial, op[1]) if op[0] in ("remove", "replace") else frozenset()
            reason, touched = _apply(op, trial, region)
            if reason is not None:
                detail = op[0]
                if isinstance(reason, tuple):  # a placement: (object id, PlacementIssue)
                    reason, detail = reason
                rejection = TransactionRejection(index, reason, detail)
                break
            created += touched["created"]
            removed += touched["removed"]
            removed_joints += touched["removed_joints"]
            replaced_ids += touched["replaced"]
            tx_events += [WorldEvent("didAdd", (i,)) for i in touched["created"]
                          if EventInterest.DID_ADD in _interest_of(trial, i)]
            tx_events += [WorldEvent("didRemove", (i,)) for i in touched["removed"] if EventInterest.DID_REMOVE in before]
            tx_events += [WorldEvent("didReplace", (i,)) for i in touched["replaced"]
                          if EventInterest.DID_REPLACE in before or EventInterest.DID_REPLACE in _interest_of(trial, i)]
        if rejection is None and tx.operations and any(b.desc.motion_role in DYNAMIC_ROLES for b in trial.bodies.values()):
            # judged on the state after the whole transaction, reported at its last operation
            # (NativeCompleteStepper.validate; a world of dynamic bodies alone steps through rigid.RigidSolver, which
            # this world API does not drive)
            reason = TransactionRejectionReason.UNSUPPORTED_BUBBLE_WITH_DYNAMIC_RIGID_BODY if trial.bubbles else \
                TransactionRejectionReason.UNSUPPORTED_OPERATION
            rejection = TransactionRejection(len(tx.operations) - 1, reason, "validate")
        if rejection is not None:
            events.append(WorldEvent("transactionRejected", token=token, rejection=rejection))
            continue
        current = trial
        receipts.append(TransactionReceipt(token, tuple(created), tuple(removed), tuple(replaced_ids),
                                           tuple(sorted(removed_joints))))
        events += tx_events
    return current, receipts, events


def _interest_of(state: _State, oid) -> frozenset:
    for table in (state.bubbles, state.bodies):
        if oid in table:
            return table[oid].desc.event_interest
    for table in (state.sensors, state.fields):
        if oid in table:
            return table[oid].event_interest
    return frozenset()


def _pair_key(a: int, b: int) -> tuple:
    ua, ub = a & 0xFFFFFFFFFFFFFFFF, b & 0xFFFFFFFFFFFFFFFF
    return (a, b) if ua <= ub else (b, a)


def contact_transitions(contacts: np.ndarray, segment_owner: dict, interested: set, history: set, step: float,
                        removed: set) -> tuple[list, set]:
    """contactBegan / contactEnded of one step from its contact records (NativePublicWorld.swift:340-391): per pair the
    point is the penetration-weighted mean, the normal the normalised sum (from the smaller id to the larger) and the
    impulse the summed F dt^2 divided by the step."""
    sums = {}
    for c in contacts:
        first = int(c["participants"][0])
        second = int(c["participants"][1]) if c["kind"] != 1 else segment_owner.get(int(c["participants"][1]))
        if second is None or not (c["penetration"] > 0 or c["impulse"] > 0):
            continue
        if first not in interested and second not in interested:
            continue
        key = _pair_key(first, second)
        normal = np.asarray(c["normal"], np.float64) * (-1.0 if c["kind"] == 1 else 1.0)
        if key[0] != first:
            normal = -normal
        weight = max(float(c["penetration"]), 0.0) + 1e-4
        s = sums.setdefault(key, [np.zeros(2), 0.0, np.zeros(2), 0.0])
        s[0] += np.asarray(c["point"], np.float64) * weight
        s[1] += weight
        s[2] += normal
        s[3] += float(c["impulse"]) / step
    order = lambda k: (k[0] & 0xFFFFFFFFFFFFFFFF, k[1] & 0xFFFFFFFFFFFFFFFF)
    events = []
    for key in sorted(sums, key=order):
        if key in history:
            continue
        point, weight, normal, impulse = sums[key]
        length = float(np.hypot(*normal))
        events.append(WorldEvent("contactBegan", key, tuple(point / weight), tuple(normal / length) if length > 0 else (0.0, 0.0),
                                 impulse))
    current = set(sums)
    for key in sorted(history, key=order):
        if key[0] in removed and key[1] in removed:
            continue  # nobody is left to tell (EventCompactorTests.swift:81-86)
        if key not in current or key[0] in removed or key[1] in removed:
            events.append(WorldEvent("contactEnded", key))
    return events, current - {k for k in current if k[0] in removed or k[1] in removed}


FIELD_KINDS = {"directional": 0, "radial": 1, "vortex": 2}


def field_records(state: _State):
    """The device records of a state's force fields (NativeForceInput.fields, NativeForceRecords.swift:160-230): in id
    order, the directional force or the radial / vortex strength, the range (a circle's radius or a polygon's
    farthest vertex), the polygon's local vertices, and the filter as a range of ascending ids (an empty filter takes
    nobody; no filter takes everyone)."""
    records, verts, ids = [], [], []
    for fid in sorted(state.fields, key=lambda v: v & 0xFFFFFFFFFFFFFFFF):
        d = state.fields[fid]
        f = N.ForceField()
        f.position[:] = [float(v) for v in d.position]
        f.rotation, f.falloff, f.kind = float(d.angle), float(d.falloff), FIELD_KINDS[d.kind]
        if d.kind == "directional":
            f.direction[:] = [float(v) for v in d.force]
        else:
            f.strength = float(d.strength)
        if isinstance(d.shape, Circle):
            f.radius, f.vertex_offset, f.vertex_count = float(d.shape.radius), 0, 0
        else:
            pts = np.asarray(d.shape.points, np.float32)
            f.radius = float(np.sqrt((pts.astype(np.float32) ** 2).sum(1)).max())
            f.vertex_offset, f.vertex_count = len(verts), len(pts)
            verts += [tuple(map(float, p)) for p in pts]
        taken = d.filter.object_ids if d.filter is not None else None
        f.has_filter = 0 if taken is None else 1
        f.filter_offset, f.filter_count = len(ids), 0 if taken is None else len(taken)
        if taken is not None:
            ids += sorted(int(v) for v in taken)
        records.append(f)
    return records, np.array(verts, np.float32).reshape(-1, 2), np.array(ids, np.int64)


def advance_transitions(state: _State, duration: float) -> bool:
    """Moves every transition by one step (MotionControllers.advanceTransitions): each value is sampled from the same
    start of step, interpolated in float from the value when the transition started, and the finished ones are dropped.
    Returns whether anything changed."""
    if not state.transitions:
        return False
    F32 = np.float32
    starts = {}
    for target in state.transitions:
        if target[0] == "globalForce":
            starts[target] = tuple(F32(v) for v in state.global_force)
        elif target[0] == "bubbleRadius":
            if target[1] in state.bubbles:
                starts[target] = F32(state.bubbles[target[1]].desc.radius)
        elif target[1] in state.materials:
            m = state.materials[target[1]]
            starts[target] = F32(m.contact_stiffness if target[2] == "contactStiffness" else m.damping)
    for target, tr in list(state.transitions.items()):
        if target not in starts:
            continue
        initial, elapsed = state.transition_progress.get(target, (starts[target], 0.0))
        elapsed += duration
        fraction = 1.0 if tr.duration == 0 else min(1.0, elapsed / tr.duration)
        t = transition_curve(tr.curve, fraction)
        one = F32(1)
        if target[0] == "globalForce":
            state.global_force = tuple(float(a * (one - t) + F32(b) * t) for a, b in zip(initial, tr.value))
        else:
            value = float(initial * (one - t) + F32(tr.value) * t)
            if target[0] == "bubbleRadius":
                b = state.bubbles[target[1]]
                b.desc = replace(b.desc, radius=value)
            else:
                m = state.materials[target[1]]
                state.materials[target[1]] = replace(m, **({"contact_stiffness": value} if target[2] == "contactStiffness"
                                                           else {"damping": value}))
        if fraction == 1.0:
            del state.transitions[target]
            state.transition_progress.pop(target, None)
        else:
            state.transition_progress[target] = (initial, elapsed)
    return True


def path_velocity(target, origin, speed: float, dt: float) -> np.ndarray:
    """The velocity that takes a bubble from `origin` towards `target` at `speed`, without passing it within the
    step (MotionControllers.swift:147-151), in float."""
    delta = (np.asarray(target, np.float32) - np.asarray(origin, np.float32)).astype(np.float32)
    distance = np.float32(math.sqrt(float(delta[0] * delta[0] + delta[1] * delta[1])))
    if not distance > 0:
        return np.zeros(2, np.float32)
    return (delta * (min(np.float32(speed), distance / np.float32(dt)) / distance)).astype(np.float32)


def prepare_kinematic(state: _State, duration: float) -> bool:
    """The start of a step for kinematic bodies (MotionControllers.swift:119-145): the velocity this step imposes,
    in float. A velocity drive tracks its pose in double and asks for the velocity that takes the float pose exactly
    there (a pose published otherwise, by a wrap or a replace, starts a new track); a path drive heads for its current
    point like a path-driven bubble but is never blocked; a target drive reaches its pose in one step; no drive stands
    still. Returns whether a body's velocity changed, which the device world must then be given."""
    dt = np.float32(duration)
    changed = False
    for body in state.bodies.values():
        if body.desc.motion_role != MotionRole.KINEMATIC:
            continue
        v, w = np.zeros(2, np.float32), np.float32(0.0)
        position, rotation = body.position.astype(np.float32), np.float32(body.angle)
        d = body.drive
        if d is not None and d.kind == "velocity":
            exact = body.exact
            if exact is None or np.float32(exact[0]) != position[0] or np.float32(exact[1]) != position[1] or \
                    np.float32(exact[2]) != rotation:
                exact = (float(position[0]), float(position[1]), float(rotation))
            linear = [float(np.float32(x)) for x in d.linear]
            exact = (exact[0] + linear[0] * duration, exact[1] + linear[1] * duration,
                     exact[2] + float(np.float32(d.angular)) * duration)
            body.exact = exact
            v = ((np.array(exact[:2], np.float64).astype(np.float32) - position) / dt).astype(np.float32)
            w = (np.float32(exact[2]) - rotation) / dt
        elif d is not None and d.kind == "path":
            points = np.asarray(d.path_drive.points, np.float32)
            body.path_index = min(body.path_index, len(points) - 1)
            while body.path_index < len(points) - 1 and \
                    float(np.linalg.norm((points[body.path_index] - position).astype(np.float32))) <= 1e-4:
                body.path_index += 1
            v = path_velocity(points[body.path_index], position, d.path_drive.speed, duration)
        elif d is not None and d.kind == "target":
            v = ((np.asarray(d.target_position, np.float32) - position) / dt).astype(np.float32)
            w = (np.float32(d.target_rotation) - rotation) / dt
        if not (np.array_equal(v, body.velocity) and np.float32(w) == np.float32(body.angular_velocity)):
            changed = True
        body.velocity, body.angular_velocity = v, float(w)
    return changed


def prepare_paths(state: _State, dt: float) -> list:
    """The start of a step for path-driven bubbles (MotionControllers.swift:85-91): the bubble heads for its path's
    current point, moving on to the next one once within 1e-4 of it; a bubble without a path, or stopped by a blocker,
    stands still. Returns the ids of the path-driven bubbles."""
    ids = []
    for oid, b in state.bubbles.items():
        if b.desc.motion_role != MotionRole.PATH_DRIVEN:
            continue
        ids.append(oid)
        if b.path is not None and not b.path_stopped:
            points = np.asarray(b.path.points, np.float32)
            while b.path_index < len(points) - 1 and \
                    float(np.linalg.norm((points[b.path_index] - b.position).astype(np.float32))) <= 1e-4:
                b.path_index += 1
            b.velocity = path_velocity(points[b.path_index], b.position, b.path.speed, dt)
        else:
            b.velocity = np.zeros(2, np.float32)
            b.angular_velocity = 0.0
    return ids


def _drop_transitions_of(state: _State, ids):
    for target in [t for t in state.transitions if t[0] == "bubbleRadius" and t[1] in ids]:
        del state.transitions[target]
        state.transition_progress.pop(target, None)


def body_contacts(state: _State, interested: set, step: float, separation_tolerance: float = 0.002) -> np.ndarray:
    """End-of-step contact records of bubbles against bodies (kind 2), for the pairs an event may concern. The device's
    records cover pairs and segments (nativeBuildContacts); the reference reports bubble-body contacts from its rigid
    solver, which is not built here, so they are taken on the host from the published poses: the signed distance d of
    the centre to the body's surface, active while r - d > -tolerance, the normal from the bubble to the body, the
    point on the surface and the impulse F dt^2 of the wall law F = K_c (r - d) r / d^2."""
    from .queries import distance_to_segment, polygon_contains
    out = []
    F32 = np.float32
    for bid, body in state.bodies.items():
        if isinstance(body.desc.shape, Polygon) and body.desc.motion_role == MotionRole.STATIC:
            continue  # static polygons are one-sided edges on the device: their records come from the step
        shape = _body_shape(body)
        for oid, b in state.bubbles.items():
            if (oid not in interested and bid not in interested) or not b.desc.filter.accepts(body.desc.filter):
                continue
            c, r = np.asarray(b.position, np.float32), F32(b.desc.radius)
            if shape[0] == "circle":
                delta = c - shape[1]
                dist = F32(math.hypot(*delta))
                surface_normal = delta / dist if dist > 0 else np.array([0, 1], np.float32)
                d = dist - shape[2]
                point = shape[1] + surface_normal * shape[2]
            elif shape[0] == "capsule":
                a, e = shape[1], shape[2]
                ab = e - a
                t = max(F32(0), min(F32(1), F32(np.dot(c - a, ab)) / max(F32(np.dot(ab, ab)), F32(1e-20))))
                nearest = a + ab * t
                delta = c - nearest
                dist = F32(math.hypot(*delta))
                surface_normal = delta / dist if dist > 0 else np.array([0, 1], np.float32)
                d = dist - shape[3]
                point = nearest + surface_normal * shape[3]
            else:
                ring = shape[1]
                best = None
                for k in range(len(ring)):
                    a, e = ring[k], ring[(k + 1) % len(ring)]
                    ab = e - a
                    t = max(F32(0), min(F32(1), F32(np.dot(c - a, ab)) / max(F32(np.dot(ab, ab)), F32(1e-20))))
                    q = a + ab * t
                    dist = F32(math.hypot(*(c - q)))
                    if best is None or dist < best[0]:
                        best = (dist, q)
                dist, point = best
                inside = polygon_contains(ring, c)
                d = -dist if inside else dist
                away = (c - point) / dist if dist > 0 else np.array([0, 1], np.float32)
                surface_normal = -away if inside else away
            if not (r - d > -separation_tolerance):
                continue
            law = float(wall_force(float(state.materials[b.desc.physics_material_id].contact_stiffness), float(r),
                                     float(d)))
            rec = np.zeros(1, N.CONTACT_DTYPE)[0]
            rec["participants"] = (oid, bid)
            rec["kind"] = 2
            rec["normal"] = -surface_normal  # from the bubble to the body
            rec["point"] = point
            rec["penetration"] = float(r - d)
            rec["impulse"] = law * step * step
            out.append(rec)
    return np.array(out, N.CONTACT_DTYPE) if out else np.zeros(0, N.CONTACT_DTYPE)


def wall_force(stiffness: float, radius: float, distance: float) -> float:
    """The wall law's force F = K_c (r - d) r / d^2 (nativeWallContactLaw, NFK:60-69), d clamped to r 1e-6."""
    d = max(distance, radius * 1e-6)
    return stiffness * (radius - d) * radius / (d * d) if d < radius else 0.0


def query_index(state: _State, effective_radii: dict | None = None) -> QueryIndex:
    """The spatial query index of a state (QueryIndex(state:)): bubbles as circles of their effective radius (the
    target radius when none is given), bodies with their exact world shapes; sensors take no part."""
    objects = []
    for oid, b in state.bubbles.items():
        r = (effective_radii or {}).get(oid, b.desc.radius)
        objects.append((oid, b.desc.filter, ("circle", np.asarray(b.position, np.float32), np.float32(max(r, 0.0)))))
    for oid, body in state.bodies.items():
        objects.append((oid, body.desc.filter, _body_shape(body)))
    return QueryIndex(objects)


class HitTestRequest:
    """A hit test answered on the state of the next completed step (BubbleWorld.hitTest of the reference, which
    suspends until then): `done` turns true with `result` (an object id or None); cancel() withdraws a waiting one."""

    def __init__(self, world, point):
        self._world = weakref.ref(world)
        self.point = (float(point[0]), float(point[1]))
        self.done = False
        self.result = None

    def _resolve(self, result):
        self.done, self.result = True, result

    def cancel(self):
        world = self._world()
        if not self.done and world is not None and self in world._hit_tests:
            world._hit_tests.remove(self)
        if not self.done:
            self._resolve(None)


# ---------------------------------------------------------------------------------------------------------------------
# Fixed-step clock
# ---------------------------------------------------------------------------------------------------------------------
class FixedStepDriver:
    """The world's time accumulator (FixedStepDriver.swift): time leaves the backlog only when a whole step completes;
    the backlog is capped at max(maximum_backlog, step) with the excess summed (saturating at the largest float); an
    invalid or overflowing increment leaves everything unchanged; after discard_next_advance() the next increment is
    dropped (time spent in the background is not game time)."""

    def __init__(self, fixed_time_step: float, maximum_steps_per_advance: int = 8, maximum_backlog: float = math.inf):
        if not (math.isfinite(fixed_time_step) and fixed_time_step > 0) or maximum_steps_per_advance <= 0 or \
                not maximum_backlog > 0:
            raise ValueError("fixed_time_step and maximum_backlog must be positive, maximum_steps_per_advance >= 1")
        self.fixed_time_step = float(fixed_time_step)
        self.maximum_steps_per_advance = int(maximum_steps_per_advance)
        self.maximum_backlog = max(float(maximum_backlog), self.fixed_time_step)
        self.backlog_seconds = 0.0
        self.simulation_time = 0.0
        self.completed_steps = 0
        self.consecutive_backlogged_advances = 0
        self.discarded_backlog_seconds = 0.0
        self._discard_next = False

    @property
    def can_step(self) -> bool:
        # a fraction of a step covers the rounding of many subtractions; none for a subnormal step
        step = self.fixed_time_step
        tolerance = 0.0 if step < sys.float_info.min else step * 1e-12
        return self.backlog_seconds >= step or (self.backlog_seconds > 0 and step - self.backlog_seconds <= tolerance)

    def accumulate(self, seconds: float) -> bool:
        if not (math.isfinite(seconds) and seconds >= 0):
            return False
        if self._discard_next:
            self._discard_next = False
            return True
        accumulated = self.backlog_seconds + seconds
        if not (math.isfinite(accumulated) and math.isfinite(self.simulation_time + accumulated)):
            return False
        if accumulated > self.maximum_backlog:
            total = self.discarded_backlog_seconds + (accumulated - self.maximum_backlog)
            self.discarded_backlog_seconds = total if math.isfinite(total) else sys.float_info.max
            self.backlog_seconds = self.maximum_backlog
        else:
            self.backlog_seconds = accumulated
        return True

    @property
    def interpolation_fraction(self) -> float:
        return min(max(self.backlog_seconds / self.fixed_time_step, 0.0), 1.0)

    @property
    def interpolation_fraction_after_next_step(self) -> float:
        return min(max((self.backlog_seconds - self.fixed_time_step) / self.fixed_time_step, 0.0), 1.0)

    def discard_next_advance(self):
        self._discard_next = True

    def complete_step(self):
        if not self.can_step:
            raise RuntimeError("no whole step in the backlog")
        self.backlog_seconds = max(0.0, self.backlog_seconds - self.fixed_time_step)
        self.simulation_time += self.fixed_time_step
        self.completed_steps += 1

    def finish_advance(self):
        self.consecutive_backlogged_advances = self.consecutive_backlogged_advances + 1 if self.can_step else 0


# ---------------------------------------------------------------------------------------------------------------------
# BubbleWorld
# ---------------------------------------------------------------------------------------------------------------------
class BubbleWorld:
    """Sole owner of a world and its transaction queue; publishes only completed steps."""

    def __init__(self, configuration: WorldConfiguration, context: Context | None = None, lifecycle=None):
        """`lifecycle` (optional, LifecycleEventSource of the reference) gets two callables, will_enter_background and
        did_become_active, that hold the world weakly; a host may also call enter_background() / become_active()."""
        self.configuration = configuration
        self._ctx = context
        self._state = _State(global_force=tuple(configuration.global_force),
                             fixed_time_step=configuration.fixed_time_step)
        self._pending: list = []
        self._next_token = 1
        self._clock = FixedStepDriver(configuration.fixed_time_step, configuration.maximum_steps_per_advance,
                                      configuration.maximum_backlog)
        self._manually_paused = False
        self._paused_in_background = False
        self._frame = WorldFrame()
        self._native: World | None = None
        self._native_ids: list = []
        self._native_order: list = []
        self._segment_owner: dict = {}
        self._history: set = set()
        self._events_dropped = 0  # step events beyond the event buffer in the current advance
        self._sensor_pairs: set = set()   # (sensor id, bubble id) pairs overlapping after the last step
        self._shapes: dict = {}           # bubble id -> (effective radius, bounds) of the last contours
        self._index: QueryIndex | None = None  # built at the first query after a publication
        self._feedback: tuple = ()
        self._hit_tests: list = []          # HitTestRequest waiting for the next step
        self._blockers: dict = {}          # driven bubble id -> the obstacle that blocked it in the last step
        self.query_index_build_count = 0
        self.diagnostics = WorldDiagnostics()
        if lifecycle is not None and configuration.automatic_pause:
            ref = weakref.ref(self)
            lifecycle.will_enter_background = lambda: (w := ref()) and w.enter_background()
            lifecycle.did_become_active = lambda: (w := ref()) and w.become_active()

    # -- public API ----------------------------------------------------------------------------------------------------
    def submit(self, transaction: WorldTransaction) -> int:
        token = self._next_token
        self._next_token += 1
        if self.diagnostics.failure_reason is None:
            self._pending.append((token, transaction))
        self.diagnostics.pending_transaction_count = len(self._pending)
        return token

    @property
    def _paused(self) -> bool:
        return self._manually_paused or self._paused_in_background

    def pause(self):
        self._manually_paused = True
        self.diagnostics.is_paused = self._paused

    def resume(self):
        self._manually_paused = False
        self.diagnostics.is_paused = self._paused

    def enter_background(self):
        """The host goes to the background: with automatic_pause the world pauses (BubbleWorld.swift:113-120)."""
        if self.configuration.automatic_pause:
            self._paused_in_background = True
            self.diagnostics.is_paused = True

    def become_active(self):
        """The host is active again: a background pause lifts and the next time increment is dropped (time spent in the
        background is not game time); a manual pause stays."""
        if self.configuration.automatic_pause and self._paused_in_background:
            self._paused_in_background = False
            self._clock.discard_next_advance()
            self.diagnostics.is_paused = self._paused

    @property
    def physics_materials(self) -> dict:
        """The published physics materials (transitions move their values step by step)."""
        return dict(self._state.materials)

    @property
    def global_force(self) -> tuple:
        return tuple(self._state.global_force)

    @property
    def last_frame(self) -> WorldFrame:
        return self._frame

    def advance(self, seconds: float) -> WorldFrame:
        """Runs the fixed-step clock: at most maximum_steps_per_advance steps; a call without a completed step (or
        after a failure) returns the last complete frame."""
        d, clock = self.diagnostics, self._clock
        d.steps_in_last_advance = 0
        d.last_advance_issue = None
        if d.failure_reason is not None:  # the final state wins over pause and step
            d.last_advance_issue = AdvanceIssue.WORLD_FAILED
            return self._frame
        if not (math.isfinite(seconds) and seconds >= 0):
            d.last_advance_issue = AdvanceIssue.INVALID_TIME_DELTA
            return self._frame
        if self._paused:
            return self._frame
        if not clock.accumulate(seconds):
            d.last_advance_issue = AdvanceIssue.TIME_ACCUMULATOR_OVERFLOW
            return self._frame
        receipts, events = [], []
        self._events_dropped = 0
        while d.steps_in_last_advance < clock.maximum_steps_per_advance and clock.can_step:
            if not self._step(receipts, events):
                d.last_advance_issue = AdvanceIssue.WORLD_FAILED if d.failure_reason is not None else \
                    AdvanceIssue.STEP_FAILED
                break
            d.last_rejection_reason = None
            clock.complete_step()
            d.steps_in_last_advance += 1
            self._frame = WorldFrame(clock.completed_steps, clock.simulation_time, tuple(receipts), tuple(events),
                                     self._objects(), self._feedback, WorldEventOverflow(self._events_dropped))
            self._index = None
        clock.finish_advance()
        d.backlog_seconds = clock.backlog_seconds
        d.discarded_backlog_seconds = clock.discarded_backlog_seconds
        d.consecutive_backlogged_advances = clock.consecutive_backlogged_advances
        d.pending_transaction_count = len(self._pending)
        return self._frame

    def request_hit_test(self, point) -> HitTestRequest:
        """The reference's asynchronous hitTest: the point goes with the next step and is answered on its state; a
        paused world keeps it waiting; a non-finite point or a failed world answers None at once."""
        request = HitTestRequest(self, point)
        if not all(math.isfinite(v) for v in request.point) or self.diagnostics.failure_reason is not None:
            request._resolve(None)
        else:
            self._hit_tests.append(request)
        return request

    def _host_hit(self, point):
        """Hit test of a world without bubbles (no device world): the bodies containing the point, the highest layer
        (Int32) then the largest id winning."""
        p = np.asarray(point, np.float32)
        best = None
        for oid, body in self._state.bodies.items():
            if _contains_including_boundary(_body_shape(body), p):
                key = (body.desc.layer, oid & 0xFFFFFFFFFFFFFFFF)
                if best is None or key > best[0]:
                    best = (key, oid)
        return None if best is None else best[1]

    @property
    def pending_hit_test_count(self) -> int:
        return len(self._hit_tests)

    def hit_test(self, point) -> int | None:
        """The object at `point` on the published state (BubbleWorld.hitTest): a bubble inside its contour, a body or a
        static polygon; the highest layer wins, then the largest id. None for empty space."""
        if self._native is None:
            return None
        cfg = self.configuration
        ids, _, found = self._native.hit_test([point], cfg.max_contour_segment_length, cfg.contour_surface_tension,
                                              cfg.position_tolerance)
        return int(ids[0]) if found[0] else None

    # -- queries on the published state (BubbleWorld.objects(at:), objects(in:), objects(inCircle:), raycast) -------
    def _query_index(self) -> QueryIndex:
        if self._index is None:
            self._index = query_index(self._state, {oid: shape[0] for oid, shape in self._shapes.items()})
            self.query_index_build_count += 1
        return self._index

    def objects_at(self, point, filter: CollisionFilter | None = None) -> list:
        """Bubbles (circles of their effective radius) and bodies containing `point`, ascending by id."""
        return self._query_index().objects_at(point, filter)

    def objects_in(self, rectangle, filter: CollisionFilter | None = None) -> list:
        """Objects intersecting the rectangle (min x, min y, max x, max y), ascending by id."""
        return self._query_index().objects_in_rect(rectangle[:2], rectangle[2:], filter)

    def objects_in_circle(self, center, radius: float, filter: CollisionFilter | None = None) -> list:
        return self._query_index().objects_in_circle(center, radius, filter)

    def raycast(self, start, end, filter: CollisionFilter | None = None) -> RaycastHit | None:
        return self._query_index().raycast(start, end, filter)

    def debug_contour_snapshot(self) -> dict:
        """Every bubble's published contour (BubbleWorld.debugContourSnapshot), read from the device."""
        if self._native is None:
            return {}
        cfg = self.configuration
        points, counts, _, _, _ = self._native.contours(cfg.max_contour_segment_length, cfg.contour_surface_tension,
                                                         cfg.position_tolerance)
        return {oid: [tuple(map(float, p)) for p in points[i, :counts[i]]] for i, oid in enumerate(self._native_order)
                if oid in self._state.bubbles}

    def close(self):
        if self._native is not None:
            self._native.close()
            self._native = None

    # -- internals -----------------------------------------------------------------------------------------------------
    def _spec(self, state: _State) -> tuple[WorldSpec, list, dict]:
        cfg = self.configuration.sanitized()
        ids = sorted(state.bubbles)
        b = np.zeros(len(ids), N.BUBBLE_DTYPE)
        bands, motors = [], []
        for i, oid in enumerate(ids):
            bub = state.bubbles[oid]
            d = bub.desc
            mat = state.materials[d.physics_material_id]
            static = d.motion_role == MotionRole.STATIC
            b[i]["id"] = oid
            b[i]["center"] = bub.position
            b[i]["previous_center"] = bub.position
            b[i]["velocity"] = bub.velocity
            b[i]["mass"] = d.mass
            b[i]["inverse_mass"] = 0.0 if static else np.float32(1.0) / np.float32(d.mass)
            b[i]["radius"] = d.radius
            b[i]["rotation"] = bub.rotation
            b[i]["angular_velocity"] = bub.angular_velocity
            b[i]["contact_stiffness"] = mat.contact_stiffness
            b[i]["damping"] = mat.damping
            # a path-driven bubble moves with the velocity its path set and feels contacts only: no forces, no damping
            force_driven = d.motion_role in (MotionRole.DYNAMIC, MotionRole.MOTOR_DRIVEN, MotionRole.PLAYER_DRIVEN)
            b[i]["flags"] = N.BUBBLE_ENABLED | (N.BUBBLE_STATIC if static else 0) | \
                (N.BUBBLE_FORCE_DRIVEN if force_driven else 0) | \
                (N.BUBBLE_WRAP if d.region_exit_policy == RegionExitPolicy.WRAP else 0)
            if d.motion_role == MotionRole.PLAYER_DRIVEN and bub.drive_target is not None:
                band = N.Band()
                band.bubble_id, band.stiffness = oid, d.drive_policy.band_stiffness
                band.maximum_force = d.drive_policy.maximum_force or 0.0  # 0: no limit
                band.target[:] = list(bub.drive_target)
                bands.append(band)
            if d.motion_role == MotionRole.MOTOR_DRIVEN and bub.motor is not None:
                motor = N.Motor()
                motor.bubble_id, motor.torque = oid, bub.motor.torque
                motor.force[:] = [float(v) for v in bub.motor.force]
                motor.inertia = float(np.float32(0.5) * np.float32(d.mass) * np.float32(d.radius) * np.float32(d.radius))
                motors.append(motor)
            b[i]["category"] = d.filter.category
            b[i]["mask"] = d.filter.mask
            b[i]["layer"] = d.layer
        segs, bodies, verts, tris = [], [], [], []
        owners = {}
        next_seg = 1
        for oid in sorted(state.bodies):
            body = state.bodies[oid]
            d, shape = body.desc, body.desc.shape
            if isinstance(shape, Polygon) and d.motion_role == MotionRole.STATIC:
                c, s = math.cos(body.angle), math.sin(body.angle)
                pts = np.asarray(shape.points, np.float64)
                world = np.stack([pts[:, 0] * c - pts[:, 1] * s, pts[:, 0] * s + pts[:, 1] * c], 1) + body.position
                e = static_polygon_edges(world.astype(np.float32), next_seg, oid)
                e["category"], e["mask"], e["layer"] = d.filter.category, d.filter.mask, d.layer
                for rec in e:
                    owners[int(rec["id"])] = oid
                next_seg += len(e)
                segs.append(e)
                continue
            rec = np.zeros(1, N.BODY_DTYPE)[0]
            rec["id"] = oid
            rec["position"] = body.position
            rec["angle"] = body.angle
            rec["velocity"] = body.velocity if d.motion_role == MotionRole.KINEMATIC else (0.0, 0.0)
            rec["angular_velocity"] = body.angular_velocity if d.motion_role == MotionRole.KINEMATIC else 0.0
            rec["flags"] = N.BODY_KINEMATIC if d.motion_role == MotionRole.KINEMATIC else N.BODY_STATIC
            rec["category"], rec["mask"], rec["layer"] = d.filter.category, d.filter.mask, d.layer
            rec["vertex_offset"] = sum(len(v) for v in verts)
            rec["triangle_offset"] = sum(len(t) for t in tris)
            if isinstance(shape, Circle):
                rec["kind"], rec["bounding_radius"], rec["core_radius"] = N.BODY_CIRCLE, shape.radius, shape.radius
                local, tri = np.zeros((1, 2), np.float32), np.zeros((0, 3), np.uint32)
            elif isinstance(shape, Capsule):
                rec["kind"], rec["core_radius"], rec["half_length"] = N.BODY_CAPSULE, shape.radius, shape.half_length
                rec["bounding_radius"] = shape.half_length + shape.radius
                local = np.array([[-shape.half_length, 0.0], [shape.half_length, 0.0]], np.float32)
                tri = np.zeros((0, 3), np.uint32)
            else:
                local, tri = polygon_triangles(shape.points)
                rec["kind"] = N.BODY_POLYGON
                rec["bounding_radius"] = float(np.sqrt((local.astype(np.float64) ** 2).sum(1)).max())
            rec["vertex_count"], rec["triangle_count"] = len(local), len(tri)
            verts.append(local)
            tris.append(tri)
            bodies.append(rec)
        spec = WorldSpec(bubbles=b,
                         segments=np.concatenate(segs) if segs else np.zeros(0, N.SEGMENT_DTYPE),
                         bodies=np.array(bodies, N.BODY_DTYPE) if bodies else np.zeros(0, N.BODY_DTYPE),
                         body_vertices=np.concatenate(verts) if verts else np.zeros((0, 2), np.float32),
                         body_triangles=np.concatenate(tris) if tris else np.zeros((0, 3), np.uint32),
                         region=tuple(cfg.simulation_region), global_force=tuple(state.global_force),
                         gravity=tuple(cfg.gravity), time_step=cfg.fixed_time_step,
                         candidate_limit=cfg.candidate_limit, substep_split_multiplier=cfg.substep_split_multiplier,
                         bands=bands, motors=motors)
        spec.fields, spec.field_vertices, spec.field_object_ids = field_records(state)
        return spec, ids, owners

    def _step(self, receipts: list, events: list) -> bool:
        cfg = self.configuration
        taken = len(self._pending)
        handed = list(self._hit_tests)  # the points this step answers; later requests wait for the next one
        staged, rec, ev = stage(self._pending[:taken], self._state, cfg.simulation_region)
        staged_events = len(ev)  # the stager's events; what the step adds below shares the event buffer
        _drop_transitions_of(staged, {i for r in rec for i in r.removed_object_ids})
        if staged.transitions and staged is self._state:
            staged = staged.copy()
        if staged is self._state and (any(b.desc.motion_role == MotionRole.PATH_DRIVEN for b in staged.bubbles.values())
                                      or any(b.drive is not None for b in staged.bodies.values())):
            staged = staged.copy()
        moved = advance_transitions(staged, cfg.fixed_time_step)
        paths = prepare_paths(staged, cfg.fixed_time_step)  # a path's velocity goes to the device every step
        steered = prepare_kinematic(staged, cfg.fixed_time_step)
        starts = {oid: staged.bubbles[oid].position.copy() for oid in paths}
        changed = bool(rec) or self._native is None or moved or bool(paths) or steered
        spec, ids, owners = self._spec(staged)
        # pairs whose sensor or bubble left in this batch end (the reference's missing-pair events)
        gone_now = {i for r in rec for i in r.removed_object_ids + r.replaced_object_ids}
        for pair in sorted(self._sensor_pairs):
            if pair[0] in gone_now or pair[1] in gone_now:
                sensor = self._state.sensors.get(pair[0])
                if sensor is not None and sensor.reports_exit:
                    ev.append(WorldEvent("exitedSensor", pair))
                self._sensor_pairs.discard(pair)
        if changed or ids != self._native_ids:
            if self._native is not None:
                self._native.close()
                self._native = None
            if len(ids) and self._ctx is None:
                self._ctx = default_context()
            try:
                self._native = World(spec, self._ctx) if len(ids) else None
            except N.NativeError as error:
                return self._solver_error(error)
            self._native_ids = ids
            self._native_order = ids  # the device world's bubble order (kept when a removal forces a rebuild)
            self._segment_owner = owners
            if self._native is not None and staged.sensors:
                records, verts, carried, allowed = self._sensor_records(staged, ids + [int(v) for v in spec.bodies["id"]])
                self._native.set_sensors(records, verts, carried, allowed)
        removed_now = set()
        contacts = np.zeros(0, N.CONTACT_DTYPE)
        if self._native is not None:
            try:
                status, reps = self._native.step(1)
            except N.NativeError as error:
                return self._solver_error(error)
            rep = reps[0]
            if status != N.OK:
                self._fail(status, rep)
                return False
            out = self._native.bubbles()
            contacts = self._native.contacts()
            for i, oid in enumerate(ids):
                bub = staged.bubbles[oid]
                bub.position = out[i]["center"].astype(np.float32).copy()
                bub.velocity = out[i]["velocity"].astype(np.float32).copy()
                bub.rotation = float(out[i]["rotation"])
                bub.angular_velocity = float(out[i]["angular_velocity"])
                interest = bub.desc.event_interest
                if out[i]["region_result"] == 1:
                    removed_now.add(oid)
                    if EventInterest.DID_EXIT_SIMULATION_REGION in interest:
                        ev.append(WorldEvent("didExitSimulationRegion", (oid,)))
                elif out[i]["region_result"] == 2 and EventInterest.DID_WRAP in interest:
                    ev.append(WorldEvent("didWrap", (oid,)))
            for oid in removed_now:
                staged.bubbles.pop(oid)
            _drop_transitions_of(staged, removed_now)
            self.diagnostics.last_step_substeps = int(rep["substep_count"])
            self.diagnostics.last_step_rebuilds = int(rep["rebuild_count"])
            self.diagnostics.contact_candidate_overflow += int(rep["candidate_overflow"])
            self.diagnostics.maximum_contact_candidates_per_object = int(rep["max_candidates_per_object"])
            if staged.sensors:
                for e in self._native.sensor_events():
                    pair, sensor = (int(e["sensor"]), int(e["object"])), staged.sensors[int(e["sensor"])]
                    point = tuple(map(float, e["point"]))  # the bubble's centre or the body's position
                    if e["kind"] == 1:  # 1 enter, 2 exit
                        self._sensor_pairs.add(pair)
                        if sensor.reports_enter:
                            ev.append(WorldEvent("enteredSensor", pair, point))
                    else:
                        self._sensor_pairs.discard(pair)
                        if sensor.reports_exit:
                            ev.append(WorldEvent("exitedSensor", pair, point))
            if cfg.contours:
                _, _, _, shape, _ = self._native.contours(cfg.max_contour_segment_length, cfg.contour_surface_tension,
                                                          cfg.position_tolerance)
                self._shapes = {oid: (float(shape[i][1]), tuple(map(float, shape[i][2:6]))) for i, oid in enumerate(ids)}
        dt = np.float32(cfg.fixed_time_step)
        for body in staged.bodies.values():  # kinematic advance (with or without bubbles), the device's float arithmetic
            if body.desc.motion_role == MotionRole.KINEMATIC:
                body.position = (body.position + body.velocity * dt).astype(np.float32)
                body.angle = float(np.float32(body.angle) + np.float32(body.angular_velocity) * dt)
        interested = {i for i, b in staged.bubbles.items() if EventInterest.CONTACT in b.desc.event_interest}
        interested |= {i for i, b in staged.bodies.items() if EventInterest.CONTACT in b.desc.event_interest}
        gone = removed_now | {i for r in rec for i in r.removed_object_ids + r.replaced_object_ids}
        if interested and staged.bodies and staged.bubbles:
            contacts = np.concatenate([contacts, body_contacts(staged, interested, cfg.fixed_time_step)])
        contact_events, self._history = contact_transitions(contacts, self._segment_owner, interested, self._history,
                                                            cfg.fixed_time_step, gone)
        self._feedback = self._drive_feedback(staged, contacts, starts)
        blockers = {}
        for fb in self._feedback:  # driveBlocked when the blocker of an interested bubble changes (EventCompactor.finish)
            bub = staged.bubbles.get(fb.object_id)
            if fb.blocking_contact is None or bub is None or EventInterest.DRIVE_BLOCKED not in bub.desc.event_interest:
                continue
            blockers[fb.object_id] = fb.blocking_contact.object_id
            if self._blockers.get(fb.object_id) != fb.blocking_contact.object_id:
                ev.append(WorldEvent("driveBlocked", (fb.object_id, fb.blocking_contact.object_id),
                                     fb.blocking_contact.point))
        self._blockers = blockers
        self._state = staged
        del self._pending[:taken]
        receipts += rec
        # the step's events fill the event buffer in order; the rest are counted as dropped (EventCompactor.finish):
        # a dropped contactEnded keeps its pair for the next step, a dropped contactBegan leaves it out of the history
        # so the pair begins again while it lasts
        step_events = ev[staged_events:] + contact_events
        kept, dropped = step_events[:cfg.event_buffer_capacity], step_events[cfg.event_buffer_capacity:]
        for e in dropped:
            if e.kind == "contactBegan":
                self._history.discard(e.objects)
            elif e.kind == "contactEnded" and not (e.objects[0] in gone and e.objects[1] in gone):
                self._history.add(e.objects)
        self._events_dropped += len(dropped)
        events += ev[:staged_events] + kept
        if handed:
            answers = [self._host_hit(r.point) for r in handed]  # no device world: bodies only, exact shapes
            if self._native is not None:
                ids, _, found = self._native.hit_test([r.point for r in handed], cfg.max_contour_segment_length,
                                                      cfg.contour_surface_tension, cfg.position_tolerance)
                answers = [int(i) if f else None for i, f in zip(ids, found)]
            for request, answer in zip(handed, answers):
                if request in self._hit_tests:
                    self._hit_tests.remove(request)
                    request._resolve(answer)
        if removed_now and self._native is not None:
            self._native_ids = None  # the removed slots leave the device world at the next step
        return True

    def _drive_feedback(self, state: _State, contacts, starts: dict) -> tuple:
        """DriveFeedback of every active player or path drive after a step (MotionControllers.swift:154-188): the
        target, the bubble's position, and its first contact whose normal (from the obstacle to the bubble) stands
        against the drive. A path-driven bubble so blocked that it moved less than 1e-4 in the step (`starts` holds
        where it began) stops for good, and keeps reporting that blocker."""
        out = []
        for oid in sorted(state.bubbles, key=lambda v: v & 0xFFFFFFFFFFFFFFFF):
            b = state.bubbles[oid]
            role = b.desc.motion_role
            if role == MotionRole.PLAYER_DRIVEN and b.drive_target is not None:
                target = b.drive_target
            elif role == MotionRole.PATH_DRIVEN and b.path is not None:
                target = b.path.points[b.path_index]
            else:
                continue
            delta = np.asarray(target, np.float32) - b.position
            blocker = None
            for c in contacts:
                a, other, kind = int(c["participants"][0]), int(c["participants"][1]), int(c["kind"])
                if a == oid:
                    # pair normals run from the first participant to the second, segment normals from the wall out
                    normal = -c["normal"] if kind == 0 else c["normal"]
                    obstacle = other if kind == 0 else self._segment_owner.get(other, other)
                elif kind == 0 and other == oid:
                    normal, obstacle = c["normal"], a
                else:
                    continue
                if float(delta[0] * normal[0] + delta[1] * normal[1]) < -1e-4:
                    blocker = DriveBlockingContact(obstacle, tuple(map(float, c["point"])), tuple(map(float, normal)))
                    break
            path_active = role == MotionRole.PATH_DRIVEN
            if path_active and blocker is not None and oid in starts and \
                    float(np.linalg.norm((b.position - starts[oid]).astype(np.float32))) < 1e-4:
                b.path_stopped, b.path_blocker = True, blocker
                b.velocity[:] = 0
                b.angular_velocity = 0.0
            out.append(DriveFeedback(oid, b.drive_id, tuple(target), tuple(map(float, b.position)),
                                     blocker or (b.path_blocker if path_active else None),
                                     path_active and b.path_stopped))
        return tuple(out)

    def _sensor_records(self, state: _State, objects: list):
        """Device records of the sensors (id order), their polygon vertices, and per (sensor, object) pair the overlap
        state carried over and whether the sensor's filter takes the object; `objects` are the device world's bubbles,
        then its bodies."""
        records, verts = [], []
        sensor_ids = sorted(state.sensors)
        for sid in sensor_ids:
            d = state.sensors[sid]
            r = N.Sensor()
            r.id, r.position[:], r.angle = sid, [float(v) for v in d.position], float(d.angle)
            if isinstance(d.shape, Circle):
                r.radius, r.vertex_offset, r.vertex_count = float(d.shape.radius), 0, 0
            else:
                r.radius, r.vertex_offset, r.vertex_count = 0.0, len(verts), len(d.shape.points)
                verts += [tuple(map(float, p)) for p in d.shape.points]
            r.flags = N.SENSOR_ENTER_EVENTS | N.SENSOR_EXIT_EVENTS  # every flip comes back; the host keeps the pair set
            records.append(r)
        index = {oid: i for i, oid in enumerate(objects)}
        row = {sid: k for k, sid in enumerate(sensor_ids)}
        carried = np.zeros(len(sensor_ids) * len(objects), np.uint8)
        for sid, b in self._sensor_pairs:
            if sid in row and b in index:
                carried[row[sid] * len(objects) + index[b]] = 1
        allowed = np.array([state.sensors[sid].filter.takes(oid) for sid in sensor_ids for oid in objects], np.uint8)
        return records, np.array(verts, np.float32).reshape(-1, 2), carried, allowed

    def _solver_error(self, error) -> bool:
        """A solver call that did not step: a failed CUDA command or device wait ends the world (the command failed);
        a bad snapshot, a step in flight, a capacity or allocation limit only rejects this step, and the same
        transactions and time retry at the next advance (BubbleWorld.handleAdvanceError). No device at all is
        raised: the product never steps without its CUDA path."""
        if error.status == N.E_UNAVAILABLE:
            raise error
        if error.status in (N.E_CUDA, N.E_TIMEOUT):
            self._fail(error.status, None)
            return False
        self.diagnostics.last_rejection_reason = {N.E_INVALID: WorldRejectionReason.INVALID_SNAPSHOT,
                                                  N.E_INFLIGHT: WorldRejectionReason.FRAME_IN_FLIGHT}.get(
            error.status, WorldRejectionReason.UNEXPECTED)
        self._native_ids = None  # rebuild the device world from the published state at the retry
        return False

    def _fail(self, status: int, rep):
        reasons = {N.E_SUBSTEP_LIMIT: WorldFailureReason.SUBSTEP_LIMIT_EXCEEDED,
                   N.E_NONFINITE: WorldFailureReason.NON_FINITE_VALUES,
                   N.E_CONTACT_VIOLATION: WorldFailureReason.CONTACT_VIOLATION}
        self.diagnostics.failure_reason = reasons.get(status, WorldFailureReason.COMMAND_EXECUTION_FAILED)
        for request in self._hit_tests:
            request._resolve(None)
        self._hit_tests.clear()
        self.diagnostics.failure_detail = None if rep is None else {
            "objects": tuple(int(v) for v in rep["violation_objects"]), "edge": int(rep["violation_edge"]),
            "distance": float(rep["violation_distance"]), "limiting_term": int(rep["limiter_term"]),
            "limiting_object": int(rep["limiter_object"])}
        self._pending.clear()

    def _objects(self) -> dict:
        out = {}
        for oid, b in self._state.bubbles.items():
            r = b.desc.radius
            effective, bounds = self._shapes.get(oid, (r, (float(b.position[0]) - r, float(b.position[1]) - r,
                                                           float(b.position[0]) + r, float(b.position[1]) + r)))
            out[oid] = ObjectState("bubble", tuple(map(float, b.position)), tuple(map(float, b.velocity)), b.rotation,
                                   b.angular_velocity, bounds, effective)
        for oid, body in self._state.bodies.items():
            shape = body.desc.shape
            kind = {Circle: "circle", Capsule: "capsule", Polygon: "polygon"}[type(shape)]
            lo, hi = shape_box(_body_shape(body))  # the box of the shape at its pose: it follows the rotation
            kinematic = body.desc.motion_role == MotionRole.KINEMATIC
            vel = body.velocity if kinematic else (0.0, 0.0)
            out[oid] = ObjectState(kind, tuple(map(float, body.position)), tuple(map(float, vel)), body.angle,
                                   body.angular_velocity if kinematic else 0.0,
                                   (float(lo[0]), float(lo[1]), float(hi[0]), float(hi[1])))
        return out
