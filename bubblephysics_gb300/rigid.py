"""Host side of the rigid body solver: joint records built like the reference's NativeJointState.prepare
(Sources/BubblePhysicsNativeMetal/NativeJointState.swift:61-141), and `RigidSolver`, which holds one world's rigid
arrays in device memory and runs the library's rigid passes on them (bp_rigid_predict, bp_rigid_body_candidates,
bp_rigid_ccd, bp_rigid_solve_contacts, bp_rigid_solve_joints, bp_rigid_guard_walls, bp_rigid_finish).

`RigidSolver.step` is the reference's rigid step (NativeMetalSolver.swift:767-799, 919): predict, body-pair rows,
CCD, 8 rounds of {body contacts + apply, joints + apply, wall guard}, and the finish (which the reference runs after
the bubble step).

Device memory comes from torch (plumbing only); every computation runs in the library's CUDA kernels.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from bubblephysics_gb300 import _native as N

ITERATIONS = 8  # NativeMetalSolver.rigidSolverIterationCount (NativeMetalSolver.swift:334)


@dataclass
class Joint:
    """A joint of the public model (Joint, with its kind): `body_b` None joins `body_a` to a world point."""
    id: int
    body_a: int
    body_b: Optional[int]
    kind: str                                   # "distance", "hinge" or "weld"
    anchor_a: tuple = (0.0, 0.0)
    anchor_b: tuple = (0.0, 0.0)
    length: float = 0.0                         # distance
    softness: float = 0.0                       # distance: compliance
    damping: float = 0.0                        # distance
    reference_angle: float = 0.0                # hinge, weld
    limits: Optional[tuple] = None              # hinge: (lower, upper)
    motor: Optional[tuple] = None               # hinge: (target angular velocity, maximum torque)
    collide_connected: bool = False


@dataclass
class JointArrays:
    records: np.ndarray      # RIGID_JOINT_DTYPE
    references: np.ndarray   # (R, 2) uint32: joint index, side
    ranges: np.ndarray       # (entities, 4) uint32: reference start / count, partner start / count
    partners: np.ndarray     # uint64 object ids


def prepare_joints(joints: Sequence[Joint], bubble_ids: Sequence[int], body_ids: Sequence[int]) -> JointArrays:
    """Joint records, per-entity reference lists and no-collision partner lists (NativeJointState.prepare).

    Records are sorted by joint id. An end that is a bubble keeps only the no-collision exclusion (the v4 engine has
    no joints with bubbles); a joint with the world puts the world at end 0 and the body at end 1. With no record at
    all the ranges are zero and no partner list is kept, like the reference's empty buffers."""
    nb = len(bubble_ids)
    entity = {int(i): k for k, i in enumerate(bubble_ids)}
    entity.update({int(i): nb + k for k, i in enumerate(body_ids)})
    count = nb + len(body_ids)
    rows, lists = [], [[] for _ in range(count)]
    partners = [[] for _ in range(count)]
    for joint in sorted(joints, key=lambda j: j.id):
        first = entity.get(int(joint.body_a))
        if first is None:
            continue
        second = N.JOINT_WORLD_END if joint.body_b is None else entity.get(int(joint.body_b), N.JOINT_WORLD_END)
        if joint.body_b is not None and second == N.JOINT_WORLD_END:
            continue
        if first < nb or (second != N.JOINT_WORLD_END and second < nb):
            if not joint.collide_connected and joint.body_b is not None:
                partners[first].append(int(joint.body_b))
                partners[second].append(int(joint.body_a))
            continue
        ends = (first, second)
        anchors = (tuple(joint.anchor_a), tuple(joint.anchor_b))
        if joint.body_b is None:
            ends, anchors = (N.JOINT_WORLD_END, first), (tuple(joint.anchor_b), tuple(joint.anchor_a))
        kind, flags = 0, 0
        parameters, limits = [0.0] * 4, [0.0] * 4
        if joint.kind == "distance":
            parameters = [joint.length, joint.softness, joint.damping, 0.0]
        elif joint.kind == "hinge":
            kind, parameters[3] = 1, joint.reference_angle
            if joint.limits is not None:
                flags |= 1
                limits[0], limits[1] = joint.limits
            if joint.motor is not None:
                flags |= 2
                limits[2], limits[3] = joint.motor
        elif joint.kind == "weld":
            kind, parameters[3] = 2, joint.reference_angle
        else:
            raise ValueError(f"unknown joint kind {joint.kind!r}")
        index = len(rows)
        rows.append((joint.id, ends, kind, flags, anchors, parameters, limits))
        if ends[0] != N.JOINT_WORLD_END:
            lists[ends[0]].append((index, 0))
        lists[ends[1]].append((index, 1))
        if not joint.collide_connected and joint.body_b is not None:
            partners[first].append(int(joint.body_b))
            partners[ends[1]].append(int(joint.body_a))
    records = np.zeros(len(rows), N.RIGID_JOINT_DTYPE)
    for k, (jid, ends, kind, flags, anchors, parameters, limits) in enumerate(rows):
        records[k]["id"] = jid
        records[k]["ends"] = (ends[0], ends[1], kind, flags)
        records[k]["anchors"] = (*anchors[0], *anchors[1])
        records[k]["parameters"] = parameters
        records[k]["limits"] = limits
    ranges = np.zeros((count, 4), np.uint32)
    if not rows:
        return JointArrays(records, np.zeros((0, 2), np.uint32), ranges, np.zeros(0, np.uint64))
    references, partner_ids = [], []
    for e in range(count):
        sorted_partners = sorted(set(partners[e]))
        ranges[e] = (len(references), len(lists[e]), len(partner_ids), len(sorted_partners))
        references.extend(lists[e])
        partner_ids.extend(sorted_partners)
    return JointArrays(records, np.array(references, np.uint32).reshape(-1, 2), ranges,
                       np.array(partner_ids, np.uint64))


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise N.NativeError(N.E_UNAVAILABLE, "rigid solver: no CUDA device")
    return torch


class RigidSolver:
    """Rigid bodies, their vertices, the static segments and the joints of one world, resident on the device.

    `bodies` are RIGID_BODY_DTYPE records (vertices local to the geometry origin, offsets into `vertices`),
    `segments` SEGMENT_DTYPE records (static within the step). `bubble_count` offsets the body entities of the joint
    arrays. The walls array (one record per body) is cleared before each predict."""

    def __init__(self, bodies: np.ndarray, vertices: np.ndarray, segments: Optional[np.ndarray] = None,
                 joints: Optional[JointArrays] = None, bubble_count: int = 0, stream=None,
                 triangles: Optional[np.ndarray] = None, row_width: int = 16):
        torch = self.torch = _torch()
        self.lib = N.library()
        self.stream = stream
        self.body_count = len(bodies)
        self.vertex_count = int(np.asarray(vertices).reshape(-1, 2).shape[0])
        self.segment_count = 0 if segments is None else len(segments)
        self.bubble_count = bubble_count
        self.joint_count = 0 if joints is None else len(joints.records)

        def dev(array, dtype=None):
            raw = np.ascontiguousarray(array if dtype is None else np.asarray(array, dtype)).view(np.uint8).reshape(-1)
            t = torch.empty(max(raw.size, 16), dtype=torch.uint8, device="cuda")
            if raw.size:
                t[:raw.size].copy_(torch.from_numpy(raw.copy()))
            return t

        self.d_bodies = dev(np.asarray(bodies, N.RIGID_BODY_DTYPE))
        self.d_vertices = dev(np.asarray(vertices, np.float32).reshape(-1, 2))
        self.d_segments = dev(np.zeros(0, N.SEGMENT_DTYPE) if segments is None else np.asarray(segments, N.SEGMENT_DTYPE))
        self.d_walls = torch.zeros(max(self.body_count, 1) * N.RIGID_WALL_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        tris = np.zeros((0, 4), np.uint32) if triangles is None else np.asarray(triangles, np.uint32).reshape(-1, 4)
        self.triangle_count = int(tris.shape[0])
        self.d_triangles = dev(tris)
        self.row_width = row_width
        slots = max(self.body_count, 1) * row_width
        self.d_rows = torch.zeros(slots * N.RIGID_CANDIDATE_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        self.d_row_counts = torch.zeros(max(self.body_count, 1) * 2, dtype=torch.int32, device="cuda")
        self.d_contact_corrections = torch.zeros(slots * N.RIGID_CORRECTION_DTYPE.itemsize, dtype=torch.uint8,
                                                 device="cuda")
        self.d_overflow = torch.zeros(4, dtype=torch.int32, device="cuda")
        self.d_safety = torch.zeros(4, dtype=torch.int32, device="cuda")
        if joints is not None and self.joint_count:
            self.d_joints = dev(joints.records)
            self.d_references = dev(joints.references, np.uint32)
            self.d_ranges = dev(joints.ranges, np.uint32)
            self.d_partners = dev(joints.partners, np.uint64)
            self.reference_count = int(joints.references.shape[0])
            self.partner_count = int(joints.partners.size)
            self.d_corrections = torch.zeros(self.joint_count * N.RIGID_CORRECTION_DTYPE.itemsize, dtype=torch.uint8,
                                             device="cuda")
        else:
            self.d_joints = self.d_references = self.d_ranges = self.d_partners = self.d_corrections = None
            self.reference_count = self.partner_count = 0

    @staticmethod
    def _p(t):
        return None if t is None else C.c_void_p(t.data_ptr())

    def _stream(self):
        return None if self.stream is None else C.c_void_p(self.stream.cuda_stream)

    def predict(self, dt: float) -> None:
        """nativeRigidPredict (NativePostSolveKernels:66-115)."""
        self.d_walls.zero_()
        N.check(self.lib.bp_rigid_predict(self._p(self.d_bodies), self.body_count, self._p(self.d_vertices),
                                          self.vertex_count, self._p(self.d_segments) if self.segment_count else None,
                                          self.segment_count, self.bubble_count, dt, self._p(self.d_ranges),
                                          self._p(self.d_partners), self.partner_count, self._p(self.d_walls),
                                          self._p(self.d_safety), self._stream()), "bp_rigid_predict")

    def solve_joints(self, dt: float, rounds: int = ITERATIONS, iteration_count: int = ITERATIONS) -> None:
        """`rounds` rounds of nativeSolveJoints + nativeApplyJointBodies (NativeContactKernels:446-562)."""
        if not self.joint_count:
            return
        N.check(self.lib.bp_rigid_solve_joints(self._p(self.d_bodies), self.body_count, self._p(self.d_joints),
                                               self.joint_count, self._p(self.d_corrections),
                                               self._p(self.d_references), self.reference_count,
                                               self._p(self.d_ranges), self.bubble_count, dt, iteration_count, rounds,
                                               self._p(self.d_safety), self._stream()), "bp_rigid_solve_joints")

    def finish(self, region: Sequence[float]) -> None:
        """nativeRigidFinish (NativePostSolveKernels:172-198); region = (min x, min y, max x, max y)."""
        r = (C.c_float * 4)(*[float(v) for v in region])
        N.check(self.lib.bp_rigid_finish(self._p(self.d_bodies), self.body_count, self._p(self.d_vertices),
                                         self.vertex_count, r, self._p(self.d_safety), self._stream()),
                "bp_rigid_finish")

    def _geometry(self):
        return (self._p(self.d_vertices), self.vertex_count,
                self._p(self.d_triangles) if self.triangle_count else None, self.triangle_count)

    def body_candidates(self) -> None:
        """Body-pair rows (nativeRigidEmitCandidates, body pairs: NativeGeometryKernels:394-415)."""
        N.check(self.lib.bp_rigid_body_candidates(self._p(self.d_bodies), self.body_count, self.bubble_count,
                                                  self._p(self.d_ranges), self._p(self.d_partners),
                                                  self.partner_count, self.row_width, self._p(self.d_rows),
                                                  self._p(self.d_row_counts), self._p(self.d_overflow),
                                                  self._stream()), "bp_rigid_body_candidates")

    def ccd(self) -> None:
        """Body-body CCD (nativeRigidResolveCCD + nativeRigidApplyCCD, NativePostSolveKernels:200-263)."""
        N.check(self.lib.bp_rigid_ccd(self._p(self.d_bodies), self.body_count, *self._geometry(), self._p(self.d_rows),
                                      self._p(self.d_row_counts), self.row_width, self._p(self.d_safety),
                                      self._stream()), "bp_rigid_ccd")

    def solve_contacts(self) -> None:
        """One contact round (nativeRigidContacts + nativeRigidApplyBodies, NativeContactKernels:375-444)."""
        N.check(self.lib.bp_rigid_solve_contacts(self._p(self.d_bodies), self.body_count, *self._geometry(),
                                                 self._p(self.d_rows), self._p(self.d_row_counts), self.row_width,
                                                 self._p(self.d_contact_corrections), self._p(self.d_safety),
                                                 self._stream()), "bp_rigid_solve_contacts")

    def guard_walls(self) -> None:
        """The wall guard (nativeRigidGuardWalls, NativePostSolveKernels:118-170)."""
        N.check(self.lib.bp_rigid_guard_walls(self._p(self.d_bodies), self.body_count, *self._geometry(),
                                              self.bubble_count, self._p(self.d_ranges), self._p(self.d_partners),
                                              self.partner_count, self._p(self.d_safety), self._stream()),
                "bp_rigid_guard_walls")

    def step(self, dt: float, region: Sequence[float], iterations: int = ITERATIONS) -> None:
        """One rigid step in the reference's order (NativeMetalSolver.swift:767-799, 919): predict, body-pair rows,
        CCD, `iterations` rounds of {contacts, one joint round, wall guard}, finish."""
        self.predict(dt)
        self.body_candidates()
        self.ccd()
        for _ in range(iterations):
            self.solve_contacts()
            self.solve_joints(dt, 1, iterations)
            self.guard_walls()
        self.finish(region)

    def step_without_contacts(self, dt: float, region: Sequence[float], iterations: int = ITERATIONS) -> None:
        """The same step for a world whose bodies meet no other body and no static polygon (jointed mechanisms):
        predict, all joint rounds in one call, finish - the same results in 3 to 2 + 2 x iterations launches."""
        self.predict(dt)
        self.solve_joints(dt, iterations, iterations)
        self.finish(region)

    def candidates(self):
        self.torch.cuda.synchronize()
        rows = self.d_rows[:self.body_count * self.row_width * 32].cpu().numpy().view(N.RIGID_CANDIDATE_DTYPE)
        counts = self.d_row_counts[:self.body_count * 2].cpu().numpy().view(np.uint32).reshape(-1, 2)
        return rows.reshape(-1, self.row_width).copy(), counts.copy()

    def overflow(self):
        self.torch.cuda.synchronize()
        return self.d_overflow[:2].cpu().numpy().view(np.uint32).copy()

    def bodies(self) -> np.ndarray:
        self.torch.cuda.synchronize()
        return self.d_bodies[:self.body_count * 160].cpu().numpy().view(N.RIGID_BODY_DTYPE).copy()

    def joints(self) -> np.ndarray:
        self.torch.cuda.synchronize()
        if not self.joint_count:
            return np.zeros(0, N.RIGID_JOINT_DTYPE)
        return self.d_joints[:self.joint_count * 96].cpu().numpy().view(N.RIGID_JOINT_DTYPE).copy()

    def walls(self) -> np.ndarray:
        self.torch.cuda.synchronize()
        return self.d_walls[:self.body_count * 48].cpu().numpy().view(N.RIGID_WALL_DTYPE).copy()

    def safety(self) -> int:
        self.torch.cuda.synchronize()
        return int(self.d_safety[0].item())
