"""World specification in array form and its packing into the C ABI's bp_world_desc / bp_world_input.

A WorldSpec is what NativeSolverInput carries for one frame (Sources/BubblePhysicsNativeMetal/NativeSolverInput.swift:
165-190): bubbles sorted by id, static segments sorted by id, obstacle bodies with their local geometry, force records
and joint exclusion lists, plus the configuration (time step, tolerances, region, global force, package switches).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _native as N


def empty(dtype) -> np.ndarray:
    return np.zeros(0, dtype=dtype)


@dataclass
class WorldSpec:
    bubbles: np.ndarray                                  # BUBBLE_DTYPE, sorted by id
    segments: np.ndarray = field(default_factory=lambda: empty(N.SEGMENT_DTYPE))
    bodies: np.ndarray = field(default_factory=lambda: empty(N.BODY_DTYPE))
    body_vertices: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.float32))
    body_triangles: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.uint32))
    fields: list = field(default_factory=list)           # list of N.ForceField
    field_vertices: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.float32))
    field_object_ids: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    bands: list = field(default_factory=list)            # list of N.Band, sorted by bubble id
    motors: list = field(default_factory=list)           # list of N.Motor, sorted by bubble id
    joint_ranges: np.ndarray | None = None               # (entities, 2) uint32
    joint_partners: np.ndarray | None = None             # int64
    time_step: float = 1.0 / 60.0
    separation_tolerance: float = 0.002
    contact_tolerance: float = 0.001
    substep_split_multiplier: float = 1.0
    region: tuple | None = None                          # (min_x, min_y, max_x, max_y)
    global_force: tuple = (0.0, 0.0)
    gravity: tuple = (0.0, 0.0)
    candidate_limit: int = 128
    flags: int = 0
    inject_object: int = 0

    @property
    def bubble_count(self) -> int:
        return int(self.bubbles.shape[0])

    def desc(self) -> N.WorldDesc:
        d = N.WorldDesc()
        d.time_step = self.time_step
        d.separation_tolerance = self.separation_tolerance
        d.contact_tolerance = self.contact_tolerance
        d.substep_split_multiplier = self.substep_split_multiplier
        flags = self.flags
        if self.region is not None:
            d.region[:] = [float(v) for v in self.region]
            flags |= N.WORLD_HAS_REGION
        d.global_force[:] = [float(v) for v in self.global_force]
        d.gravity[:] = [float(v) for v in self.gravity]
        d.candidate_limit = self.candidate_limit
        d.flags = flags
        d.inject_object = self.inject_object
        return d


class PackedInput:
    """A bp_world_input whose arrays stay alive as long as this object."""

    def __init__(self, spec: WorldSpec):
        self.keep = []

        def arr(a, dtype):
            a = np.ascontiguousarray(a, dtype=dtype)
            self.keep.append(a)
            return a

        inp = N.WorldInput()
        b = arr(spec.bubbles, N.BUBBLE_DTYPE)
        inp.bubbles = C.cast(b.ctypes.data, C.POINTER(N.Bubble)) if b.size else None
        inp.bubble_count = b.shape[0]
        s = arr(spec.segments, N.SEGMENT_DTYPE)
        inp.segments = C.cast(s.ctypes.data, C.POINTER(N.Segment)) if s.size else None
        inp.segment_count = s.shape[0]
        bo = arr(spec.bodies, N.BODY_DTYPE)
        inp.bodies = C.cast(bo.ctypes.data, C.POINTER(N.Body)) if bo.size else None
        inp.body_count = bo.shape[0]
        bv = arr(spec.body_vertices, np.float32)
        inp.body_vertices = N.ptr(bv, C.c_float)
        inp.body_vertex_count = bv.shape[0] if bv.ndim == 2 else bv.size // 2
        bt = arr(spec.body_triangles, np.uint32)
        inp.body_triangles = N.ptr(bt, C.c_uint32)
        inp.body_triangle_count = bt.shape[0] if bt.ndim == 2 else bt.size // 3
        if spec.fields:
            fa = (N.ForceField * len(spec.fields))(*spec.fields)
            self.keep.append(fa)
            inp.fields = C.cast(fa, C.POINTER(N.ForceField))
        inp.field_count = len(spec.fields)
        fv = arr(spec.field_vertices, np.float32)
        inp.field_vertices = N.ptr(fv, C.c_float)
        inp.field_vertex_count = fv.shape[0] if fv.ndim == 2 else fv.size // 2
        fi = arr(spec.field_object_ids, np.int64)
        inp.field_object_ids = N.ptr(fi, C.c_int64)
        inp.field_object_id_count = fi.size
        if spec.bands:
            ba = (N.Band * len(spec.bands))(*spec.bands)
            self.keep.append(ba)
            inp.bands = C.cast(ba, C.POINTER(N.Band))
        inp.band_count = len(spec.bands)
        if spec.motors:
            ma = (N.Motor * len(spec.motors))(*spec.motors)
            self.keep.append(ma)
            inp.motors = C.cast(ma, C.POINTER(N.Motor))
        inp.motor_count = len(spec.motors)
        if spec.joint_ranges is not None and len(spec.joint_ranges):
            jr = arr(spec.joint_ranges, np.uint32)
            inp.joint_ranges = N.ptr(jr, C.c_uint32)
            inp.joint_entity_count = jr.shape[0]
            jp = arr(spec.joint_partners if spec.joint_partners is not None else np.zeros(0, np.int64), np.int64)
            inp.joint_partners = N.ptr(jp, C.c_int64)
            inp.joint_partner_count = jp.size
        self.input = inp
        self.desc = spec.desc()


def make_bubbles(centers, radii, *, ids=None, velocities=None, masses=None, stiffness=229.0, damping=0.0,
                 flags=N.BUBBLE_FORCE_DRIVEN, category=1, mask=0xFFFFFFFF, static=None) -> np.ndarray:
    """Bubble records in id order (ids default to 1..n). Static bubbles get inverse mass 0."""
    centers = np.asarray(centers, np.float32).reshape(-1, 2)
    n = centers.shape[0]
    b = np.zeros(n, N.BUBBLE_DTYPE)
    b["id"] = np.arange(1, n + 1, dtype=np.int64) if ids is None else np.asarray(ids, np.int64)
    b["center"] = centers
    b["previous_center"] = centers
    if velocities is not None:
        b["velocity"] = np.asarray(velocities, np.float32).reshape(-1, 2)
    b["radius"] = np.broadcast_to(np.asarray(radii, np.float32), (n,))
    m = np.ones(n, np.float32) if masses is None else np.broadcast_to(np.asarray(masses, np.float32), (n,))
    b["mass"] = m
    b["inverse_mass"] = (1.0 / m.astype(np.float64)).astype(np.float32)
    b["contact_stiffness"] = np.broadcast_to(np.asarray(stiffness, np.float32), (n,))
    b["damping"] = np.broadcast_to(np.asarray(damping, np.float32), (n,))
    b["flags"] = flags
    b["category"] = category
    b["mask"] = mask
    if static is not None:
        st = np.asarray(static, bool)
        b["inverse_mass"][st] = 0.0
        b["flags"][st] = (b["flags"][st] | N.BUBBLE_ENABLED | N.BUBBLE_STATIC) & ~np.uint32(N.BUBBLE_FORCE_DRIVEN)
    return b
