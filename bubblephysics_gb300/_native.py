"""ctypes binding of include/bubblephysics.h (the C ABI of the native library).

The record types mirror the C structs field for field; sizes are checked against the header's pinned sizes at import.
The library is loaded from the package directory. There is no fallback: if the CUDA library is missing or no
suitable GPU is present, calls fail loudly with NativeError.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PACKAGE_DIR = Path(__file__).resolve().parent
LIBRARY_PATH = PACKAGE_DIR / "libbubblephysics_gb300.so"

# status codes (bp_status)
OK, E_INVALID, E_SUBSTEP_LIMIT, E_NONFINITE, E_CONTACT_VIOLATION, E_INFLIGHT, E_TIMEOUT, E_CUDA, E_CAPACITY, \
    E_UNAVAILABLE, E_ALLOC, E_WORLD_FAILED = range(12)

BUBBLE_ENABLED, BUBBLE_STATIC, BUBBLE_WRAP, BUBBLE_FORCE_DRIVEN = 1, 2, 4, 8
SEGMENT_POLYGON_EDGE, SEGMENT_CONVEX_START, SEGMENT_CONVEX_END, SEGMENT_HAS_OWNER, SEGMENT_ALLOWED_SIDE, \
    SEGMENT_KINEMATIC = 1, 2, 4, 8, 16, 32
BODY_POLYGON, BODY_CIRCLE, BODY_CAPSULE = 0, 1, 2
BODY_STATIC, BODY_KINEMATIC = 1, 2
WORLD_HAS_REGION, WORLD_MINIMUM_MARGIN_ONLY, WORLD_ASSERT_EVERY_SUBSTEP, WORLD_INJECT_STATE, \
    WORLD_NO_END_ASSERTION, WORLD_FORCE_MULTI_CTA, WORLD_RIGID_TREE, WORLD_NO_RIGID_TREE = 1, 2, 4, 8, 16, 32, 64, 128
BATCH_PER_WORLD_LAUNCH, BATCH_USE_GRAPH, BATCH_AUTOTUNE, BATCH_NO_STAGING = 1, 2, 4, 8
TERM_REMAINING, TERM_STIFFNESS, TERM_DISTANCE, TERM_MARGIN = range(4)
VIOLATION_NONE, VIOLATION_PAIR, VIOLATION_INSIDE_BODY, VIOLATION_EDGE_SIDE = range(4)

f2 = C.c_float * 2
f4 = C.c_float * 4


class Bubble(C.Structure):
    _fields_ = [("id", C.c_int64), ("center", f2), ("previous_center", f2), ("velocity", f2), ("mass", C.c_float),
                ("inverse_mass", C.c_float), ("radius", C.c_float), ("rotation", C.c_float),
                ("angular_velocity", C.c_float), ("contact_stiffness", C.c_float), ("damping", C.c_float),
                ("flags", C.c_uint32), ("category", C.c_uint32), ("mask", C.c_uint32),
                ("region_result", C.c_uint32), ("layer", C.c_int32)]


class Segment(C.Structure):
    _fields_ = [("id", C.c_int64), ("owner_id", C.c_int64), ("a", f2), ("b", f2), ("previous_start", f2),
                ("outward_sign", C.c_float), ("allowed_side", C.c_float), ("flags", C.c_uint32),
                ("category", C.c_uint32), ("mask", C.c_uint32), ("layer", C.c_int32)]


class Body(C.Structure):
    _fields_ = [("id", C.c_int64), ("position", f2), ("angle", C.c_float), ("bounding_radius", C.c_float),
                ("velocity", f2), ("angular_velocity", C.c_float), ("core_radius", C.c_float),
                ("half_length", C.c_float), ("kind", C.c_uint32), ("flags", C.c_uint32),
                ("vertex_offset", C.c_uint32), ("vertex_count", C.c_uint32), ("triangle_offset", C.c_uint32),
                ("triangle_count", C.c_uint32), ("category", C.c_uint32), ("mask", C.c_uint32),
                ("layer", C.c_int32)]


class ForceField(C.Structure):
    _fields_ = [("position", f2), ("rotation", C.c_float), ("falloff", C.c_float), ("direction", f2),
                ("strength", C.c_float), ("radius", C.c_float), ("kind", C.c_uint32), ("vertex_offset", C.c_uint32),
                ("vertex_count", C.c_uint32), ("filter_offset", C.c_uint32), ("filter_count", C.c_uint32),
                ("has_filter", C.c_uint32), ("reserved", C.c_uint32 * 2)]


class Band(C.Structure):
    _fields_ = [("bubble_id", C.c_int64), ("target", f2), ("stiffness", C.c_float), ("maximum_force", C.c_float)]


class Motor(C.Structure):
    _fields_ = [("bubble_id", C.c_int64), ("force", f2), ("torque", C.c_float), ("inertia", C.c_float)]


class WorldDesc(C.Structure):
    _fields_ = [("time_step", C.c_float), ("separation_tolerance", C.c_float), ("contact_tolerance", C.c_float),
                ("substep_split_multiplier", C.c_float), ("region", f4), ("global_force", f2), ("gravity", f2),
                ("candidate_limit", C.c_uint32), ("flags", C.c_uint32), ("inject_object", C.c_int64)]


class WorldDiagnostics(C.Structure):
    _fields_ = [("inject_substep", C.c_uint32), ("inject_position", f2), ("reserved", C.c_uint32)]


class WorldInput(C.Structure):
    _fields_ = [("bubbles", C.POINTER(Bubble)), ("bubble_count", C.c_uint32),
                ("segments", C.POINTER(Segment)), ("segment_count", C.c_uint32),
                ("bodies", C.POINTER(Body)), ("body_count", C.c_uint32),
                ("body_vertices", C.POINTER(C.c_float)), ("body_vertex_count", C.c_uint32),
                ("body_triangles", C.POINTER(C.c_uint32)), ("body_triangle_count", C.c_uint32),
                ("fields", C.POINTER(ForceField)), ("field_count", C.c_uint32),
                ("field_vertices", C.POINTER(C.c_float)), ("field_vertex_count", C.c_uint32),
                ("field_object_ids", C.POINTER(C.c_int64)), ("field_object_id_count", C.c_uint32),
                ("bands", C.POINTER(Band)), ("band_count", C.c_uint32),
                ("motors", C.POINTER(Motor)), ("motor_count", C.c_uint32),
                ("joint_ranges", C.POINTER(C.c_uint32)), ("joint_entity_count", C.c_uint32),
                ("joint_partners", C.POINTER(C.c_int64)), ("joint_partner_count", C.c_uint32)]


class StepReport(C.Structure):
    _fields_ = [("status", C.c_int32), ("substep_count", C.c_uint32), ("rebuild_count", C.c_uint32),
                ("candidate_count", C.c_uint32), ("body_candidate_count", C.c_uint32),
                ("candidate_overflow", C.c_uint32), ("max_candidates_per_object", C.c_uint32),
                ("contact_count", C.c_uint32), ("limiter_term", C.c_uint32), ("violation_kind", C.c_uint32),
                ("limiter_object", C.c_int64), ("violation_objects", C.c_int64 * 2), ("violation_edge", C.c_int64),
                ("violation_distance", C.c_float), ("cell_width", C.c_float), ("gpu_ms", C.c_float),
                ("removed_count", C.c_uint32), ("wrapped_count", C.c_uint32), ("contact_overflow", C.c_uint32)]

    def as_dict(self) -> dict:
        d = {name: getattr(self, name) for name, _ in self._fields_}
        d["violation_objects"] = list(self.violation_objects)
        return d


class Contact(C.Structure):
    _fields_ = [("participants", C.c_int64 * 2), ("kind", C.c_uint32), ("feature", C.c_uint32), ("normal", f2),
                ("point", f2), ("impulse", C.c_float), ("penetration", C.c_float), ("allowed_side", C.c_float),
                ("reserved", C.c_uint32 * 3)]


class CandidateKey(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("reserved", C.c_uint32), ("first", C.c_int64), ("second", C.c_int64)]


class BatchConfig(C.Structure):
    _fields_ = [("flags", C.c_uint32), ("threads_per_world", C.c_uint32), ("warp_world_max", C.c_uint32),
                ("group_width", C.c_uint32)]


class ContourConfig(C.Structure):
    _fields_ = [("max_edge", C.c_float), ("surface_tension", C.c_float), ("clearance", C.c_float),
                ("stride", C.c_uint32)]


class Sensor(C.Structure):
    _fields_ = [("id", C.c_int64), ("position", f2), ("angle", C.c_float), ("radius", C.c_float),
                ("vertex_offset", C.c_uint32), ("vertex_count", C.c_uint32), ("flags", C.c_uint32),
                ("reserved", C.c_uint32 * 3)]


SENSOR_ENTER_EVENTS, SENSOR_EXIT_EVENTS = 1, 2

class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("max_worlds", C.c_uint32), ("max_batch_worlds", C.c_uint32),
                ("streams", C.c_uint32), ("threads_per_world", C.c_uint32), ("warp_world_max", C.c_uint32),
                ("flags", C.c_uint32), ("group_width", C.c_uint32), ("reserved", C.c_uint32)]


class ServerCompletion(C.Structure):
    _fields_ = [("request_id", C.c_uint64), ("world", C.c_uint32), ("status", C.c_int32), ("steps", C.c_uint32),
                ("substeps", C.c_uint32), ("submitted_s", C.c_double), ("completed_s", C.c_double),
                ("report", StepReport)]


class ServerStats(C.Structure):
    _fields_ = [("worlds", C.c_uint32), ("resident", C.c_uint32), ("resident_bytes", C.c_uint64),
                ("hbm_budget_bytes", C.c_uint64), ("admissions", C.c_uint64), ("evictions", C.c_uint64),
                ("batches", C.c_uint64), ("batched_worlds", C.c_uint64), ("requests_done", C.c_uint64),
                ("bubble_substeps", C.c_uint64), ("device_ms", C.c_double)]


SERVER_PER_WORLD = 1

RECORD_SIZES = {Sensor: 48, ContourConfig: 16, ServerConfig: 40, ServerCompletion: 136, ServerStats: 80, Bubble: 80, Segment: 64, Body: 80, ForceField: 64, Band: 24, Motor: 24, WorldDesc: 64,
                StepReport: 96, Contact: 64, CandidateKey: 24}
for _t, _n in RECORD_SIZES.items():
    assert C.sizeof(_t) == _n, f"{_t.__name__} is {C.sizeof(_t)} bytes, the C ABI says {_n}"

# numpy views of the records (for bulk packing)
BUBBLE_DTYPE = np.dtype({"names": ["id", "center", "previous_center", "velocity", "mass", "inverse_mass", "radius",
                                   "rotation", "angular_velocity", "contact_stiffness", "damping", "flags", "category",
                                   "mask", "region_result", "layer"],
                         "formats": ["<i8", ("<f4", 2), ("<f4", 2), ("<f4", 2), "<f4", "<f4", "<f4", "<f4", "<f4",
                                     "<f4", "<f4", "<u4", "<u4", "<u4", "<u4", "<i4"],
                         "offsets": [0, 8, 16, 24, 32, 36, 40, 44, 48, 52, 56, 60, 64, 68, 72, 76], "itemsize": 80})
SEGMENT_DTYPE = np.dtype({"names": ["id", "owner_id", "a", "b", "previous_start", "outward_sign", "allowed_side",
                                    "flags", "category", "mask", "layer"],
                          "formats": ["<i8", "<i8", ("<f4", 2), ("<f4", 2), ("<f4", 2), "<f4", "<f4", "<u4", "<u4",
                                      "<u4", "<i4"],
                          "offsets": [0, 8, 16, 24, 32, 40, 44, 48, 52, 56, 60], "itemsize": 64})
BODY_DTYPE = np.dtype({"names": ["id", "position", "angle", "bounding_radius", "velocity", "angular_velocity",
                                 "core_radius", "half_length", "kind", "flags", "vertex_offset", "vertex_count",
                                 "triangle_offset", "triangle_count", "category", "mask", "layer"],
                       "formats": ["<i8", ("<f4", 2), "<f4", "<f4", ("<f4", 2), "<f4", "<f4", "<f4", "<u4", "<u4",
                                   "<u4", "<u4", "<u4", "<u4", "<u4", "<u4", "<i4"],
                       "offsets": [0, 8, 16, 20, 24, 32, 36, 40, 44, 48, 52, 56, 60, 64, 68, 72, 76], "itemsize": 80})
CONTACT_DTYPE = np.dtype({"names": ["participants", "kind", "feature", "normal", "point", "impulse", "penetration",
                                    "allowed_side", "reserved"],
                          "formats": [("<i8", 2), "<u4", "<u4", ("<f4", 2), ("<f4", 2), "<f4", "<f4", "<f4",
                                      ("<u4", 3)],
                          "offsets": [0, 16, 20, 24, 32, 40, 44, 48, 52], "itemsize": 64})
SENSOR_EVENT_DTYPE = np.dtype({"names": ["sensor", "object", "kind", "point", "object_kind"],
                               "formats": ["<i8", "<i8", "<u4", ("<f4", 2), "<u4"],
                               "offsets": [0, 8, 16, 20, 28], "itemsize": 32})
CONTACT_EVENT_DTYPE = np.dtype({"names": ["kind", "reserved", "objects", "point", "normal", "impulse", "reserved2"],
                                "formats": ["<u4", "<u4", ("<i8", 2), ("<f4", 2), ("<f4", 2), "<f4", "<f4"],
                                "offsets": [0, 4, 8, 24, 32, 40, 44], "itemsize": 48})
KEY_DTYPE = np.dtype({"names": ["kind", "reserved", "first", "second"], "formats": ["<u4", "<u4", "<i8", "<i8"],
                      "offsets": [0, 4, 8, 16], "itemsize": 24})
# rigid solver records (bp_rigid_body 160 B, bp_rigid_joint 96 B, bp_rigid_correction 64 B, bp_rigid_wall 48 B)
RIGID_BODY_DTYPE = np.dtype({"names": ["id", "reserved0", "pose", "previous", "motion", "physical", "ranges", "flags",
                                       "filter", "shape", "limits"],
                             "formats": ["<u8", "<u8", ("<f4", 4), ("<f4", 4), ("<f4", 4), ("<f4", 4), ("<u4", 4),
                                         ("<u4", 4), ("<u4", 4), ("<f4", 4), ("<f4", 4)],
                             "offsets": [0, 8, 16, 32, 48, 64, 80, 96, 112, 128, 144], "itemsize": 160})
RIGID_JOINT_DTYPE = np.dtype({"names": ["id", "reserved0", "ends", "anchors", "parameters", "limits", "state"],
                              "formats": ["<u8", "<u8", ("<u4", 4), ("<f4", 4), ("<f4", 4), ("<f4", 4), ("<f4", 4)],
                              "offsets": [0, 8, 16, 32, 48, 64, 80], "itemsize": 96})
RIGID_CORRECTION_DTYPE = np.dtype({"names": ["first", "second", "velocity_first", "velocity_second"],
                                   "formats": [("<f4", 4)] * 4, "offsets": [0, 16, 32, 48], "itemsize": 64})
RIGID_WALL_DTYPE = np.dtype({"names": ["participants", "geometry", "extra"],
                             "formats": [("<i8", 2), ("<f4", 4), ("<f4", 4)], "offsets": [0, 16, 32], "itemsize": 48})
RIGID_CANDIDATE_DTYPE = np.dtype({"names": ["participants", "metadata"], "formats": [("<i8", 2), ("<u4", 4)],
                                  "offsets": [0, 16], "itemsize": 32})
JOINT_WORLD_END = 0xFFFFFFFF
RIGID_SAFETY_NONFINITE, RIGID_SAFETY_ROTATION_BUDGET, RIGID_SAFETY_INVALID = 1, 18, 256
REPORT_DTYPE = np.dtype({"names": [n for n, _ in StepReport._fields_],
                         "formats": ["<i4"] + ["<u4"] * 9 + ["<i8", ("<i8", 2), "<i8", "<f4", "<f4", "<f4",
                                                             "<u4", "<u4", "<u4"],
                         "offsets": [0, 4, 8, 12, 16, 20, 24, 28, 32, 36, 40, 48, 64, 72, 76, 80, 84, 88, 92],
                         "itemsize": 96})


class NativeError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)} ({status})")


STATUS_NAMES = {OK: "ok", E_INVALID: "invalid snapshot", E_SUBSTEP_LIMIT: "substep limit exceeded",
                E_NONFINITE: "non-finite values", E_CONTACT_VIOLATION: "contact violation",
                E_INFLIGHT: "frame in flight", E_TIMEOUT: "bounded device wait timed out", E_CUDA: "CUDA failure",
                E_CAPACITY: "capacity overflow", E_UNAVAILABLE: "CUDA device unavailable",
                E_ALLOC: "allocation failed", E_WORLD_FAILED: "world failed earlier"}

_P = C.c_void_p
_SIGNATURES = {
    "bp_abi_version": (C.c_int, []),
    "bp_status_string": (C.c_char_p, [C.c_int]),
    "bp_device_available": (C.c_int, [C.c_int]),
    "bp_context_create": (C.c_int, [C.c_int, C.c_uint32, C.POINTER(_P)]),
    "bp_context_destroy": (C.c_int, [_P]),
    "bp_world_create": (C.c_int, [_P, C.POINTER(WorldDesc), C.POINTER(WorldInput), C.POINTER(_P)]),
    "bp_world_destroy": (C.c_int, [_P]),
    "bp_world_write_bubbles": (C.c_int, [_P, _P, C.c_uint32]),
    "bp_world_set_diagnostics": (C.c_int, [_P, C.POINTER(WorldDiagnostics)]),
    "bp_world_step": (C.c_int, [_P, C.c_uint32, _P]),
    "bp_world_read_bubbles": (C.c_int, [_P, _P, C.c_uint32, C.POINTER(C.c_uint32)]),
    "bp_world_read_contacts": (C.c_int, [_P, _P, C.c_uint32, C.POINTER(C.c_uint32)]),
    "bp_world_contact_events": (C.c_int, [_P, _P, C.c_uint32, _P, C.c_uint32, _P, C.c_uint32, C.c_float, _P, C.c_uint32,
                                          C.POINTER(C.c_uint32)]),
    "bp_world_set_contact_history": (C.c_int, [_P, _P, C.c_uint32]),
    "bp_world_read_contact_history": (C.c_int, [_P, _P, C.c_uint32, C.POINTER(C.c_uint32)]),
    "bp_world_read_candidates": (C.c_int, [_P, _P, C.c_uint32, C.POINTER(C.c_uint32)]),
    "bp_world_read_cells": (C.c_int, [_P, _P, C.c_uint32, C.POINTER(C.c_uint32)]),
    "bp_world_read_rigid_keys": (C.c_int, [_P, _P, C.c_uint32, C.POINTER(C.c_uint32)]),
    "bp_world_read_substeps": (C.c_int, [_P, _P, C.c_uint32, C.POINTER(C.c_uint32)]),
    "bp_batch_create": (C.c_int, [_P, C.c_uint32, C.POINTER(WorldDesc), C.POINTER(WorldInput),
                                  C.POINTER(BatchConfig), C.POINTER(_P)]),
    "bp_batch_destroy": (C.c_int, [_P]),
    "bp_batch_step": (C.c_int, [_P, C.c_uint32, _P]),
    "bp_batch_counters": (C.c_int, [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "bp_batch_read_bubbles": (C.c_int, [_P, C.c_uint32, _P, C.c_uint32, C.POINTER(C.c_uint32)]),
    "bp_batch_write_state": (C.c_int, [_P, _P, C.c_uint64]),
    "bp_batch_read_state": (C.c_int, [_P, _P, C.c_uint64]),
    "bp_batch_tuning": (C.c_int, [_P, C.POINTER(C.c_uint32), C.c_uint32]),
    "bp_batch_adjacency_entries": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
    "bp_static_polygon_edges": (C.c_int, [C.POINTER(C.c_float), C.c_uint32, C.c_int64, C.c_int64, C.c_uint32,
                                          C.POINTER(Segment), C.c_uint32, C.POINTER(C.c_uint32)]),
    "bp_device_contact_law": (C.c_int, [_P, C.c_uint32, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_uint32]),
    "bp_world_step_noalloc": (C.c_int, [C.POINTER(WorldDesc), _P, C.c_uint32, _P, C.c_uint32, C.c_uint32, _P, _P]),
    "bp_world_contours": (C.c_int, [_P, C.POINTER(ContourConfig), _P, _P, _P, _P, C.POINTER(C.c_uint32),
                                    C.POINTER(C.c_float)]),
    "bp_world_hit_test": (C.c_int, [_P, C.POINTER(ContourConfig), _P, C.c_uint32, _P, _P, _P]),
    "bp_world_set_sensors": (C.c_int, [_P, _P, C.c_uint32, _P, C.c_uint32, _P, _P]),
    "bp_world_read_sensor_events": (C.c_int, [_P, _P, C.c_uint32, C.POINTER(C.c_uint32)]),
    "bp_server_create": (C.c_int, [_P, C.POINTER(ServerConfig), C.POINTER(_P)]),
    "bp_server_destroy": (C.c_int, [_P]),
    "bp_server_add_world": (C.c_int, [_P, C.POINTER(WorldDesc), C.POINTER(WorldInput), C.POINTER(C.c_uint32)]),
    "bp_server_submit": (C.c_int, [_P, C.c_uint32, C.c_uint32, C.POINTER(C.c_uint64)]),
    "bp_server_progress": (C.c_int, [_P, C.c_uint32, C.POINTER(C.c_uint32)]),
    "bp_server_poll": (C.c_int, [_P, _P, C.c_uint32, C.POINTER(C.c_uint32)]),
    "bp_server_pending": (C.c_int, [_P, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    "bp_server_read_bubbles": (C.c_int, [_P, C.c_uint32, _P, C.c_uint32, C.POINTER(C.c_uint32)]),
    "bp_server_read_stats": (C.c_int, [_P, C.POINTER(ServerStats)]),
    "bp_server_clock": (C.c_double, []),
    "bp_rigid_predict": (C.c_int, [_P, C.c_uint32, _P, C.c_uint32, _P, C.c_uint32, C.c_uint32, C.c_float, _P, _P,
                                   C.c_uint32, _P, _P, _P]),
    "bp_rigid_solve_joints": (C.c_int, [_P, C.c_uint32, _P, C.c_uint32, _P, _P, C.c_uint32, _P, C.c_uint32, C.c_float,
                                        C.c_uint32, C.c_uint32, _P, _P]),
    "bp_rigid_finish": (C.c_int, [_P, C.c_uint32, _P, C.c_uint32, C.POINTER(C.c_float), _P, _P]),
    "bp_rigid_body_candidates": (C.c_int, [_P, C.c_uint32, C.c_uint32, _P, _P, C.c_uint32, C.c_uint32, _P, _P, _P,
                                           _P]),
    "bp_rigid_ccd": (C.c_int, [_P, C.c_uint32, _P, C.c_uint32, _P, C.c_uint32, _P, _P, C.c_uint32, _P, _P]),
    "bp_rigid_solve_contacts": (C.c_int, [_P, C.c_uint32, _P, C.c_uint32, _P, C.c_uint32, _P, _P, C.c_uint32, _P,
                                          _P, _P]),
    "bp_rigid_guard_walls": (C.c_int, [_P, C.c_uint32, _P, C.c_uint32, _P, C.c_uint32, C.c_uint32, _P, _P,
                                       C.c_uint32, _P, _P]),
}
EXPORTED_SYMBOLS = tuple(_SIGNATURES)

_lib = None


def library(path: os.PathLike | str | None = None) -> C.CDLL:
    """Loads the native library (once). Raises if it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIBRARY_PATH
    if not p.exists():
        raise NativeError(E_UNAVAILABLE, f"native library {p.name} is not built (run __graft_entry__.build())")
    lib = C.CDLL(str(p))
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(status: int, where: str) -> int:
    if status != OK:
        raise NativeError(status, where)
    return status


def ptr(array: np.ndarray, ctype=C.c_void_p):
    """ctypes pointer to a contiguous numpy array (None for an empty array)."""
    if array is None or array.size == 0:
        return None
    assert array.flags["C_CONTIGUOUS"]
    return C.cast(array.ctypes.data, C.POINTER(ctype)) if ctype is not C.c_void_p else C.c_void_p(array.ctypes.data)
