"""ctypes loader of the CPU oracle (liboracle built from bp_oracle.cpp). TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs use this module, and only as the checker / the timed CPU
baseline. The product package never imports it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

from bubblephysics_gb300 import _native as N
from bubblephysics_gb300.spec import PackedInput, WorldSpec

ORACLE_DIR = Path(__file__).resolve().parent
ORACLE_LIB = ORACLE_DIR / "libbp_oracle.so"

_lib = None


def build(force: bool = False) -> Path:
    """Builds the oracle shared library with its Makefile (gcc, -ffp-contract=off, OpenMP)."""
    src = ORACLE_DIR / "bp_oracle.cpp"
    header = ORACLE_DIR.parent / "include" / "bubblephysics.h"
    if force or not ORACLE_LIB.exists() or ORACLE_LIB.stat().st_mtime < max(src.stat().st_mtime, header.stat().st_mtime):
        subprocess.run(["make", "-s", "-B" if force else "-s", "-C", str(ORACLE_DIR)], check=True)
    return ORACLE_LIB


def library() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(ORACLE_LIB))
        P = C.c_void_p
        sig = {
            "bpo_world_create": (C.c_int, [C.POINTER(N.WorldDesc), C.POINTER(N.WorldInput), C.c_int, C.POINTER(P)]),
            "bpo_world_destroy": (None, [P]),
            "bpo_world_set_injection": (C.c_int, [P, C.c_uint32, C.c_float, C.c_float]),
            "bpo_world_step": (C.c_int, [P, C.c_uint32, P]),
            "bpo_worlds_step": (C.c_int, [C.POINTER(P), C.c_uint32, C.c_uint32, C.c_int, C.POINTER(C.c_uint64)]),
            "bpo_worlds_step_reports": (C.c_int, [C.POINTER(P), C.c_uint32, C.c_uint32, C.c_int, P]),
            "bpo_set_threads": (C.c_int, [C.c_int]),
            "bpo_world_read_bubbles": (C.c_int, [P, P, C.c_uint32, C.POINTER(C.c_uint32)]),
            "bpo_world_read_state64": (C.c_int, [P, P, C.c_uint32]),
            "bpo_world_read_contacts": (C.c_int, [P, P, C.c_uint32, C.POINTER(C.c_uint32)]),
            "bpo_world_read_candidates": (C.c_int, [P, P, C.c_uint32, C.POINTER(C.c_uint32)]),
            "bpo_world_read_cells": (C.c_int, [P, P, C.c_uint32, C.POINTER(C.c_uint32)]),
            "bpo_world_rigid_keys": (C.c_uint32, [P, P, C.c_uint32]),
            "bpo_world_contours": (C.c_int, [P, C.c_float, C.c_float, C.c_float, C.c_uint32, P, P, P, P]),
            "bpo_world_hit_test": (C.c_int, [P, C.c_float, C.c_float, C.c_float, P, C.c_uint32, P, P, P]),
            "bpo_world_sensor_events": (C.c_uint32, [P, P, C.c_uint32, P, P, P, P, C.c_uint32]),
            "bpo_world_read_substeps": (C.c_int, [P, P, C.c_uint32, C.POINTER(C.c_uint32)]),
            "bpo_world_set_trace": (C.c_int, [P, C.c_int]),
            "bpo_world_read_trace": (C.c_int, [P, P, C.c_uint32, C.POINTER(C.c_uint32)]),
            "bpo_contact_law": (C.c_int, [C.c_uint32, C.c_int, P, P, C.c_uint32]),
            "bpo_contact_events": (C.c_int, [P, C.c_uint32, P, P, P, C.c_uint32, P, C.c_uint32, P, C.c_uint32, P,
                                             C.c_uint32, C.c_float, P, C.c_uint32, P, P, P]),
            "bpo_rigid_predict": (C.c_int, [P, C.c_uint32, P, C.c_uint32, P, C.c_uint32, C.c_uint32, C.c_float, P, P,
                                            C.c_uint32, P, P]),
            "bpo_rigid_solve_joints": (C.c_int, [P, C.c_uint32, P, C.c_uint32, P, P, C.c_uint32, P, C.c_uint32,
                                                 C.c_float, C.c_uint32, C.c_uint32, P]),
            "bpo_rigid_finish": (C.c_int, [P, C.c_uint32, P, C.c_uint32, P, P]),
            "bpo_sincos": (C.c_int, [P, P, C.c_uint32]),
            "bpo_rigid_body_candidates": (C.c_int, [P, C.c_uint32, C.c_uint32, P, P, C.c_uint32, C.c_uint32, P, P,
                                                    P]),
            "bpo_rigid_ccd": (C.c_int, [P, C.c_uint32, P, C.c_uint32, P, C.c_uint32, P, P, C.c_uint32, P]),
            "bpo_rigid_solve_contacts": (C.c_int, [P, C.c_uint32, P, C.c_uint32, P, C.c_uint32, P, P, C.c_uint32, P,
                                                   P]),
            "bpo_rigid_guard_walls": (C.c_int, [P, C.c_uint32, P, C.c_uint32, P, C.c_uint32, C.c_uint32, P, P,
                                                C.c_uint32, P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


class OracleWorld:
    """The oracle's counterpart of bubblephysics_gb300.solver.World (same methods, CPU, float or double)."""

    def __init__(self, spec: WorldSpec, precision: int = 32):
        self.lib = library()
        self.spec = spec
        packed = PackedInput(spec)
        handle = C.c_void_p()
        st = self.lib.bpo_world_create(C.byref(packed.desc), C.byref(packed.input), precision, C.byref(handle))
        if st != 0:
            raise N.NativeError(st, "bpo_world_create")
        self.handle = handle
        self.n = spec.bubble_count
        self.precision = precision

    def __del__(self):
        try:
            if self.handle:
                self.lib.bpo_world_destroy(self.handle)
                self.handle = None
        except Exception:
            pass

    def set_injection(self, substep: int, position):
        self.lib.bpo_world_set_injection(self.handle, substep, float(position[0]), float(position[1]))

    def step(self, steps: int = 1):
        reports = np.zeros(max(steps, 1), N.REPORT_DTYPE)
        status = self.lib.bpo_world_step(self.handle, steps, C.c_void_p(reports.ctypes.data))
        return status, reports[:steps]

    def bubbles(self) -> np.ndarray:
        out = np.zeros(self.n, N.BUBBLE_DTYPE)
        count = C.c_uint32()
        self.lib.bpo_world_read_bubbles(self.handle, C.c_void_p(out.ctypes.data), self.n, C.byref(count))
        return out

    def state64(self) -> np.ndarray:
        out = np.zeros((self.n, 4), np.float64)
        self.lib.bpo_world_read_state64(self.handle, C.c_void_p(out.ctypes.data), self.n)
        return out

    def _read(self, fn, dtype):
        count = C.c_uint32()
        fn(self.handle, None, 0, C.byref(count))
        out = np.zeros(count.value, dtype)
        if count.value:
            fn(self.handle, C.c_void_p(out.ctypes.data), count.value, C.byref(count))
        return out

    def contacts(self) -> np.ndarray:
        return self._read(self.lib.bpo_world_read_contacts, N.CONTACT_DTYPE)

    def candidates(self) -> np.ndarray:
        return self._read(self.lib.bpo_world_read_candidates, N.KEY_DTYPE)

    def cells(self) -> np.ndarray:
        out = np.zeros((self.n, 2), np.int64)
        count = C.c_uint32()
        self.lib.bpo_world_read_cells(self.handle, C.c_void_p(out.ctypes.data), self.n, C.byref(count))
        return out

    def set_trace(self, on: bool = True):
        """Record every bubble's state after each substep of the following steps."""
        self.lib.bpo_world_set_trace(self.handle, 1 if on else 0)

    def trace(self):
        """The last step's substeps: h (substeps,) and the state after each, (substeps, n, 4: x, y, vx, vy)."""
        t = self._read(self.lib.bpo_world_read_trace, np.float64).reshape(-1, 1 + 4 * self.n)
        return t[:, 0], t[:, 1:].reshape(-1, self.n, 4)

    def substeps(self) -> np.ndarray:
        return self._read(self.lib.bpo_world_read_substeps, np.float64)

    def contours(self, max_edge=8.0, surface_tension=20.0, clearance=1e-4, stride=0):
        """Contours of the published state (the CUDA path's contour passes restated in float): points (n, stride, 2),
        counts (n,), level (n, stride), shape (n, 6)."""
        radii = self.bubbles()["radius"]
        need = max([64] + [int(np.ceil(np.float32(r) / np.float32(max_edge) * np.float32(4.0 * np.float32(np.pi))))
                           for r in radii])
        stride = stride or need
        points = np.zeros((self.n, stride, 2), np.float32)
        counts = np.zeros(self.n, np.uint32)
        level = np.zeros((self.n, stride), np.float32)
        shape = np.zeros((self.n, 6), np.float32)
        st = self.lib.bpo_world_contours(self.handle, max_edge, surface_tension, clearance, stride,
                                         C.c_void_p(points.ctypes.data), C.c_void_p(counts.ctypes.data),
                                         C.c_void_p(level.ctypes.data), C.c_void_p(shape.ctypes.data))
        assert st == 0, st
        return points, counts, level, shape

    def hit_test(self, points, max_edge=8.0, surface_tension=20.0, clearance=1e-4):
        """Hit test of query points (the CUDA path's rule restated in float): ids, layers, found."""
        q = np.ascontiguousarray(points, np.float32).reshape(-1, 2)
        ids = np.zeros(q.shape[0], np.int64)
        layers = np.zeros(q.shape[0], np.int32)
        found = np.zeros(q.shape[0], np.uint32)
        st = self.lib.bpo_world_hit_test(self.handle, max_edge, surface_tension, clearance, C.c_void_p(q.ctypes.data),
                                         q.shape[0], C.c_void_p(ids.ctypes.data), C.c_void_p(layers.ctypes.data),
                                         C.c_void_p(found.ctypes.data))
        assert st == 0, st
        return ids, layers, found

    def sensor_events(self, sensors, vertices, state, allowed=None):
        """Sensor events of the published state against `state` (uint8, sensors x (bubbles, then bodies), updated in
        place); `allowed` (same shape, optional) masks pairs out."""
        arr = (N.Sensor * max(len(sensors), 1))(*sensors)
        v = np.ascontiguousarray(np.zeros((0, 2)) if vertices is None else vertices, np.float32).reshape(-1, 2)
        cap = max(state.size, 1)
        ok = None if allowed is None else np.ascontiguousarray(allowed, np.uint8)
        out = np.zeros(cap, N.SENSOR_EVENT_DTYPE)
        count = self.lib.bpo_world_sensor_events(self.handle, C.cast(arr, C.c_void_p), len(sensors),
                                                 C.c_void_p(v.ctypes.data),
                                                 None if ok is None else C.c_void_p(ok.ctypes.data),
                                                 C.c_void_p(state.ctypes.data),
                                                 C.c_void_p(out.ctypes.data), cap)
        return out[:count]

    def rigid_keys(self) -> np.ndarray:
        """Sorted LBVH keys of the rigid leaves for the last step (the CUDA path's key rule restated in float)."""
        count = self.lib.bpo_world_rigid_keys(self.handle, None, 0)
        out = np.zeros(count, np.uint64)
        if count:
            self.lib.bpo_world_rigid_keys(self.handle, C.c_void_p(out.ctypes.data), count)
        return out


def step_worlds(worlds: list[OracleWorld], steps: int, threads: int = 0) -> int:
    """Steps many oracle worlds with OpenMP over worlds; returns bubble-substeps advanced."""
    lib = library()
    arr = (C.c_void_p * len(worlds))(*[w.handle.value for w in worlds])
    total = C.c_uint64()
    lib.bpo_worlds_step(arr, len(worlds), steps, threads, C.byref(total))
    return total.value


def step_worlds_reports(worlds: list[OracleWorld], steps: int, threads: int = 0) -> np.ndarray:
    """Steps many oracle worlds with OpenMP over worlds and returns every report, shape (steps, worlds)."""
    lib = library()
    arr = (C.c_void_p * len(worlds))(*[w.handle.value for w in worlds])
    out = np.zeros((max(steps, 1), len(worlds)), N.REPORT_DTYPE)
    lib.bpo_worlds_step_reports(arr, len(worlds), steps, threads, C.c_void_p(out.ctypes.data))
    return out[:steps]


def contact_events(records: np.ndarray, segments: np.ndarray, interested, history, removed=(), step: float = 1 / 60):
    """Contact began / ended events of one step from its contact records (CONTACT_DTYPE, id form; extra records
    appended) and the world's segments (their owners): (events CONTACT_EVENT_DTYPE, new history (pairs, 2))."""
    rec = np.ascontiguousarray(records, N.CONTACT_DTYPE)
    seg_ids = np.ascontiguousarray(segments["id"], np.int64)
    seg_owners = np.ascontiguousarray(segments["owner_id"], np.int64)
    has_owner = np.ascontiguousarray((segments["flags"] & N.SEGMENT_HAS_OWNER) != 0, np.uint8)
    ids = np.ascontiguousarray(np.asarray(list(interested), np.int64))
    gone = np.ascontiguousarray(np.asarray(list(removed), np.int64))
    hist = np.ascontiguousarray(np.asarray(history, np.int64).reshape(-1, 2)).view(np.uint64)
    cap = 2 * (rec.size + hist.shape[0]) + 1
    out = np.zeros(cap, N.CONTACT_EVENT_DTYPE)
    nxt = np.zeros((rec.size + 1, 2), np.uint64)
    n_ev, n_hist = C.c_uint32(), C.c_uint32()
    ptr = lambda a: C.c_void_p(a.ctypes.data) if a.size else None
    library().bpo_contact_events(ptr(rec), rec.size, ptr(seg_ids), ptr(seg_owners), ptr(has_owner), seg_ids.size,
                                 ptr(ids), ids.size, ptr(hist), hist.shape[0], ptr(gone), gone.size, float(step),
                                 C.c_void_p(out.ctypes.data), cap, C.byref(n_ev), C.c_void_p(nxt.ctypes.data),
                                 C.byref(n_hist))
    return out[:n_ev.value], nxt[:n_hist.value].view(np.int64)


def set_threads(threads: int) -> int:
    return library().bpo_set_threads(threads)


def contact_law(mode: int, cases: np.ndarray, precision: int = 32) -> np.ndarray:
    cases = np.ascontiguousarray(cases, np.float64).reshape(-1, 8)
    out = np.zeros_like(cases)
    library().bpo_contact_law(mode, precision, C.c_void_p(cases.ctypes.data), C.c_void_p(out.ctypes.data), cases.shape[0])
    return out


def sincos(x: np.ndarray) -> np.ndarray:
    """(cos, sin) of float32 angles by the library's own float sin / cos (the oracle's copy)."""
    x = np.ascontiguousarray(x, np.float32)
    out = np.zeros((x.size, 2), np.float32)
    library().bpo_sincos(C.c_void_p(x.ctypes.data), C.c_void_p(out.ctypes.data), x.size)
    return out


class OracleRigid:
    """The rigid solver passes on host arrays (the oracle of bubblephysics_gb300.rigid.RigidSolver): predict
    (NPK:66-115), body-pair rows, CCD, contact rounds, the joint rounds (NCK:375-562), the wall guard and finish
    (NPK:118-263), same arguments and record layouts."""

    def __init__(self, bodies, vertices, segments=None, joints=None, bubble_count: int = 0, triangles=None,
                 row_width: int = 16):
        self.body_records = np.array(bodies, N.RIGID_BODY_DTYPE)
        self.vertices = np.ascontiguousarray(np.asarray(vertices, np.float32).reshape(-1, 2))
        self.triangles = np.ascontiguousarray(np.zeros((0, 4), np.uint32) if triangles is None
                                              else np.asarray(triangles, np.uint32).reshape(-1, 4))
        self.row_width = row_width
        self.rows = np.zeros(max(len(self.body_records), 1) * row_width, N.RIGID_CANDIDATE_DTYPE)
        self.row_counts = np.zeros((max(len(self.body_records), 1), 2), np.uint32)
        self.contact_corrections = np.zeros(max(len(self.body_records), 1) * row_width, N.RIGID_CORRECTION_DTYPE)
        self.overflow_words = np.zeros(2, np.uint32)
        self.segments = np.zeros(0, N.SEGMENT_DTYPE) if segments is None else np.array(segments, N.SEGMENT_DTYPE)
        self.bubble_count = bubble_count
        if joints is not None and len(joints.records):
            self.joint_records = np.array(joints.records, N.RIGID_JOINT_DTYPE)
            self.references = np.ascontiguousarray(joints.references, np.uint32)
            self.ranges = np.ascontiguousarray(joints.ranges, np.uint32)
            self.partners = np.ascontiguousarray(joints.partners, np.uint64)
        else:
            self.joint_records = np.zeros(0, N.RIGID_JOINT_DTYPE)
            self.references = np.zeros((0, 2), np.uint32)
            self.ranges = None
            self.partners = np.zeros(0, np.uint64)
        self.corrections = np.zeros(len(self.joint_records), N.RIGID_CORRECTION_DTYPE)
        self.wall_records = np.zeros(len(self.body_records), N.RIGID_WALL_DTYPE)
        self.safety_word = np.zeros(1, np.uint32)

    @staticmethod
    def _p(a):
        return None if a is None else C.c_void_p(a.ctypes.data)

    def predict(self, dt: float) -> None:
        self.wall_records[:] = np.zeros(1, N.RIGID_WALL_DTYPE)
        library().bpo_rigid_predict(self._p(self.body_records), len(self.body_records), self._p(self.vertices),
                                    self.vertices.shape[0], self._p(self.segments), len(self.segments),
                                    self.bubble_count, dt, self._p(self.ranges), self._p(self.partners),
                                    self.partners.size, self._p(self.wall_records), self._p(self.safety_word))

    def solve_joints(self, dt: float, rounds: int = 8, iteration_count: int = 8) -> None:
        if not len(self.joint_records):
            return
        library().bpo_rigid_solve_joints(self._p(self.body_records), len(self.body_records),
                                         self._p(self.joint_records), len(self.joint_records),
                                         self._p(self.corrections), self._p(self.references),
                                         self.references.shape[0], self._p(self.ranges), self.bubble_count, dt,
                                         iteration_count, rounds, self._p(self.safety_word))

    def finish(self, region) -> None:
        r = np.asarray(region, np.float32)
        library().bpo_rigid_finish(self._p(self.body_records), len(self.body_records), self._p(self.vertices),
                                   self.vertices.shape[0], self._p(r), self._p(self.safety_word))

    def _geometry(self):
        return (self._p(self.vertices), self.vertices.shape[0], self._p(self.triangles), self.triangles.shape[0])

    def body_candidates(self) -> None:
        library().bpo_rigid_body_candidates(self._p(self.body_records), len(self.body_records), self.bubble_count,
                                            self._p(self.ranges), self._p(self.partners), self.partners.size,
                                            self.row_width, self._p(self.rows), self._p(self.row_counts),
                                            self._p(self.overflow_words))

    def ccd(self) -> None:
        library().bpo_rigid_ccd(self._p(self.body_records), len(self.body_records), *self._geometry(),
                                self._p(self.rows), self._p(self.row_counts), self.row_width, self._p(self.safety_word))

    def solve_contacts(self) -> None:
        library().bpo_rigid_solve_contacts(self._p(self.body_records), len(self.body_records), *self._geometry(),
                                           self._p(self.rows), self._p(self.row_counts), self.row_width,
                                           self._p(self.contact_corrections), self._p(self.safety_word))

    def guard_walls(self) -> None:
        library().bpo_rigid_guard_walls(self._p(self.body_records), len(self.body_records), *self._geometry(),
                                        self.bubble_count, self._p(self.ranges), self._p(self.partners),
                                        self.partners.size, self._p(self.safety_word))

    def step_without_contacts(self, dt: float, region, iterations: int = 8) -> None:
        self.predict(dt)
        self.solve_joints(dt, iterations, iterations)
        self.finish(region)

    def overflow_counts(self):
        return self.overflow_words.copy()

    def step(self, dt: float, region, iterations: int = 8) -> None:
        """The reference's rigid step order: predict, body-pair rows, CCD, `iterations` rounds of {contacts, one
        joint round, wall guard}, finish."""
        self.predict(dt)
        self.body_candidates()
        self.ccd()
        for _ in range(iterations):
            self.solve_contacts()
            self.solve_joints(dt, 1, iterations)
            self.guard_walls()
        self.finish(region)

    def candidates(self) -> np.ndarray:
        return self.rows.reshape(-1, self.row_width).copy(), self.row_counts.copy()

    def bodies(self) -> np.ndarray:
        return self.body_records.copy()

    def joints(self) -> np.ndarray:
        return self.joint_records.copy()

    def walls(self) -> np.ndarray:
        return self.wall_records.copy()

    def safety(self) -> int:
        return int(self.safety_word[0])
