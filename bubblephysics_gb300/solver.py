"""Native solver handles over the C ABI: Context, World (plain single world), Batch (many independent worlds).

World mirrors the reference's persistent NativeMetalSolver + executeFrame seam
(Sources/BubblePhysicsNativeMetal/NativeMetalSolver.swift:380-1218): state stays resident on the GPU between steps,
each step returns a report, a failed step publishes nothing and stops the world.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .spec import PackedInput, WorldSpec


class Context:
    """One CUDA device + one stream (bp_context)."""

    def __init__(self, device: int = 0):
        self.lib = N.library()
        handle = C.c_void_p()
        N.check(self.lib.bp_context_create(device, 0, C.byref(handle)), "bp_context_create")
        self.handle = handle
        self.device = device

    def close(self):
        if self.handle:
            self.lib.bp_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def contact_law(self, mode: int, cases: np.ndarray) -> np.ndarray:
        """Contact law on the device (known-answer tests): cases (n, 8) float32 -> (n, 8) float32."""
        cases = np.ascontiguousarray(cases, np.float32).reshape(-1, 8)
        out = np.zeros_like(cases)
        N.check(self.lib.bp_device_contact_law(self.handle, mode, N.ptr(cases, C.c_float), N.ptr(out, C.c_float),
                                               cases.shape[0]), "bp_device_contact_law")
        return out


_default_context: Context | None = None


def default_context() -> Context:
    global _default_context
    if _default_context is None:
        _default_context = Context(0)
    return _default_context


class World:
    """A single world stepped by the plain per-world launch path."""

    def __init__(self, spec: WorldSpec, context: Context | None = None):
        self.ctx = context or default_context()
        self.lib = self.ctx.lib
        self.spec = spec
        packed = PackedInput(spec)
        handle = C.c_void_p()
        N.check(self.lib.bp_world_create(self.ctx.handle, C.byref(packed.desc), C.byref(packed.input), C.byref(handle)),
                "bp_world_create")
        self.handle = handle
        self.n = spec.bubble_count

    def close(self):
        if self.handle:
            self.lib.bp_world_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_injection(self, substep: int, position):
        d = N.WorldDiagnostics()
        d.inject_substep = substep
        d.inject_position[:] = [float(position[0]), float(position[1])]
        N.check(self.lib.bp_world_set_diagnostics(self.handle, C.byref(d)), "bp_world_set_diagnostics")

    def step(self, steps: int = 1) -> tuple[int, np.ndarray]:
        """Advances `steps` steps; returns (status, reports[steps]). Stops at the first failed step."""
        reports = np.zeros(max(steps, 1), N.REPORT_DTYPE)
        status = self.lib.bp_world_step(self.handle, steps, C.c_void_p(reports.ctypes.data))
        if status in (N.E_CUDA, N.E_ALLOC, N.E_INVALID, N.E_INFLIGHT, N.E_UNAVAILABLE):
            raise N.NativeError(status, "bp_world_step")
        return status, reports[:steps]

    def write_bubbles(self, bubbles: np.ndarray):
        b = np.ascontiguousarray(bubbles, N.BUBBLE_DTYPE)
        N.check(self.lib.bp_world_write_bubbles(self.handle, C.c_void_p(b.ctypes.data), b.shape[0]),
                "bp_world_write_bubbles")

    def bubbles(self) -> np.ndarray:
        out = np.zeros(self.n, N.BUBBLE_DTYPE)
        count = C.c_uint32()
        N.check(self.lib.bp_world_read_bubbles(self.handle, C.c_void_p(out.ctypes.data), self.n, C.byref(count)),
                "bp_world_read_bubbles")
        return out

    def _read(self, fn, dtype, where):
        count = C.c_uint32()
        N.check(fn(self.handle, None, 0, C.byref(count)), where)
        out = np.zeros(count.value, dtype)
        if count.value:
            N.check(fn(self.handle, C.c_void_p(out.ctypes.data), count.value, C.byref(count)), where)
        return out

    def contacts(self) -> np.ndarray:
        return self._read(self.lib.bp_world_read_contacts, N.CONTACT_DTYPE, "bp_world_read_contacts")

    def contact_events(self, interested, removed=(), step: float | None = None, extra=None,
                       capacity: int = 0) -> np.ndarray:
        """Contact began / ended events of the last step, compacted on the device (bp_world_contact_events):
        interested / removed are object ids, extra a CONTACT_DTYPE array of records the step does not make (e.g.
        bubble-body contacts), step the step's duration (the world's time step by default)."""
        ids = np.ascontiguousarray(np.asarray(list(interested), np.int64))
        gone = np.ascontiguousarray(np.asarray(list(removed), np.int64))
        more = np.zeros(0, N.CONTACT_DTYPE) if extra is None else np.ascontiguousarray(extra, N.CONTACT_DTYPE)
        dt = float(self.spec.time_step if step is None else step)
        cap = capacity or max(64, 2 * (len(self.contacts()) + more.size + self.contact_history().shape[0]))
        out = np.zeros(cap, N.CONTACT_EVENT_DTYPE)
        count = C.c_uint32()
        N.check(self.lib.bp_world_contact_events(self.handle, N.ptr(ids), ids.size, N.ptr(gone), gone.size,
                                                 N.ptr(more), more.size, dt, C.c_void_p(out.ctypes.data), cap,
                                                 C.byref(count)), "bp_world_contact_events")
        return out[:min(count.value, cap)]

    def set_contact_history(self, pairs):
        arr = np.ascontiguousarray(np.asarray(pairs, np.int64).reshape(-1, 2))
        N.check(self.lib.bp_world_set_contact_history(self.handle, N.ptr(arr), arr.shape[0]),
                "bp_world_set_contact_history")

    def contact_history(self) -> np.ndarray:
        count = C.c_uint32()
        N.check(self.lib.bp_world_read_contact_history(self.handle, None, 0, C.byref(count)),
                "bp_world_read_contact_history")
        out = np.zeros((count.value, 2), np.int64)
        if count.value:
            N.check(self.lib.bp_world_read_contact_history(self.handle, C.c_void_p(out.ctypes.data), count.value,
                                                           C.byref(count)), "bp_world_read_contact_history")
        return out

    def candidates(self) -> np.ndarray:
        return self._read(self.lib.bp_world_read_candidates, N.KEY_DTYPE, "bp_world_read_candidates")

    def cells(self) -> np.ndarray:
        out = np.zeros((self.n, 2), np.int64)
        count = C.c_uint32()
        N.check(self.lib.bp_world_read_cells(self.handle, C.c_void_p(out.ctypes.data), self.n, C.byref(count)),
                "bp_world_read_cells")
        return out

    def substeps(self) -> np.ndarray:
        return self._read(self.lib.bp_world_read_substeps, np.float32, "bp_world_read_substeps")

    def contours(self, max_edge: float = 8.0, surface_tension: float = 20.0, clearance: float = 1e-4, stride: int = 0):
        """Contours of the published state built on the device (bp_world_contours): points (n, stride, 2), counts (n,),
        level (n, stride), shape (n, 6: largest deficit, effective radius, bounds) and the kernel's device ms."""
        cfg = N.ContourConfig(max_edge, surface_tension, clearance, stride)
        used = C.c_uint32()
        N.check(self.lib.bp_world_contours(self.handle, C.byref(cfg), None, None, None, None, C.byref(used), None),
                "bp_world_contours")
        s = used.value
        points = np.zeros((self.n, s, 2), np.float32)
        counts = np.zeros(self.n, np.uint32)
        level = np.zeros((self.n, s), np.float32)
        shape = np.zeros((self.n, 6), np.float32)
        ms = C.c_float()
        N.check(self.lib.bp_world_contours(self.handle, C.byref(cfg), C.c_void_p(points.ctypes.data),
                                           C.c_void_p(counts.ctypes.data), C.c_void_p(level.ctypes.data),
                                           C.c_void_p(shape.ctypes.data), C.byref(used), C.byref(ms)), "bp_world_contours")
        return points, counts, level, shape, ms.value

    def hit_test(self, points, max_edge: float = 8.0, surface_tension: float = 20.0, clearance: float = 1e-4):
        """Hit test of query points on the published state (bp_world_hit_test): ids, layers, found."""
        q = np.ascontiguousarray(points, np.float32).reshape(-1, 2)
        ids = np.zeros(q.shape[0], np.int64)
        layers = np.zeros(q.shape[0], np.int32)
        found = np.zeros(q.shape[0], np.uint32)
        cfg = N.ContourConfig(max_edge, surface_tension, clearance, 0)
        N.check(self.lib.bp_world_hit_test(self.handle, C.byref(cfg), C.c_void_p(q.ctypes.data), q.shape[0],
                                           C.c_void_p(ids.ctypes.data), C.c_void_p(layers.ctypes.data),
                                           C.c_void_p(found.ctypes.data)), "bp_world_hit_test")
        return ids, layers, found

    def set_sensors(self, sensors, vertices=None, state=None, allowed=None):
        """Sensors (a list of N.Sensor) with their polygon vertices ((m, 2) float32) and, optionally, per pair (uint8,
        sensors x (bubbles, then bodies)) the overlap state to start from and which pairs the sensors' object filters
        allow: from the next step on, each step lists the bubbles and bodies that entered or left them."""
        arr = (N.Sensor * max(len(sensors), 1))(*sensors)
        v = np.ascontiguousarray(np.zeros((0, 2)) if vertices is None else vertices, np.float32).reshape(-1, 2)
        st = None if state is None else np.ascontiguousarray(state, np.uint8)
        ok = None if allowed is None else np.ascontiguousarray(allowed, np.uint8)
        N.check(self.lib.bp_world_set_sensors(self.handle, C.cast(arr, C.c_void_p), len(sensors),
                                              C.c_void_p(v.ctypes.data), v.shape[0],
                                              None if ok is None else C.c_void_p(ok.ctypes.data),
                                              None if st is None else C.c_void_p(st.ctypes.data)),
                "bp_world_set_sensors")

    def sensor_events(self) -> np.ndarray:
        return self._read(self.lib.bp_world_read_sensor_events, N.SENSOR_EVENT_DTYPE, "bp_world_read_sensor_events")

    def rigid_keys(self) -> np.ndarray:
        """Sorted LBVH keys (Morton code << 32 | leaf) of the last step; empty when the step used no tree."""
        return self._read(self.lib.bp_world_read_rigid_keys, np.uint64, "bp_world_read_rigid_keys")


class Batch:
    """Many independent worlds stepped together: one fused launch per size class and step (or, with
    per_world_launch=True, the plain path: one launch per world, one after another)."""

    def __init__(self, specs: list[WorldSpec], context: Context | None = None, *, per_world_launch=False,
                 use_graph=True, autotune=False, threads_per_world=0, warp_world_max=0, group_width=0, staging=True):
        self.ctx = context or default_context()
        self.lib = self.ctx.lib
        self.specs = specs
        packed = [PackedInput(s) for s in specs]
        descs = (N.WorldDesc * len(specs))(*[p.desc for p in packed])
        inputs = (N.WorldInput * len(specs))(*[p.input for p in packed])
        cfg = N.BatchConfig()
        cfg.flags = (N.BATCH_PER_WORLD_LAUNCH if per_world_launch else 0) | (N.BATCH_USE_GRAPH if use_graph else 0) | \
                    (N.BATCH_AUTOTUNE if autotune else 0) | (0 if staging else N.BATCH_NO_STAGING)
        cfg.threads_per_world = threads_per_world
        cfg.warp_world_max = warp_world_max
        cfg.group_width = group_width
        handle = C.c_void_p()
        N.check(self.lib.bp_batch_create(self.ctx.handle, len(specs), descs, inputs, C.byref(cfg), C.byref(handle)),
                "bp_batch_create")
        self.handle = handle
        self.sizes = np.array([s.bubble_count for s in specs], np.int64)
        self.total_bubbles = int(self.sizes.sum())

    def close(self):
        if self.handle:
            self.lib.bp_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, steps: int = 1) -> tuple[int, np.ndarray]:
        reports = np.zeros(len(self.specs), N.REPORT_DTYPE)
        status = self.lib.bp_batch_step(self.handle, steps, C.c_void_p(reports.ctypes.data))
        if status in (N.E_CUDA, N.E_ALLOC, N.E_INVALID, N.E_INFLIGHT, N.E_UNAVAILABLE, N.E_TIMEOUT):
            raise N.NativeError(status, "bp_batch_step")
        return status, reports

    def counters(self) -> tuple[int, int, int]:
        a, b, c = C.c_uint64(), C.c_uint64(), C.c_uint64()
        N.check(self.lib.bp_batch_counters(self.handle, C.byref(a), C.byref(b), C.byref(c)), "bp_batch_counters")
        return a.value, b.value, c.value

    def bubbles(self, world: int) -> np.ndarray:
        n = int(self.sizes[world])
        out = np.zeros(n, N.BUBBLE_DTYPE)
        count = C.c_uint32()
        N.check(self.lib.bp_batch_read_bubbles(self.handle, world, C.c_void_p(out.ctypes.data), n, C.byref(count)),
                "bp_batch_read_bubbles")
        return out

    def write_state(self, center_velocity: np.ndarray):
        """Bulk host -> device write of (center.xy, velocity.xy) float32 for every bubble, worlds in order."""
        assert center_velocity.dtype == np.float32 and center_velocity.flags["C_CONTIGUOUS"]
        N.check(self.lib.bp_batch_write_state(self.handle, C.c_void_p(center_velocity.ctypes.data), self.total_bubbles),
                "bp_batch_write_state")

    def read_state(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.zeros((self.total_bubbles, 4), np.float32)
        N.check(self.lib.bp_batch_read_state(self.handle, C.c_void_p(out.ctypes.data), self.total_bubbles),
                "bp_batch_read_state")
        return out

    def adjacency_entries(self) -> int:
        v = C.c_uint64()
        N.check(self.lib.bp_batch_adjacency_entries(self.handle, C.byref(v)), "bp_batch_adjacency_entries")
        return v.value

    def tuning(self) -> dict:
        out = (C.c_uint32 * 6)()
        N.check(self.lib.bp_batch_tuning(self.handle, out, 6), "bp_batch_tuning")
        return dict(zip(["threads", "warp_max", "blocks", "cta_worlds", "warp_worlds", "group_width"], list(out)))


def static_polygon_edges(points, first_id: int, owner_id: int | None = None) -> np.ndarray:
    """One-sided edges of a static polygon (NativeStaticPolygonEdges.segments) computed by the native library."""
    lib = N.library()
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 2)
    count = C.c_uint32()
    cap = max(pts.shape[0], 1)
    out = np.zeros(cap, N.SEGMENT_DTYPE)
    N.check(lib.bp_static_polygon_edges(N.ptr(pts, C.c_float), pts.shape[0], first_id, owner_id or 0,
                                        1 if owner_id is not None else 0,
                                        C.cast(out.ctypes.data, C.POINTER(N.Segment)), cap, C.byref(count)),
            "bp_static_polygon_edges")
    return out[:count.value]


COMPLETION_DTYPE = np.dtype([("request_id", "<u8"), ("world", "<u4"), ("status", "<i4"), ("steps", "<u4"),
                             ("substeps", "<u4"), ("submitted_s", "<f8"), ("completed_s", "<f8"),
                             ("report", N.REPORT_DTYPE)])
assert COMPLETION_DTYPE.itemsize == C.sizeof(N.ServerCompletion)


class Server:
    """Serving loop over resident worlds (bp_server): step requests for any registered world, batched continuously
    onto the device under a device-memory budget, idle worlds evicted to pinned host memory in LRU order.
    per_world=True serves every world step with its own launch, one at a time (the plain per-world path)."""

    def __init__(self, max_worlds: int, context: Context | None = None, *, hbm_budget_bytes: int = 0,
                 max_batch_worlds: int = 0, streams: int = 0, threads_per_world: int = 0, warp_world_max: int = 0,
                 group_width: int = 0, per_world: bool = False):
        self.ctx = context or default_context()
        self.lib = self.ctx.lib
        cfg = N.ServerConfig()
        cfg.hbm_budget_bytes = hbm_budget_bytes
        cfg.max_worlds = max_worlds
        cfg.max_batch_worlds = max_batch_worlds
        cfg.streams = streams
        cfg.threads_per_world = threads_per_world
        cfg.warp_world_max = warp_world_max
        cfg.group_width = group_width
        cfg.flags = N.SERVER_PER_WORLD if per_world else 0
        handle = C.c_void_p()
        N.check(self.lib.bp_server_create(self.ctx.handle, C.byref(cfg), C.byref(handle)), "bp_server_create")
        self.handle = handle
        self.sizes: list[int] = []

    def close(self):
        if self.handle:
            self.lib.bp_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_world(self, spec: WorldSpec) -> int:
        packed = PackedInput(spec)
        index = C.c_uint32()
        N.check(self.lib.bp_server_add_world(self.handle, C.byref(packed.desc), C.byref(packed.input), C.byref(index)),
                "bp_server_add_world")
        self.sizes.append(spec.bubble_count)
        return index.value

    def submit(self, world: int, steps: int = 1) -> int:
        rid = C.c_uint64()
        N.check(self.lib.bp_server_submit(self.handle, world, steps, C.byref(rid)), "bp_server_submit")
        return rid.value

    def progress(self, wait_us: int = 0) -> int:
        done = C.c_uint32()
        N.check(self.lib.bp_server_progress(self.handle, wait_us, C.byref(done)), "bp_server_progress")
        return done.value

    def poll(self) -> np.ndarray:
        """Every finished request not taken yet, oldest first."""
        count = C.c_uint32()
        N.check(self.lib.bp_server_poll(self.handle, None, 0, C.byref(count)), "bp_server_poll")
        out = np.zeros(count.value, COMPLETION_DTYPE)
        if count.value:
            N.check(self.lib.bp_server_poll(self.handle, C.c_void_p(out.ctypes.data), count.value, C.byref(count)),
                    "bp_server_poll")
        return out[: count.value]

    def pending(self) -> tuple[int, int]:
        waiting, inflight = C.c_uint32(), C.c_uint32()
        N.check(self.lib.bp_server_pending(self.handle, C.byref(waiting), C.byref(inflight)), "bp_server_pending")
        return waiting.value, inflight.value

    def drain(self, wait_us: int = 200, max_rounds: int = 10_000_000) -> np.ndarray:
        """Runs the loop until every submitted request has finished; returns their completions."""
        done = []
        for _ in range(max_rounds):
            if self.progress(wait_us):
                done.append(self.poll())
            if self.pending() == (0, 0):
                break
        done.append(self.poll())
        return np.concatenate(done) if done else np.zeros(0, COMPLETION_DTYPE)

    def bubbles(self, world: int) -> np.ndarray:
        n = self.sizes[world]
        out = np.zeros(n, N.BUBBLE_DTYPE)
        count = C.c_uint32()
        N.check(self.lib.bp_server_read_bubbles(self.handle, world, C.c_void_p(out.ctypes.data), n, C.byref(count)),
                "bp_server_read_bubbles")
        return out

    def stats(self) -> dict:
        st = N.ServerStats()
        N.check(self.lib.bp_server_read_stats(self.handle, C.byref(st)), "bp_server_read_stats")
        return {name: getattr(st, name) for name, _ in st._fields_}

    def clock(self) -> float:
        return self.lib.bp_server_clock()
