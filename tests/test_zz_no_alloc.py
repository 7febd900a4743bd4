"""The allocation-free entry point bp_world_step_noalloc, for callers that cannot allocate device memory while they
step (a host framework that owns all device allocations through its own pool, a real-time thread, a process with a
fixed memory reservation). The test owns the device buffers (allocated by torch here, as such a caller's pool would),
steps the plain world twice in a row through the C ABI and checks every result against the regular entry point
(bp_world_create + bp_world_step) bit for bit. This file is collected last so a failure here leaves every other test
already run; it passes alone in a fresh process as well."""
import ctypes as C
import dataclasses

import numpy as np
import pytest

from bubblephysics_gb300 import _native as N
from bubblephysics_gb300 import scenes
from bubblephysics_gb300.solver import World
from bubblephysics_gb300.spec import WorldSpec, make_bubbles

pytestmark = pytest.mark.gpu


def noalloc_call(torch, desc, dev_bubbles, n, dev_segments, s, steps):
    lib = N.library()
    dev_reports = torch.zeros(steps * 96, dtype=torch.uint8, device="cuda")
    status = lib.bp_world_step_noalloc(C.byref(desc), C.c_void_p(dev_bubbles.data_ptr()), n,
                                       C.c_void_p(dev_segments.data_ptr()) if s else None, s, steps,
                                       C.c_void_p(dev_reports.data_ptr()), None)
    torch.cuda.synchronize()
    assert status == N.OK, N.STATUS_NAMES.get(status, status)
    return dev_reports.cpu().numpy().view(N.REPORT_DTYPE)


def on_device(torch, records):
    return torch.from_numpy(np.ascontiguousarray(records).view(np.uint8).copy()).cuda()


def same_as_regular(torch, ctx, spec, calls, report_keys):
    """Steps `spec` through the allocation-free entry point (one call per entry of `calls`, each that many steps)
    and through bp_world_create + bp_world_step with the rigid tree off (the allocation-free step always takes the
    brute-force rigid loops); returns (allocation-free reports, regular reports) of every call."""
    n, s = spec.bubble_count, len(spec.segments)
    regular = World(dataclasses.replace(spec, flags=spec.flags | N.WORLD_NO_RIGID_TREE), ctx)
    desc = spec.desc()
    dev_bubbles, dev_segments = on_device(torch, spec.bubbles), on_device(torch, spec.segments)
    out = []
    for steps in calls:
        reports = noalloc_call(torch, desc, dev_bubbles, n, dev_segments, s, steps)
        status, expected = regular.step(steps)
        for key in report_keys:
            assert reports[key].tolist() == expected[key].tolist(), key
        got = dev_bubbles.cpu().numpy().view(N.BUBBLE_DTYPE)
        want = regular.bubbles()
        for f in ("center", "previous_center", "velocity", "rotation", "angular_velocity", "region_result"):
            assert np.array_equal(got[f], want[f]), f
        out.append((reports, expected))
    regular.close()
    return out


def test_noalloc_step_matches_the_regular_entry_point_on_two_calls_in_a_row(ctx):
    torch = pytest.importorskip("torch")
    spec = scenes.plain_world(seed=5)
    spec.candidate_limit = 32
    n, s = spec.bubble_count, len(spec.segments)
    regular = World(spec, ctx)
    desc = spec.desc()
    dev_bubbles = torch.from_numpy(spec.bubbles.view(np.uint8).copy()).cuda()
    dev_segments = torch.from_numpy(np.ascontiguousarray(spec.segments).view(np.uint8).copy()).cuda()
    for steps in (3, 2):
        reports = noalloc_call(torch, desc, dev_bubbles, n, dev_segments, s, steps)
        status, expected = regular.step(steps)
        assert status == N.OK
        for key in ("status", "substep_count", "rebuild_count", "candidate_count", "contact_count", "limiter_term",
                    "limiter_object"):
            assert reports[key].tolist() == expected[key].tolist(), key
        got = dev_bubbles.cpu().numpy().view(N.BUBBLE_DTYPE)
        want = regular.bubbles()
        for f in ("center", "previous_center", "velocity", "rotation", "angular_velocity", "region_result"):
            assert np.array_equal(got[f], want[f]), f


def test_noalloc_rejects_sizes_beyond_its_limits(ctx):
    torch = pytest.importorskip("torch")
    lib = N.library()
    spec = scenes.plain_world(seed=5)
    desc = spec.desc()
    desc.candidate_limit = 64
    buf = torch.zeros(80, dtype=torch.uint8, device="cuda")
    rep = torch.zeros(96, dtype=torch.uint8, device="cuda")
    assert lib.bp_world_step_noalloc(C.byref(desc), C.c_void_p(buf.data_ptr()), 1, None, 0, 1,
                                     C.c_void_p(rep.data_ptr()), None) == N.E_CAPACITY
    desc.candidate_limit = 32
    assert lib.bp_world_step_noalloc(C.byref(desc), C.c_void_p(buf.data_ptr()), 2000, None, 0, 1,
                                     C.c_void_p(rep.data_ptr()), None) == N.E_CAPACITY


def test_noalloc_at_its_limits_matches_the_regular_entry_point(ctx):
    """1,024 bubbles and 256 segments (the array's stated limits, where its layout and the ~110 KB shared request
    are tightest): 16 wall edges and 240 short two-sided segments on the floor line that the lowest bubbles touch."""
    torch = pytest.importorskip("torch")
    spec = scenes.batched_world(np.random.default_rng(17), 1024, world_index=0, max_bodies=0)
    assert spec.bubble_count == 1024 and len(spec.segments) == 16
    side = spec.region[2]
    floor = np.zeros(240, N.SEGMENT_DTYPE)
    floor["id"] = 5_000_000 + np.arange(240)
    floor["category"] = 1
    floor["mask"] = 0xFFFFFFFF
    x0 = np.arange(240) * (side / 240.0)
    floor["a"] = np.stack([x0, np.zeros(240)], 1)
    floor["b"] = np.stack([x0 + 0.5 * side / 240.0, np.zeros(240)], 1)
    spec = dataclasses.replace(spec, segments=np.sort(np.concatenate([spec.segments, floor]), order="id"),
                               candidate_limit=32)
    assert len(spec.segments) == 256
    calls = same_as_regular(torch, ctx, spec, (2, 2), ("status", "substep_count", "rebuild_count", "candidate_count",
                                                       "contact_count", "candidate_overflow", "limiter_term",
                                                       "limiter_object"))
    for reports, expected in calls:
        assert reports["status"].tolist() == [N.OK, N.OK]
    assert calls[0][1]["contact_count"][0] > 0


def test_noalloc_caps_contact_records_and_reports_the_overflow(ctx):
    """Each of 64 static bubbles overlaps 32 stacked floor segments: 2,048 contact records against the allocation-free
    cap of 4 per bubble + 64 = 320. The count stops at the cap, the rest is reported as overflow, and the state is the
    regular entry point's (the records feed nothing back into the step)."""
    torch = pytest.importorskip("torch")
    n, layers = 64, 32
    centers = np.stack([30.0 * np.arange(n) + 20.0, np.full(n, 50.0)], 1)
    b = make_bubbles(centers, 10.0, ids=np.arange(1, n + 1), masses=0.25, stiffness=229.0,
                     flags=N.BUBBLE_FORCE_DRIVEN | N.BUBBLE_ENABLED, static=np.ones(n, bool))
    segs = np.zeros(layers, N.SEGMENT_DTYPE)
    segs["id"] = 100 + np.arange(layers)
    segs["category"] = 1
    segs["mask"] = 0xFFFFFFFF
    y = 50.0 - 9.9 + 0.02 * np.arange(layers)
    segs["a"] = np.stack([np.full(layers, -10.0), y], 1)
    segs["b"] = np.stack([np.full(layers, 30.0 * n + 40.0), y], 1)
    spec = WorldSpec(bubbles=b, segments=segs, candidate_limit=32)
    (reports, expected), = same_as_regular(torch, ctx, spec, (1,), ("status", "substep_count", "candidate_count"))
    assert reports["status"][0] == N.OK
    assert expected["contact_count"][0] == n * layers and expected["contact_overflow"][0] == 0
    assert reports["contact_count"][0] == 4 * n + 64
    assert reports["contact_overflow"][0] == n * layers - (4 * n + 64)


def test_noalloc_rejects_unsorted_ids_in_every_report(ctx):
    """bp_world_create refuses bubbles whose ids are not strictly ascending; the allocation-free step cannot read its
    device buffer on the host, so its kernel checks and reports BP_E_INVALID for every step, leaving the bubbles."""
    torch = pytest.importorskip("torch")
    spec = scenes.plain_world(seed=5, n=64)
    spec.candidate_limit = 32
    bubbles = spec.bubbles.copy()
    bubbles["id"][[10, 11]] = bubbles["id"][[11, 10]]
    dev_bubbles, dev_segments = on_device(torch, bubbles), on_device(torch, spec.segments)
    reports = noalloc_call(torch, spec.desc(), dev_bubbles, len(bubbles), dev_segments, len(spec.segments), 3)
    assert reports["status"].tolist() == [N.E_INVALID] * 3
    assert np.array_equal(dev_bubbles.cpu().numpy().view(N.BUBBLE_DTYPE)["center"], bubbles["center"])
