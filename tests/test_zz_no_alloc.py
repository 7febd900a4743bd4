"""The allocation-free entry point bp_world_step_noalloc, for callers that cannot allocate device memory while they
step (a host framework that owns all device allocations through its own pool, a real-time thread, a process with a
fixed memory reservation). The test owns the device buffers (allocated by torch here, as such a caller's pool would),
steps the plain world twice in a row through the C ABI and checks every result against the regular entry point
(bp_world_create + bp_world_step) bit for bit. This file is collected last so a failure here leaves every other test
already run; it passes alone in a fresh process as well."""
import ctypes as C

import numpy as np
import pytest

from bubblephysics_gb300 import _native as N
from bubblephysics_gb300 import scenes
from bubblephysics_gb300.solver import World

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
