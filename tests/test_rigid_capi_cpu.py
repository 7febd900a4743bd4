"""Argument checks of the rigid solver's C entries, which need no GPU: empty calls succeed without touching the
device, and NULL, misaligned or non-finite arguments are rejected with BP_E_INVALID before anything is launched.
Every call here fails or returns before a kernel launch, so the addresses below are never dereferenced."""
import ctypes as C
import math

from bubblephysics_gb300 import _native as N

ALIGNED = C.c_void_p(0x10000)     # 16-byte aligned, never dereferenced
MISALIGNED = C.c_void_p(0x10008)  # 8- but not 16-byte aligned
REGION = (C.c_float * 4)(0.0, 0.0, 1.0, 1.0)


def lib():
    return N.library()


def test_empty_calls_succeed_without_a_device():
    l = lib()
    assert l.bp_rigid_predict(None, 0, None, 0, None, 0, 0, 1 / 60, None, None, 0, None, None, None) == N.OK
    assert l.bp_rigid_solve_joints(None, 0, None, 0, None, None, 0, None, 0, 1 / 60, 8, 8, None, None) == N.OK
    assert l.bp_rigid_solve_joints(ALIGNED, 4, ALIGNED, 3, ALIGNED, ALIGNED, 1, ALIGNED, 0, 1 / 60, 8, 0, ALIGNED,
                                   None) == N.OK  # zero rounds
    assert l.bp_rigid_finish(None, 0, None, 0, REGION, None, None) == N.OK
    assert l.bp_rigid_body_candidates(None, 0, 0, None, None, 0, 16, None, None, None, None) == N.OK
    assert l.bp_rigid_ccd(None, 0, None, 0, None, 0, None, None, 16, None, None) == N.OK
    assert l.bp_rigid_solve_contacts(None, 0, None, 0, None, 0, None, None, 16, None, None, None) == N.OK
    assert l.bp_rigid_guard_walls(None, 0, None, 0, None, 0, 0, None, None, 0, None, None) == N.OK


def test_missing_arrays_are_rejected():
    l = lib()
    assert l.bp_rigid_predict(None, 4, ALIGNED, 4, None, 0, 0, 1 / 60, None, None, 0, ALIGNED, ALIGNED, None) == N.E_INVALID
    assert l.bp_rigid_predict(ALIGNED, 4, None, 4, None, 0, 0, 1 / 60, None, None, 0, ALIGNED, ALIGNED, None) == N.E_INVALID
    assert l.bp_rigid_predict(ALIGNED, 4, ALIGNED, 4, None, 2, 0, 1 / 60, None, None, 0, ALIGNED, ALIGNED, None) == N.E_INVALID
    assert l.bp_rigid_solve_joints(ALIGNED, 4, ALIGNED, 3, ALIGNED, None, 2, ALIGNED, 0, 1 / 60, 8, 8, ALIGNED,
                                   None) == N.E_INVALID
    assert l.bp_rigid_solve_joints(ALIGNED, 4, ALIGNED, 3, ALIGNED, ALIGNED, 2, None, 0, 1 / 60, 8, 8, ALIGNED,
                                   None) == N.E_INVALID
    assert l.bp_rigid_finish(ALIGNED, 4, ALIGNED, 4, None, ALIGNED, None) == N.E_INVALID
    assert l.bp_rigid_body_candidates(ALIGNED, 4, 0, None, None, 0, 0, ALIGNED, ALIGNED, ALIGNED, None) == N.E_INVALID
    assert l.bp_rigid_ccd(ALIGNED, 4, ALIGNED, 4, None, 2, ALIGNED, ALIGNED, 16, ALIGNED, None) == N.E_INVALID
    assert l.bp_rigid_solve_contacts(ALIGNED, 4, ALIGNED, 4, ALIGNED, 2, ALIGNED, ALIGNED, 16, None, ALIGNED,
                                     None) == N.E_INVALID
    assert l.bp_rigid_guard_walls(ALIGNED, 4, ALIGNED, 4, ALIGNED, 2, 0, None, None, 3, ALIGNED, None) == N.E_INVALID


def test_misaligned_records_are_rejected():
    l = lib()
    assert l.bp_rigid_predict(MISALIGNED, 4, ALIGNED, 4, None, 0, 0, 1 / 60, None, None, 0, ALIGNED, ALIGNED,
                              None) == N.E_INVALID
    assert l.bp_rigid_solve_joints(ALIGNED, 4, MISALIGNED, 3, ALIGNED, ALIGNED, 2, ALIGNED, 0, 1 / 60, 8, 8, ALIGNED,
                                   None) == N.E_INVALID
    assert l.bp_rigid_finish(MISALIGNED, 4, ALIGNED, 4, REGION, ALIGNED, None) == N.E_INVALID
    assert l.bp_rigid_body_candidates(ALIGNED, 4, 0, None, None, 0, 16, MISALIGNED, ALIGNED, ALIGNED,
                                      None) == N.E_INVALID
    assert l.bp_rigid_ccd(ALIGNED, 4, ALIGNED, 4, MISALIGNED, 2, ALIGNED, ALIGNED, 16, ALIGNED, None) == N.E_INVALID
    assert l.bp_rigid_solve_contacts(ALIGNED, 4, ALIGNED, 4, ALIGNED, 2, ALIGNED, ALIGNED, 16, MISALIGNED, ALIGNED,
                                     None) == N.E_INVALID
    assert l.bp_rigid_guard_walls(MISALIGNED, 4, ALIGNED, 4, ALIGNED, 2, 0, None, None, 0, ALIGNED, None) == N.E_INVALID


def test_non_finite_time_steps_are_rejected():
    l = lib()
    for dt in (math.nan, math.inf):
        assert l.bp_rigid_predict(ALIGNED, 4, ALIGNED, 4, None, 0, 0, dt, None, None, 0, ALIGNED, ALIGNED,
                                  None) == N.E_INVALID
        assert l.bp_rigid_solve_joints(ALIGNED, 4, ALIGNED, 3, ALIGNED, ALIGNED, 2, ALIGNED, 0, dt, 8, 8, ALIGNED,
                                       None) == N.E_INVALID


def test_record_layouts_match_the_header():
    assert N.RIGID_BODY_DTYPE.itemsize == 160 and N.RIGID_JOINT_DTYPE.itemsize == 96
    assert N.RIGID_CORRECTION_DTYPE.itemsize == 64 and N.RIGID_WALL_DTYPE.itemsize == 48
    assert N.RIGID_CANDIDATE_DTYPE.itemsize == 32
    assert N.RIGID_BODY_DTYPE.fields["limits"][1] == 144 and N.RIGID_JOINT_DTYPE.fields["state"][1] == 80
