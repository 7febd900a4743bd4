"""NativeSolverInputTests.swift:17-49 restated on the oracle through the records of the C ABI that replaces the
reference's NativeSolverInput seam (NativeSolverInput.swift): a neutral bubble advances and publishes its contour, two
overlapping bubbles give one bubble-bubble contact, and a bubble meeting a static segment gives a segment contact that
names the segment. The scenes are the reference test's: time step 0.5, no damping, radius 1, mass 1, contact stiffness
0 (NativeSolverBubble's default)."""
import numpy as np

from bubblephysics_gb300 import _native as N
from bubblephysics_gb300.spec import WorldSpec, make_bubbles
from oracle.oracle import OracleWorld


def neutral_world(centers, velocities=None, ids=None, segments=None):
    b = make_bubbles(centers, 1.0, ids=ids or list(range(1, len(centers) + 1)),
                     velocities=velocities if velocities is not None else np.zeros((len(centers), 2)), masses=1.0,
                     stiffness=0.0)
    segments = segments if segments is not None else np.zeros(0, N.SEGMENT_DTYPE)
    return OracleWorld(WorldSpec(bubbles=b, segments=segments, time_step=0.5))


def test_neutral_bubble_advances_and_publishes_its_contour():
    """NativeSolverInputTests.swift:17-28."""
    w = neutral_world([(0.0, 0.0)], velocities=[(2.0, 0.0)], ids=[7])
    status, rep = w.step(1)
    assert status == N.OK
    b = w.bubbles()
    assert list(b["id"]) == [7]
    assert abs(b["center"][0][0] - 1) <= 1e-5
    assert abs(b["previous_center"][0][0]) <= 1e-5
    _, counts, _, shape = w.contours()
    assert counts[0] >= 32
    assert abs(shape[0][1] - 1) <= 1e-5  # the effective radius
    assert len(w.contacts()) == 0 and rep[0]["contact_count"] == 0


def test_overlapping_bubbles_produce_a_bubble_contact():
    """NativeSolverInputTests.swift:30-40."""
    w = neutral_world([(0.0, 0.0), (1.5, 0.0)])
    status, rep = w.step(1)
    assert status == N.OK  # no non-finite state
    contacts = w.contacts()
    assert len(contacts) >= 1
    assert contacts[0]["kind"] == 0
    assert set(map(int, contacts[0]["participants"])) == {1, 2}
    assert rep[0]["contact_count"] == len(contacts)


def test_bubble_meets_a_static_segment_as_a_segment_contact():
    """NativeSolverInputTests.swift:42-49."""
    wall = np.zeros(1, N.SEGMENT_DTYPE)
    wall[0]["id"], wall[0]["a"], wall[0]["b"] = 40, (-5.0, 0.5), (5.0, 0.5)
    wall[0]["category"], wall[0]["mask"] = 1, 0xFFFFFFFF
    w = neutral_world([(0.0, 0.0)], segments=wall)
    assert w.step(1)[0] == N.OK
    contacts = w.contacts()
    assert len(contacts) >= 1
    assert contacts[0]["kind"] == 1
    assert int(contacts[0]["participants"][1]) == 40
