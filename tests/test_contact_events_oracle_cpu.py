"""The contact-event restatement (oracle bpo_contact_events, NativePublicWorld.swift:347-391) on hand-made records:
the began / ended rules, the per-pair sums, the key order, the interest and activity filters, the segment owner,
and the removal rules the world API adds. The device compaction is compared with this restatement bit for bit in
tests/test_gpu_events.py; here the restatement is also held against the world API's host version (float64 sums)."""
import numpy as np
import pytest

from bubblephysics_gb300 import _native as N
from bubblephysics_gb300 import world as W
from oracle import oracle

STEP = np.float32(1.0 / 60.0)


def record(a, b, kind=0, point=(0.0, 0.0), normal=(1.0, 0.0), penetration=0.5, impulse=0.01):
    r = np.zeros(1, N.CONTACT_DTYPE)
    r["participants"] = (a, b)
    r["kind"] = kind
    r["point"] = point
    r["normal"] = normal
    r["penetration"] = penetration
    r["impulse"] = impulse
    return r


def segments(*rows):
    s = np.zeros(len(rows), N.SEGMENT_DTYPE)
    for q, (sid, owner) in enumerate(rows):
        s[q]["id"] = sid
        s[q]["owner_id"] = owner if owner is not None else 0
        s[q]["flags"] = N.SEGMENT_HAS_OWNER if owner is not None else 0
    return s


NO_SEGMENTS = segments()


def test_began_then_nothing_then_ended():
    r = record(1, 2, point=(3.0, 4.0), normal=(0.6, 0.8), penetration=0.25, impulse=0.5)
    ev, hist = oracle.contact_events(r, NO_SEGMENTS, {1}, [], step=STEP)
    assert ev["kind"].tolist() == [0] and ev["objects"].tolist() == [[1, 2]]
    w = np.float32(0.25) + np.float32(1e-4)
    assert ev["point"][0].tolist() == [np.float32(3.0 * w) / w, np.float32(4.0 * w) / w]
    assert ev["impulse"][0] == np.float32(0.5) / STEP
    assert np.allclose(ev["normal"][0], [0.6, 0.8])
    assert hist.tolist() == [[1, 2]]
    ev2, hist2 = oracle.contact_events(r, NO_SEGMENTS, {1}, hist, step=STEP)
    assert ev2.size == 0 and hist2.tolist() == [[1, 2]]
    ev3, hist3 = oracle.contact_events(np.zeros(0, N.CONTACT_DTYPE), NO_SEGMENTS, {1}, hist2, step=STEP)
    assert ev3["kind"].tolist() == [1] and ev3["objects"].tolist() == [[1, 2]] and hist3.size == 0


def test_pair_key_orders_ids_and_flips_the_normal():
    ev, _ = oracle.contact_events(record(9, 4, normal=(1.0, 0.0)), NO_SEGMENTS, {9}, [], step=STEP)
    assert ev["objects"].tolist() == [[4, 9]] and ev["normal"][0].tolist() == [-1.0, 0.0]


def test_keys_ascend_as_unsigned_values():
    recs = np.concatenate([record(5, -3), record(5, 7), record(1, 5)])
    ev, hist = oracle.contact_events(recs, NO_SEGMENTS, {5}, [], step=STEP)
    assert ev["objects"].tolist() == [[1, 5], [5, 7], [5, -3]]  # -3 is the largest unsigned value
    assert hist.tolist() == [[1, 5], [5, 7], [5, -3]]


def test_segment_records_merge_into_their_owner_with_the_normal_reversed():
    segs = segments((100, 900), (101, 900), (102, None))
    recs = np.concatenate([record(1, 100, kind=1, point=(0.0, 0.0), normal=(0.0, 1.0), penetration=0.1),
                           record(1, 101, kind=1, point=(2.0, 0.0), normal=(0.0, 1.0), penetration=0.3),
                           record(1, 102, kind=1, point=(9.0, 9.0))])  # no owner: not reported
    ev, hist = oracle.contact_events(recs, segs, {1}, [], step=STEP)
    assert ev["objects"].tolist() == [[1, 900]] and hist.tolist() == [[1, 900]]
    w0, w1 = np.float32(0.1) + np.float32(1e-4), np.float32(0.3) + np.float32(1e-4)
    px = (np.float32(0.0) * w0 + np.float32(2.0) * w1) / (w0 + w1)
    assert ev["point"][0][0] == np.float32(px)
    assert ev["normal"][0].tolist() == [0.0, -1.0]  # from the bubble (key first) towards the owner


def test_interest_and_activity_filters():
    recs = np.concatenate([record(1, 2), record(3, 4, penetration=0.0, impulse=0.0),
                           record(5, 6, penetration=-0.001, impulse=0.2)])
    ev, _ = oracle.contact_events(recs, NO_SEGMENTS, {2, 3, 6}, [], step=STEP)
    assert ev["objects"].tolist() == [[1, 2], [5, 6]]
    ev, _ = oracle.contact_events(recs, NO_SEGMENTS, set(), [], step=STEP)
    assert ev.size == 0


def test_removal_rules():
    hist = [[1, 2], [3, 4], [5, 6]]
    recs = np.concatenate([record(1, 2), record(5, 6)])
    ev, nxt = oracle.contact_events(recs, NO_SEGMENTS, {1, 3, 5}, hist, removed={2, 3, 4}, step=STEP)
    # (1,2) lost object 2: ended; (3,4) lost both: nothing; (5,6) continues
    assert ev["kind"].tolist() == [1] and ev["objects"].tolist() == [[1, 2]]
    assert nxt.tolist() == [[5, 6]]


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_restatement_agrees_with_the_world_api_host_version(seed):
    rng = np.random.default_rng(seed)
    ids = [1, 2, 3, 4, 5, -7, 900]
    segs = segments((100, 900), (101, 900), (102, 5))
    recs = []
    for _ in range(40):
        a = int(rng.choice(ids[:6]))
        if rng.random() < 0.3:
            recs.append(record(a, int(rng.choice([100, 101, 102])), kind=1, point=rng.normal(size=2),
                               normal=rng.normal(size=2), penetration=rng.uniform(-0.1, 1), impulse=rng.uniform(0, 1)))
        else:
            b = int(rng.choice([i for i in ids[:6] if i != a]))
            recs.append(record(a, b, point=rng.normal(size=2), normal=rng.normal(size=2),
                               penetration=rng.uniform(-0.1, 1), impulse=rng.uniform(0, 1) * (rng.random() < 0.5)))
    recs = np.concatenate(recs)
    interested = {1, 3, -7}
    history = {W._pair_key(1, 2), W._pair_key(4, 5), W._pair_key(3, 900)}
    owners = {100: 900, 101: 900, 102: 5}
    host_events, host_next = W.contact_transitions(recs, owners, interested, set(history), float(STEP), set())
    ev, nxt = oracle.contact_events(recs, segs, interested, [list(k) for k in history], step=STEP)
    assert [e.kind for e in host_events] == ["contactBegan" if k == 0 else "contactEnded" for k in ev["kind"]]
    assert [list(e.objects) for e in host_events] == ev["objects"].tolist()
    for e, o in zip(host_events, ev):
        if o["kind"] == 0:
            assert np.allclose(e.point, o["point"], rtol=1e-5, atol=1e-5)
            assert np.allclose(e.normal, o["normal"], rtol=1e-5, atol=1e-5)
            assert np.isclose(e.impulse, o["impulse"], rtol=1e-5)
    assert sorted(map(list, host_next)) == sorted(nxt.tolist())
