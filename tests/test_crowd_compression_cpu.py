"""The soft crowd of CrowdCompressionTests.swift:81-112, through the world API on a stand-in device world that forwards
to the oracle. `run_crowd` follows CrowdScene.runCrowd (CrowdSceneSupport.swift:257-326): every 0.25 s one bubble with
a target radius drawn from [12, 48] is placed at a random interior point of the 360 x 640 frame of static walls at 10 %
of that radius (mass r^2 / 400 of the target radius) and grows to full radius in 1 s through a ParameterTransition; a
point refused with invalidPlacement is drawn again at once. The crowd grows until the area balance B = sum(pi r^2) /
(360 * 640) reaches the target and then runs `extra_steps` more steps. Every step stays accepted, no bubble leaves the
region or the frame, and the mean ratio of effective to target radius over the last 60 steps falls below 1; it is
lower for the softer material and for the denser crowd. The reference draws its points with its own seeded generator;
these crowds are seeded synthetic data under the same rules."""
import math

import numpy as np
import pytest

from bubblephysics_gb300 import world as W
from bubblephysics_gb300.world import (BubbleDescriptor, BubbleWorld, EventInterest, ParameterTransition,
                                       PhysicsMaterial, Polygon, RigidBodyDescriptor, WorldConfiguration,
                                       WorldTransaction, TransactionRejectionReason)
from test_world_api_oracle_cpu import OracleBackedWorld

HALF = (180.0, 320.0)                 # CrowdScene.interiorHalfSize
THICK = 48.0                          # CrowdScene.wallThickness
AREA = 360.0 * 640.0                  # CrowdScene.interiorArea
STEP = 1.0 / 60                       # CrowdScene.step
FRAME_TOLERANCE = 1e-3                # CrowdScene.frameTolerance
LAST_SECOND = 60                      # CrowdScene.lastSecondSteps
INTEREST = frozenset({EventInterest.DID_ADD, EventInterest.DID_EXIT_SIMULATION_REGION})  # CrowdScene.bubble


@pytest.fixture(autouse=True)
def oracle_backed(monkeypatch):
    monkeypatch.setattr(W, "World", OracleBackedWorld)
    monkeypatch.setattr(W, "default_context", lambda: None)


def soft_material(base, reference_radius=20.0):
    """CrowdScene.softBubblePhysics: K_c = r_ref / c0 in float."""
    return PhysicsMaterial(float(np.float32(reference_radius) / np.float32(base)), 0.0)


def make_world(material):
    """CrowdScene.makeWorld: the frame of four static rectangles and the bubble material, accepted in one step."""
    hx, hy = HALF
    ox, oy = hx + THICK, hy + THICK
    world = BubbleWorld(WorldConfiguration((-ox, -oy, ox, oy)))
    tx = WorldTransaction().update_physics_material("bubble", material)
    for k, ((lx, ly), (ux, uy)) in enumerate([((-ox, -oy), (-hx, oy)), ((hx, -oy), (ox, oy)),
                                              ((-hx, -oy), (hx, -hy)), ((-hx, hy), (hx, oy))]):
        tx = tx.add(RigidBodyDescriptor(9001 + k, Polygon(((lx, ly), (ux, ly), (ux, uy), (lx, uy))), (0.0, 0.0)))
    world.submit(tx)
    frame = world.advance(STEP)
    assert world.diagnostics.last_advance_issue is None and len(frame.transaction_receipts) == 1
    return world


def inside_frame(p):
    return abs(p[0]) <= HALF[0] + FRAME_TOLERANCE and abs(p[1]) <= HALF[1] + FRAME_TOLERANCE


def run_crowd(world, target, seed=2500, extra_steps=600, maximum_steps=8000):
    """CrowdScene.runCrowd; returns the report's counters and the mean effective / target radius of the last second."""
    rng = np.random.default_rng(seed)
    report = dict(steps=0, issue=None, exits=0, vanished=0, outside=[], rejections=[])
    areas, next_id, added, targets = 0.0, 1, [], {}
    pending, to_next, after = None, 0, None
    last_second = []
    while True:
        if pending is None and areas / AREA < target:
            if to_next == 0:
                to_next = 14
                radius = float(np.float32(rng.uniform(12.0, 48.0)))
                initial = float(np.float32(radius) * np.float32(0.1))
                lx, ly = (float(np.float32(h) - np.float32(initial)) for h in HALF)
                point = (float(np.float32(rng.uniform(-lx, lx))), float(np.float32(rng.uniform(-ly, ly))))
                mass = float(np.float32(radius) * np.float32(radius) / np.float32(400))
                tx = WorldTransaction().add(BubbleDescriptor(next_id, point, initial, mass, "bubble",
                                                             event_interest=INTEREST))
                tx = tx.start_transition(ParameterTransition(("bubbleRadius", next_id), radius, 1.0))
                pending = (world.submit(tx), next_id, radius)
            else:
                to_next -= 1
        frame = world.advance(STEP)
        report["steps"] += 1
        if world.diagnostics.last_advance_issue is not None:
            report["issue"] = (report["steps"], world.diagnostics.last_advance_issue, world.diagnostics.last_rejection_reason)
            return report, None
        if pending is not None:
            token, oid, radius = pending
            for e in frame.events:
                if e.kind == "transactionRejected" and e.token == token:
                    report["rejections"].append(e.rejection.reason)
                    pending, to_next = None, 0
            if pending is not None and any(r.token == token for r in frame.transaction_receipts):
                added.append(oid)
                targets[oid] = radius
                next_id += 1
                areas += math.pi * radius * radius
                pending = None
                if areas / AREA >= target:
                    after = 0
        report["exits"] += sum(e.kind == "didExitSimulationRegion" for e in frame.events)
        sample = []
        for oid in added:
            state = frame.objects.get(oid)
            if state is None:
                report["vanished"] += 1
                continue
            if not inside_frame(state.position):
                report["outside"].append((report["steps"], oid, state.position))
            sample.append((oid, state.effective_radius))
        last_second = (last_second + [sample])[-LAST_SECOND:]
        if after is not None:
            if after >= extra_steps:
                break
            after += 1
        assert report["steps"] < maximum_steps, f"the crowd did not reach B = {target} in {maximum_steps} steps"
    report["balance"] = areas / AREA
    report["last_second"] = len(last_second)
    ratios = [r / targets[oid] for frame in last_second for oid, r in frame]
    return report, float(np.mean(ratios))


def assert_crowd_kept_steps_accepted(report, failure_reason, balance):
    """assertCrowdKeptStepsAccepted (CrowdCompressionTests.swift:13-32) with centres required inside the frame."""
    assert report["issue"] is None, report["issue"]
    assert failure_reason is None
    assert report["exits"] == 0 and report["vanished"] == 0
    assert not report["outside"], report["outside"][:3]
    assert report["balance"] >= balance
    assert report["steps"] >= 600
    assert all(r == TransactionRejectionReason.INVALID_PLACEMENT for r in report["rejections"]), report["rejections"]
    assert report["last_second"] == LAST_SECOND


_RUNS = {}


def crowd(base, balance):
    """One seeded crowd per (material, balance), shared by the tests of this module: (report, ratio, failure reason)."""
    if (base, balance) not in _RUNS:
        world = make_world(soft_material(base))
        report, ratio = run_crowd(world, balance)
        _RUNS[base, balance] = report, ratio, world.diagnostics.failure_reason
        world.close()
    return _RUNS[base, balance]


SOFT = 3.85e-3  # CrowdScene.softCrowdPhysics: c0 = 3.85e-3 at r_ref = 20, K_c ~ 5195


def test_soft_crowd_at_balance_2_5_keeps_steps_accepted_and_softer_material_compresses_contours_more():
    """CrowdCompressionTests.swift:81-97: B = 2.5 with the soft material keeps every step accepted and every centre in
    the frame with a mean effective / target radius below 1 (the reference reports 0.414 for this material); at
    B = 1.5 from the same seed a bubble 15 times softer (K_c 1333) ends with a more dented contour than a stiff one
    (K_c 20 000)."""
    report, ratio, failure = crowd(SOFT, 2.5)
    assert_crowd_kept_steps_accepted(report, failure, 2.5)
    assert ratio < 1
    ratios = {}
    for base in (0.015, 0.001):
        report, ratios[base], failure = crowd(base, 1.5)
        assert_crowd_kept_steps_accepted(report, failure, 1.5)
    assert ratios[0.015] < ratios[0.001], ratios


def test_soft_crowd_compresses_more_at_higher_balance():
    """CrowdCompressionTests.swift:99-112: from the same seed the denser crowd (B = 2.5) compresses the contours more
    than B = 1.5."""
    ratios = {}
    for balance in (1.5, 2.5):
        report, ratios[balance], _ = crowd(SOFT, balance)
        assert report["issue"] is None and report["last_second"] == LAST_SECOND
    assert ratios[1.5] > 0
    assert ratios[2.5] < ratios[1.5], ratios
