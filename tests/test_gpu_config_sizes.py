"""GPU parity at the workloads' own sizes: the CUDA path against the CPU oracle on the full large world (65,536 bubbles,
whole-GPU cooperative team), all 4,096 batched worlds (one persistent launch per step under the CUDA graph, autotuned
schedule) and the full rigid-heavy world (16,384 bubbles, ~3,000 bodies and ~5,600 static edges through the LBVH),
through the C ABI.

What must be bit-exact at these sizes is what the smaller parity cases already pin: cell keys, sorted candidate keys
(the k-row truncation under dense packing included), contact lists, substep histories and counts, limiter reports,
Morton keys of the rigid leaves, and with damping 0 every FP32 position and velocity. The grid reductions of the
whole-GPU team (cell width, h terms over 65,536 bubbles) and the scheduler's queue order are exercised here and
nowhere smaller. The reference rules behind these outputs are NativeGeometryKernels:179-330 (cells, rows) and
:350-415 (body rows).
"""
import numpy as np
import pytest

from bubblephysics_gb300 import _native as N
from bubblephysics_gb300 import scenes
from bubblephysics_gb300.solver import Batch, World
from oracle import oracle
from oracle.oracle import OracleWorld

pytestmark = pytest.mark.gpu

REPORT_KEYS = ("status", "substep_count", "rebuild_count", "candidate_count", "body_candidate_count",
               "candidate_overflow", "max_candidates_per_object", "contact_count", "limiter_term", "limiter_object",
               "violation_kind", "removed_count", "wrapped_count")


def same_reports(rg, rc, where=""):
    for key in REPORT_KEYS:
        assert rg[key].tolist() == rc[key].tolist(), (where, key)
    assert rg["cell_width"].tolist() == rc["cell_width"].tolist(), (where, "cell_width")


def same_bubbles(bg, bc, where=""):
    for f in ("center", "previous_center", "velocity", "rotation", "angular_velocity", "region_result"):
        if not np.array_equal(bg[f], bc[f]):
            differ = (bg[f].reshape(len(bg), -1) != bc[f].reshape(len(bc), -1)).any(axis=1)
            bad = np.flatnonzero(differ)
            raise AssertionError(f"{where} {f}: {bad.size} bubbles differ, first {bad[:5].tolist()}")


def test_large_world_full_size_bit_exact(ctx):
    """65,536 bubbles in 8192^2 on the whole-GPU team: 13 steps (the single-world measurement's warm-up and timed
    steps), every step's report, cells, candidates, contacts, substep history and state against the oracle."""
    spec = scenes.large_world()
    assert spec.bubble_count == 65536
    gpu, cpu = World(spec, ctx), OracleWorld(spec, 32)
    total_substeps = 0
    for step in range(13):
        sg, rg = gpu.step(1)
        sc, rc = cpu.step(1)
        assert sg == sc == N.OK, (step, sg, sc)
        same_reports(rg, rc, f"step {step}")
        total_substeps += int(rg["substep_count"][0])
        assert np.array_equal(gpu.substeps(), cpu.substeps().astype(np.float32)), step
        assert np.array_equal(gpu.cells(), cpu.cells()), step
        assert np.array_equal(gpu.candidates(), cpu.candidates()), step
        assert np.array_equal(gpu.contacts(), cpu.contacts()), step
        same_bubbles(gpu.bubbles(), cpu.bubbles(), f"step {step}")
    assert total_substeps > 13  # the grid is rebuilt inside steps: more than one substep per step on average


@pytest.fixture(scope="module")
def batched_specs():
    return scenes.batched_worlds(4096, seed=3)


def test_all_batched_worlds_bit_exact(ctx, batched_specs):
    """All 4,096 worlds of the batched workload (seed 3, ~903k bubbles, 0-32 bodies each) through the persistent
    kernel with the CUDA graph and the autotuned schedule: two steps, every world's report and bubbles against the
    oracle stepped world by world."""
    specs = batched_specs
    batch = Batch(specs, ctx, use_graph=True, autotune=True)
    cpu = [OracleWorld(s, 32) for s in specs]
    for step in range(2):
        st, rg = batch.step(1)
        rc = oracle.step_worlds_reports(cpu, 1)[0]
        assert st == N.OK, np.unique(rg["status"])
        bad = [w for w in range(len(specs)) if any(rg[k][w] != rc[k][w] for k in REPORT_KEYS)]
        assert not bad, (step, bad[:10])
        for w in range(len(specs)):
            same_bubbles(batch.bubbles(w), cpu[w].bubbles(), f"step {step} world {w}")


def test_rigid_world_full_size_bit_exact(ctx):
    """The rigid-heavy world at its full size (16,384 bubbles, bodies of extent U[4,48] in 4096^2): three steps with
    the LBVH rebuilt every step; Morton keys, candidates, contacts, reports and state against the oracle's
    brute-force loops every step."""
    spec = scenes.rigid_world()
    assert spec.bubble_count == 16384
    leaves = len(spec.segments) + len(spec.bodies)
    gpu, cpu = World(spec, ctx), OracleWorld(spec, 32)
    for step in range(3):
        sg, rg = gpu.step(1)
        sc, rc = cpu.step(1)
        assert sg == sc == N.OK, (step, sg, sc)
        same_reports(rg, rc, f"step {step}")
        keys = gpu.rigid_keys()
        assert keys.size == leaves
        assert np.array_equal(keys, cpu.rigid_keys()), step
        assert np.array_equal(gpu.candidates(), cpu.candidates()), step
        assert np.array_equal(gpu.contacts(), cpu.contacts()), step
        same_bubbles(gpu.bubbles(), cpu.bubbles(), f"step {step}")
    assert rg["body_candidate_count"][0] > 0
