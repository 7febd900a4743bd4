"""GPU parity: the CUDA path against the CPU oracle on the same seeded inputs, through the C ABI.

Discrete outputs (cell keys, candidate keys, contact lists, substep counts, limiter, violations) must be bit-exact;
with damping 0 and no rotating bodies every FP32 value is bit-exact too, because both sides evaluate the same
formulas in the same order with IEEE division / square root and no fused multiply-add.
"""
import numpy as np
import pytest

from bubblephysics_gb300 import _native as N
from bubblephysics_gb300 import scenes
from bubblephysics_gb300.solver import Batch, World
from oracle.oracle import OracleWorld

pytestmark = pytest.mark.gpu


def assert_same_state(bg, bc, exact=True, atol=0.0):
    for f in ("center", "velocity", "previous_center"):
        if exact:
            assert np.array_equal(bg[f], bc[f]), (f, np.abs(bg[f] - bc[f]).max())
        else:
            np.testing.assert_allclose(bg[f], bc[f], atol=atol, rtol=0)
    assert np.array_equal(bg["region_result"], bc["region_result"])


def test_plain_world_one_step_bit_exact(ctx):
    spec = scenes.plain_world(seed=1)
    gpu, cpu = World(spec, ctx), OracleWorld(spec, 32)
    sg, rg = gpu.step(1)
    sc, rc = cpu.step(1)
    assert sg == sc == N.OK
    for key in ("substep_count", "rebuild_count", "candidate_count", "contact_count", "limiter_term",
                "limiter_object", "candidate_overflow", "max_candidates_per_object"):
        assert rg[key].tolist() == rc[key].tolist(), key
    assert rg["cell_width"][0] == rc["cell_width"][0]
    assert np.array_equal(gpu.cells(), cpu.cells())
    assert np.array_equal(gpu.candidates(), cpu.candidates())
    assert np.array_equal(gpu.contacts(), cpu.contacts())
    assert_same_state(gpu.bubbles(), cpu.bubbles())


def test_plain_world_sixty_steps_bit_exact(ctx):
    spec = scenes.plain_world(seed=1)
    gpu, cpu = World(spec, ctx), OracleWorld(spec, 32)
    sg, rg = gpu.step(60)
    sc, rc = cpu.step(60)
    assert sg == sc == N.OK
    assert rg["substep_count"].tolist() == rc["substep_count"].tolist()
    assert rg["rebuild_count"].tolist() == rc["rebuild_count"].tolist()
    assert np.array_equal(gpu.substeps(), cpu.substeps().astype(np.float32))
    assert np.array_equal(gpu.candidates(), cpu.candidates())
    assert np.array_equal(gpu.contacts(), cpu.contacts())
    assert_same_state(gpu.bubbles(), cpu.bubbles())


def test_batch_equals_single_worlds(ctx):
    rng = np.random.default_rng(7)
    specs = [scenes.batched_world(rng, int(n), world_index=i, max_bodies=0) for i, n in enumerate([16, 40, 100, 300, 700])]
    batch = Batch(specs, ctx, use_graph=False)
    st, reps = batch.step(5)
    assert st == N.OK, reps["status"]
    for w, spec in enumerate(specs):
        cpu = OracleWorld(spec, 32)
        sc, rc = cpu.step(5)
        assert sc == N.OK
        assert reps["substep_count"][w] == rc["substep_count"].sum()
        assert_same_state(batch.bubbles(w), cpu.bubbles())


def test_multi_cta_path_matches_oracle_and_single_cta(ctx):
    """Execution-path twin (ExecutionPathTwinTests): the whole-GPU cooperative path and the one-block path give the
    same bits, and both match the oracle."""
    import dataclasses
    spec = scenes.plain_world(seed=4)
    forced = dataclasses.replace(spec, flags=spec.flags | N.WORLD_FORCE_MULTI_CTA)
    a, b, cpu = World(spec, ctx), World(forced, ctx), OracleWorld(spec, 32)
    sa, ra = a.step(20)
    sb, rb = b.step(20)
    sc, rc = cpu.step(20)
    assert sa == sb == sc == N.OK
    assert ra["substep_count"].tolist() == rb["substep_count"].tolist() == rc["substep_count"].tolist()
    assert_same_state(a.bubbles(), b.bubbles())
    assert_same_state(b.bubbles(), cpu.bubbles())
    assert np.array_equal(b.candidates(), cpu.candidates())
    assert np.array_equal(b.contacts(), cpu.contacts())


def test_large_world_matches_oracle(ctx):
    spec = scenes.large_world(seed=2, n=6000, side=2048.0)
    gpu, cpu = World(spec, ctx), OracleWorld(spec, 32)
    sg, rg = gpu.step(3)
    sc, rc = cpu.step(3)
    assert sg == sc == N.OK
    assert rg["substep_count"].tolist() == rc["substep_count"].tolist()
    assert rg["rebuild_count"].tolist() == rc["rebuild_count"].tolist()
    assert np.array_equal(gpu.cells(), cpu.cells())
    assert np.array_equal(gpu.candidates(), cpu.candidates())
    assert_same_state(gpu.bubbles(), cpu.bubbles())


def test_device_contact_law_matches_oracle_float(ctx):
    from oracle import oracle
    rng = np.random.default_rng(5)
    q = np.zeros((601, 8), np.float32)
    q[:, 0] = (10.0 ** (-4.0 + 10.0 * np.arange(601) / 600)).astype(np.float32)
    assert np.array_equal(ctx.contact_law(0, q)[:, 0], oracle.contact_law(0, q)[:, 0].astype(np.float32))
    pairs = np.zeros((2000, 8), np.float32)
    pairs[:, 0] = rng.choice([229, 343.5, 2290, 229000, 22], 2000)
    pairs[:, 1] = rng.uniform(1, 150, 2000)
    pairs[:, 2] = rng.choice([229, 343.5, 2290, 229000, 22], 2000)
    pairs[:, 3] = rng.uniform(1, 150, 2000)
    pairs[:, 4] = (pairs[:, 1] + pairs[:, 3]) * rng.uniform(0.001, 1.2, 2000)
    assert np.array_equal(ctx.contact_law(2, pairs)[:, :4], oracle.contact_law(2, pairs)[:, :4].astype(np.float32))
    walls = pairs.copy()
    walls[:, 2] = walls[:, 1] * rng.uniform(-0.1, 1.2, 2000)
    assert np.array_equal(ctx.contact_law(1, walls)[:, :3], oracle.contact_law(1, walls)[:, :3].astype(np.float32))
