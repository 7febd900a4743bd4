"""Contours on the GPU (bp_world_contours) against the oracle's restatement of the reference's contour passes
(NativePostSolveKernels:268-527): sample counts, points, levels and shapes bit-exact. Both take the sample directions
as the double-precision cosine and sine of the float angle, rounded to float."""
import numpy as np
import pytest

import fixtures
from bubblephysics_gb300 import scenes
from bubblephysics_gb300.solver import World
from oracle.oracle import OracleWorld

pytestmark = pytest.mark.gpu


def compare(spec, ctx, steps, **cfg):
    gpu, cpu = World(spec, ctx), OracleWorld(spec, 32)
    assert gpu.step(steps)[0] == cpu.step(steps)[0] == 0
    pg, cg, lg, sg, ms = gpu.contours(**cfg)
    pc, cc, lc, sc = cpu.contours(stride=pg.shape[1], **cfg)
    assert np.array_equal(cg, cc)
    mask = np.arange(pg.shape[1])[None, :] < cg[:, None]
    assert np.array_equal(lg[mask], lc[mask])
    assert np.array_equal(pg[mask], pc[mask])
    assert np.array_equal(sg, sc)
    return cg, lg, ms


def test_plain_world_contours_match_oracle(ctx):
    counts, level, ms = compare(scenes.plain_world(seed=1), ctx, 20)
    assert level.max() > 0.05  # the pile presses bubbles flat


def test_contours_against_one_sided_walls(ctx):
    compare(fixtures.press_scene(), ctx, 3)


def test_batched_world_contours_with_options(ctx):
    rng = np.random.default_rng(5)
    spec = scenes.batched_world(rng, 300, world_index=1)
    compare(spec, ctx, 5, max_edge=4.0, surface_tension=5.0, clearance=0.01)
