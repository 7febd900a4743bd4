"""FP32 on the GPU against the FP64 rerun of the oracle, on the reference's accuracy scenes
(docs/sdlc/changes/2026-11-23-engine-4-0-0/change-design.md G4-AC3 and G4-AC5: after 1 s positions within 1 unit and
velocities within 2 % of the scene's largest speed; the radial-field orbit within 1 unit of a double-precision
integration after 2 s), plus momentum and energy drift of an elastic pair (NativeMetalSubstepKernelTests.swift:957-979:
momentum exact up to rounding, energy within 2 %) and the error growth of the dense plain world. Each test prints the
measured errors (pytest -s shows them)."""
import math

import numpy as np
import pytest

import fixtures
from bubblephysics_gb300 import _native as N
from bubblephysics_gb300 import scenes
from bubblephysics_gb300.solver import World
from bubblephysics_gb300.spec import WorldSpec, make_bubbles
from oracle.oracle import OracleWorld

pytestmark = pytest.mark.gpu

R2, M2 = 12.0, 0.36  # the reference scenes' bubble "2"


def head_on_pair() -> WorldSpec:
    b = make_bubbles([(310.0, 360.0), (410.0, 360.0)], R2, velocities=[(100.0, 0.0), (-100.0, 0.0)], masses=M2,
                     stiffness=229.0, damping=1.0)
    return WorldSpec(bubbles=b)


def wall_bounce() -> WorldSpec:
    b = make_bubbles([(360.0, 300.0)], R2, velocities=[(0.0, 100.0)], masses=M2, stiffness=229.0, damping=1.0)
    return WorldSpec(bubbles=b, segments=fixtures.floor_wall(y=360.0))


def crowd_hit() -> WorldSpec:
    grid = [(360.0 + 25.0 * (i % 4), 360.0 + 25.0 * (i // 4)) for i in range(16)]
    centers = grid + [(260.0, 397.5)]
    vel = [(0.0, 0.0)] * 16 + [(100.0, 0.0)]
    b = make_bubbles(centers, R2, velocities=vel, masses=M2, stiffness=229.0, damping=1.0)
    return WorldSpec(bubbles=b)


def radial_orbit() -> WorldSpec:
    b = make_bubbles([(460.0, 360.0)], R2, velocities=[(0.0, 100.0)], masses=1.0, stiffness=229.0, damping=0.0)
    f = N.ForceField()
    f.position[:] = [360.0, 360.0]
    f.kind = 1
    f.strength = -500.0
    f.radius = 400.0
    f.falloff = 0.0
    return WorldSpec(bubbles=b, fields=[f])


def errors(ctx, spec: WorldSpec, steps: int):
    gpu, ref = World(spec, ctx), OracleWorld(spec, 64)
    s1, _ = gpu.step(steps)
    s2, _ = ref.step(steps)
    assert s1 == s2 == N.OK
    b, st = gpu.bubbles(), ref.state64()
    dx = float(np.hypot(*(b["center"].astype(np.float64) - st[:, :2]).T).max())
    dv = float(np.hypot(*(b["velocity"].astype(np.float64) - st[:, 2:]).T).max())
    vmax = max(float(np.hypot(*spec.bubbles["velocity"].astype(np.float64).T).max()),
               float(np.hypot(*st[:, 2:].T).max()))
    return dx, dv, vmax


@pytest.mark.parametrize("name,build", [("head-on pair", head_on_pair), ("wall bounce", wall_bounce),
                                        ("crowd hit", crowd_hit), ("radial field", radial_orbit)])
def test_fp32_against_fp64_after_one_second(ctx, name, build):
    dx, dv, vmax = errors(ctx, build(), 60)
    print(f"\n[fp32 vs fp64, 1 s] {name}: max |dx| {dx:.3e}, max |dv| {dv:.3e} ({100 * dv / vmax:.4f} % of {vmax:.1f})")
    assert dx <= 1.0 and dv <= 0.02 * vmax


def test_radial_orbit_against_double_integration(ctx):
    """G4-AC5: 2 s in the field, against the same field integrated in double with step 1e-4 (velocity Verlet)."""
    spec = radial_orbit()
    w = World(spec, ctx)
    status, _ = w.step(120)
    assert status == N.OK
    p = np.array([460.0, 360.0])
    v = np.array([0.0, 100.0])
    centre = np.array([360.0, 360.0])

    def acc(x):
        d = x - centre
        r = math.hypot(*d)
        return d * (-500.0 / r) if 0 < r <= 400.0 else np.zeros(2)

    h = 1e-4
    a = acc(p)
    for _ in range(int(round(2.0 / h))):
        v = v + 0.5 * h * a
        p = p + h * v
        a = acc(p)
        v = v + 0.5 * h * a
    got = w.bubbles()["center"][0].astype(np.float64)
    err = float(np.hypot(*(got - p)))
    print(f"\n[radial field, 2 s] GPU vs double integration: {err:.4f} units")
    assert err <= 1.0


def test_pair_bounce_momentum_and_energy_drift(ctx):
    spec = fixtures.pair_bounce_scene()
    m = spec.bubbles["mass"].astype(np.float64)
    v0 = spec.bubbles["velocity"].astype(np.float64)
    p0 = (m[:, None] * v0).sum(0)
    e0 = 0.5 * (m * (v0 ** 2).sum(1)).sum()
    w = World(spec, ctx)
    status, _ = w.step(60)
    assert status == N.OK
    v = w.bubbles()["velocity"].astype(np.float64)
    p1 = (m[:, None] * v).sum(0)
    e1 = 0.5 * (m * (v ** 2).sum(1)).sum()
    scale = (m * np.hypot(*v0.T)).sum()
    dp, de = float(np.hypot(*(p1 - p0))) / scale, abs(e1 - e0) / e0
    print(f"\n[elastic pair, 1 s] momentum drift {dp:.3e} of sum |p|, kinetic energy drift {100 * de:.3f} %")
    assert dp <= 1e-5 and de <= 0.02


def test_dense_plain_world_error_growth(ctx):
    """The 256-bubble plain world under gravity is a dense, chaotic pile: FP32 and FP64 stay within 1e-3 units for the
    first steps and separate later (a contact that flips order changes the pile); the growth is printed."""
    spec = scenes.plain_world(seed=1)
    gpu, ref = World(spec, ctx), OracleWorld(spec, 64)
    grown = []
    done = 0
    for mark in (1, 10, 30, 60):
        s1, _ = gpu.step(mark - done)
        s2, _ = ref.step(mark - done)
        done = mark
        assert s1 == s2 == N.OK
        b, st = gpu.bubbles(), ref.state64()
        grown.append((mark, float(np.hypot(*(b["center"].astype(np.float64) - st[:, :2]).T).max())))
    print("\n[plain world] max |dx| fp32 vs fp64 after steps: " + ", ".join(f"{k}: {e:.2e}" for k, e in grown))
    assert grown[0][1] <= 1e-3 and grown[1][1] <= 1e-2
