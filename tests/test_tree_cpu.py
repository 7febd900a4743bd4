"""The LBVH key rule on the CPU: the oracle's keys equal an independent numpy float32 restatement of the rule, and
the sorted keys carry each leaf exactly once. The reference has no tree (its rigid candidates are brute force), so the
rule itself is this library's; what the reference fixes is the candidate set, checked on the GPU."""
import numpy as np

from bubblephysics_gb300 import scenes
from oracle.oracle import OracleWorld


def spread15(v):
    v = v.astype(np.uint64) & np.uint64(0x7FFF)
    out = np.zeros_like(v)
    for bit in range(15):
        out |= ((v >> np.uint64(bit)) & np.uint64(1)) << np.uint64(2 * bit)
    return out


def keys_by_rule(spec, bodies_prev, bodies_pos):
    f = np.float32
    a, b = spec.segments["a"].astype(f), spec.segments["b"].astype(f)
    lo = np.concatenate([np.minimum(a, b), np.minimum(bodies_pos, bodies_prev) - spec.bodies["bounding_radius"].astype(f)[:, None]])
    hi = np.concatenate([np.maximum(a, b), np.maximum(bodies_pos, bodies_prev) + spec.bodies["bounding_radius"].astype(f)[:, None]])
    c = (lo + hi) * f(0.5)
    cmin, cmax = c.min(axis=0), c.max(axis=0)
    ext = cmax - cmin
    scale = np.where(ext > 0, f(32767.0) / np.where(ext > 0, ext, f(1.0)), f(0.0)).astype(f)
    q = np.minimum(np.maximum((c - cmin) * scale, f(0.0)), f(32767.0)).astype(np.uint32)
    code = spread15(q[:, 0]) | (spread15(q[:, 1]) << np.uint64(1))
    return np.sort((code << np.uint64(32)) | np.arange(c.shape[0], dtype=np.uint64))


def test_oracle_keys_follow_the_rule_for_static_bodies():
    spec = scenes.rigid_world(seed=11, n=300, bodies=120, side=700.0, kinematic_fraction=0.0)
    w = OracleWorld(spec, 32)
    status, _ = w.step(1)
    assert status == 0
    pos = spec.bodies["position"].astype(np.float32)
    keys = w.rigid_keys()
    assert np.array_equal(keys, keys_by_rule(spec, pos, pos))
    leaves = len(spec.segments) + len(spec.bodies)
    assert np.array_equal(np.sort(keys & np.uint64(0xFFFFFFFF)), np.arange(leaves, dtype=np.uint64))
    assert int(keys.max() >> np.uint64(32)) < 2**30
    assert np.all(np.diff(keys.astype(np.float64)) >= 0)


def test_oracle_keys_use_the_swept_box_of_kinematic_bodies():
    spec = scenes.rigid_world(seed=12, n=300, bodies=120, side=700.0, kinematic_fraction=1.0)
    w = OracleWorld(spec, 32)
    steps = 3
    status, _ = w.step(steps)
    assert status == 0
    # pose after `steps` kinematic advances and the one before it, advanced in float like the oracle
    pos = spec.bodies["position"].astype(np.float32)
    vel = spec.bodies["velocity"].astype(np.float32)
    dt = np.float32(spec.time_step)
    prev = pos
    for _ in range(steps):
        prev = pos
        pos = (pos + vel * dt).astype(np.float32)
    assert np.array_equal(w.rigid_keys(), keys_by_rule(spec, prev, pos))
