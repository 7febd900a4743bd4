"""Double-precision contact-law reference for tests: a Python restatement of the reference test suite's own oracle
(Tests/BubblePhysicsRuntimeTests/ContactLawReference.swift:10-217): the law F = K eps / (1 - eps)^2, its inverse,
the elastic energy, the equilibrium distance, the pair solution by bisection and the 1-D h-rule wall simulation.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field


def force(epsilon: float, stiffness: float) -> float:
    if not epsilon > 0:
        return 0.0
    return stiffness * epsilon / ((1 - epsilon) * (1 - epsilon))


def epsilon(q: float) -> float:
    if not q > 0:
        return 0.0
    return 2 * q / ((2 * q + 1) + math.sqrt(4 * q + 1))


def energy(eps: float, stiffness: float, radius: float) -> float:
    if not eps > 0:
        return 0.0
    return stiffness * radius * (eps / (1 - eps) + math.log1p(-eps))


def equilibrium_distance(f: float, stiffness: float, radius: float) -> float:
    return radius * (1 - epsilon(f / stiffness))


def maximum_epsilon(target: float, stiffness: float, radius: float) -> float:
    if not target > 0:
        return 0.0
    low, high = 0.0, 1.0
    for _ in range(200):
        mid = 0.5 * (low + high)
        if energy(mid, stiffness, radius) < target:
            low = mid
        else:
            high = mid
    return 0.5 * (low + high)


def pair_contact(overlap: float, ra: float, ka: float, rb: float, kb: float):
    """(force, eps_a, eps_b) solving ra eps(F/ka) + rb eps(F/kb) = overlap by bisection; None outside [0, ra + rb)."""
    if not (overlap >= 0 and overlap < ra + rb):
        return None

    def total(f):
        return ra * epsilon(f / ka) + rb * epsilon(f / kb)

    low, high = 0.0, max(ka, kb)
    while total(high) < overlap:
        high *= 2
    for _ in range(400):
        mid = 0.5 * (low + high)
        if total(mid) < overlap:
            low = mid
        else:
            high = mid
    f = 0.0 if overlap == 0 else 0.5 * (low + high)
    return f, epsilon(f / ka), epsilon(f / kb)


@dataclass
class WallScene:
    """Bubble moving perpendicular to a wall (ContactLawReference.WallScene): leapfrog with the h rule
    h = min(remaining, 1/omega, d / (4 |v|)), contact for d < r."""
    radius: float
    mass: float
    stiffness: float
    damping: float
    start_distance: float
    velocity: float
    press_force: float = 0.0
    band_stiffness: float = 0.0
    frame_step: float = 1.0 / 60
    maximum_substeps: int = 1024
    frames: list = field(default_factory=list)
    substeps: list = field(default_factory=list)

    def contact_force(self, d):
        return force(1 - d / self.radius, self.stiffness)

    def energy(self, d, v):
        return 0.5 * self.mass * v * v + energy(1 - d / self.radius, self.stiffness, self.radius) + self.press_force * d

    def _acc(self, d, v):
        return (self.contact_force(d) - self.press_force) / self.mass - self.damping * v

    def _limit(self, d, v):
        bound = self.frame_step
        k = self.band_stiffness
        eps = 1 - d / self.radius
        if eps > 0:
            k += self.stiffness * (1 + eps) / ((1 - eps) ** 3 * self.radius)
        if k > 0:
            bound = min(bound, 1 / math.sqrt(k / self.mass))
        if v != 0:
            bound = min(bound, d / (4 * abs(v)))
        return bound

    def run(self, frames: int):
        s, v = self.start_distance, self.velocity
        limit_exceeded = penetrated = False
        for _ in range(frames):
            remaining, count = self.frame_step, 0
            while remaining > 0:
                if count == self.maximum_substeps:
                    limit_exceeded = True
                    break
                lim = self._limit(s, v)
                h = min(remaining, lim)
                remaining = 0.0 if h >= remaining else remaining - h
                half = v + 0.5 * h * self._acc(s, v)
                s += h * half
                if s <= 0:
                    penetrated = True
                    count += 1
                    break
                v = half + 0.5 * h * self._acc(s, half)
                self.substeps.append((s, v, half, h, lim))
                count += 1
            self.frames.append((count, s, v))
            if limit_exceeded or penetrated:
                break
        return limit_exceeded, penetrated
