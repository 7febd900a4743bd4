"""Seeded synthetic worlds with the shapes and value distributions of the benchmark workloads.

No dataset is involved: every world is generated from a numpy PCG64 stream. Materials follow the reference's public
defaults: contact stiffness K_c = 229 (the stress scenes' material) and damping gamma = 0; gravity is an acceleration
(0, -980) on force-driven bubbles. Walls are static thin rectangles just outside the region, turned into one-sided
polygon edges exactly like NativeStaticPolygonEdges.segments.

Resolutions of infeasible or unspecified parts of the workload descriptions (stated once here):
 - plain_world (256 bubbles, r ~ U[8,24] in 375 x 700): the bubbles cover ~85 % of the region, so strict non-overlap
   rejection sampling cannot finish; the sampler shrinks the required centre distance by 5 % after every 2000 failed
   tries (soft contact resolves the initial overlap).
 - large_world (65,536 bubbles, log-normal radii): 60 % area fraction is met locally by a jittered grid in a square
   block at the bottom of the 8192^2 region (the bubbles' total area is only ~15 % of the region); the grid is rebuilt
   almost every substep through the minimum-margin switch.
 - batched worlds: the description gives no gravity and no mass, so there is none and masses follow the reference's
   crowd scenes (m = r^2 / 400, Tests/BubblePhysicsRuntimeTests/CrowdSceneSupport.swift:71); placement is a jittered
   grid at 40 % area fraction, velocities N(0, 30^2); bubbles whose centre would lie inside a rigid body are dropped;
   bodies are static (circles, capsules, polygons) or kinematic (any shape, slow constant drive), since the reference
   rejects dynamic bodies next to bubbles.
"""
from __future__ import annotations

import math

import numpy as np

from . import _native as N
from .spec import WorldSpec, make_bubbles

K_C = 229.0
GRAVITY = (0.0, -980.0)
DT = 1.0 / 60.0


def polygon_edges(points, first_id: int, owner_id: int | None = None) -> np.ndarray:
    """One-sided edges of a static polygon; numpy restatement of NativeStaticPolygonEdges.segments
    (Sources/BubblePhysicsNativeMetal/NativeStaticPolygonEdges.swift:16-72)."""
    pts = np.asarray(points, np.float32).reshape(-1, 2)
    n = pts.shape[0]

    def cross(u, v):
        return float(u[0]) * float(v[1]) - float(u[1]) * float(v[0])

    area = 0.0
    if n >= 3:
        for i in range(1, n - 1):
            area += cross(pts[i] - pts[0], pts[i + 1] - pts[0])
    out = []

    def seg(sid, a, b):
        s = np.zeros(1, N.SEGMENT_DTYPE)[0]
        s["id"] = sid
        s["owner_id"] = owner_id if owner_id is not None else 0
        s["a"] = a
        s["b"] = b
        s["flags"] = N.SEGMENT_HAS_OWNER if owner_id is not None else 0
        s["category"] = 1
        s["mask"] = 0xFFFFFFFF
        return s

    if n < 3 or area == 0.0:
        for i in range(n):
            out.append(seg(first_id + i, pts[i], pts[(i + 1) % n]))
        return np.array(out, N.SEGMENT_DTYPE)
    ring = [p.copy() for p in pts]
    removed = True
    while removed and len(ring) > 3:
        removed = False
        index = 0
        while index < len(ring) and len(ring) > 3:
            c = len(ring)
            incoming = ring[index] - ring[(index + c - 1) % c]
            outgoing = ring[(index + 1) % c] - ring[index]
            lengths = float(np.float32(math.sqrt(float(incoming[0] * incoming[0] + incoming[1] * incoming[1])))) * \
                float(np.float32(math.sqrt(float(outgoing[0] * outgoing[0] + outgoing[1] * outgoing[1]))))
            dt = float(incoming[0]) * float(outgoing[0]) + float(incoming[1]) * float(outgoing[1])
            if lengths > 0 and dt > 0 and abs(cross(incoming, outgoing)) <= 1e-5 * lengths:
                ring.pop(index)
                removed = True
            else:
                index += 1
    orientation = 1.0 if area > 0 else -1.0
    c = len(ring)
    for index in range(c):
        previous, a, b, nxt = ring[(index + c - 1) % c], ring[index], ring[(index + 1) % c], ring[(index + 2) % c]
        s = seg(first_id + index, a, b)
        convex_start = cross(a - previous, b - a) * orientation > 0
        convex_end = cross(b - a, nxt - b) * orientation > 0
        s["flags"] |= N.SEGMENT_POLYGON_EDGE | (N.SEGMENT_CONVEX_START if convex_start else 0) | \
            (N.SEGMENT_CONVEX_END if convex_end else 0)
        s["outward_sign"] = -1.0 if area > 0 else 1.0
        s["previous_start"] = previous
        out.append(s)
    return np.array(out, N.SEGMENT_DTYPE)


def wall_segments(region, thickness=32.0, first_id=1_000_000, owner_base=2_000_000) -> np.ndarray:
    """Four static thin rectangles just outside the region edges, as one-sided polygon edges."""
    x0, y0, x1, y1 = region
    t = thickness
    rects = [((x0 - t, y0 - t), (x1 + t, y0)), ((x0 - t, y1), (x1 + t, y1 + t)),
             ((x0 - t, y0), (x0, y1)), ((x1, y0), (x1 + t, y1))]
    segs = []
    sid = first_id
    for k, ((ax, ay), (bx, by)) in enumerate(rects):
        poly = [(ax, ay), (bx, ay), (bx, by), (ax, by)]
        e = polygon_edges(poly, sid, owner_base + k)
        sid += len(e)
        segs.append(e)
    return np.concatenate(segs)


def _rejection_place(rng, radii, region, max_tries=2000):
    x0, y0, x1, y1 = region
    n = radii.shape[0]
    centers = np.zeros((n, 2), np.float64)
    placed = 0
    scale = 1.0
    cell = 2.0 * float(radii.max())
    grid: dict = {}
    while placed < n:
        r = radii[placed]
        ok = False
        for _ in range(max_tries):
            c = np.array([rng.uniform(x0 + r, x1 - r), rng.uniform(y0 + r, y1 - r)])
            gx, gy = int(c[0] // cell), int(c[1] // cell)
            clash = False
            for dx in (-1, 0, 1):
                for dy in (-1, 0, 1):
                    for j in grid.get((gx + dx, gy + dy), ()):
                        if np.hypot(*(centers[j] - c)) < (radii[j] + r) * scale:
                            clash = True
                            break
                    if clash:
                        break
                if clash:
                    break
            if not clash:
                ok = True
                break
        if not ok:
            scale *= 0.95
            continue
        centers[placed] = c
        grid.setdefault((int(c[0] // cell), int(c[1] // cell)), []).append(placed)
        placed += 1
    return centers


def plain_world(seed: int = 1, n: int = 256) -> WorldSpec:
    """Plain single world: region [0,375] x [0,700] with static walls, 256 bubbles r ~ U[8,24], mass 8,
    velocities N(0, 30^2), K_c 229, gamma 0, gravity (0,-980), dt 1/60."""
    rng = np.random.default_rng(seed)
    region = (0.0, 0.0, 375.0, 700.0)
    radii = rng.uniform(8.0, 24.0, n)
    centers = _rejection_place(rng, radii, region)
    vel = rng.normal(0.0, 30.0, (n, 2))
    b = make_bubbles(centers, radii, velocities=vel, masses=8.0, stiffness=K_C, damping=0.0,
                     flags=N.BUBBLE_FORCE_DRIVEN | N.BUBBLE_ENABLED)
    return WorldSpec(bubbles=b, segments=wall_segments(region), region=region, gravity=GRAVITY, time_step=DT)


def large_world(seed: int = 2, n: int = 65536, side: float = 8192.0) -> WorldSpec:
    """Plain single large world: 8192^2 with walls, log-normal radii (median 6, sigma 0.4, clipped [3,20]),
    mass proportional to r^2 (mass 1 at r = 6), jittered grid at 60 % local area fraction at the bottom, velocities
    N(0, 30^2), minimum-margin switch so the grid is rebuilt almost every substep."""
    rng = np.random.default_rng(seed)
    region = (0.0, 0.0, side, side)
    radii = np.clip(rng.lognormal(math.log(6.0), 0.4, n), 3.0, 20.0)
    per = math.pi * float(np.mean(radii ** 2)) / 0.6
    spacing = math.sqrt(per)
    cols = int(math.ceil(math.sqrt(n)))
    ij = np.stack(np.divmod(np.arange(n), cols), axis=1)[:, ::-1].astype(np.float64)
    jitter = rng.uniform(-0.25, 0.25, (n, 2)) * spacing
    centers = (ij + 0.5) * spacing + jitter + np.array([spacing, spacing])
    vel = rng.normal(0.0, 30.0, (n, 2))
    masses = (radii / 6.0) ** 2
    b = make_bubbles(centers, radii, velocities=vel, masses=masses, stiffness=K_C, damping=0.0,
                     flags=N.BUBBLE_FORCE_DRIVEN | N.BUBBLE_ENABLED)
    return WorldSpec(bubbles=b, segments=wall_segments(region), region=region, gravity=GRAVITY, time_step=DT,
                     flags=N.WORLD_MINIMUM_MARGIN_ONLY)


def _regular_polygon(rng, sides, half):
    """Convex polygon: vertices on a circle of radius `half` (a cyclic polygon is convex), angles jittered by at most
    a quarter of the even spacing so no edge degenerates."""
    step = 2 * math.pi / sides
    angles = np.arange(sides) * step + rng.uniform(-0.25, 0.25, sides) * step + rng.uniform(0, 2 * math.pi)
    return np.stack([np.cos(angles) * half, np.sin(angles) * half], axis=1)


def _body_geometry(kind, rng, half):
    """Local geometry of a body about its centre of mass (NativeRigidGeometry, NativeRigidPolygonState.swift:76-158):
    vertices, fan triangles of a convex ring, bounding radius, core radius."""
    if kind == N.BODY_CIRCLE:
        return np.zeros((1, 2), np.float32), np.zeros((0, 3), np.uint32), half, half, 0.0
    if kind == N.BODY_CAPSULE:
        r = half * 0.4
        h = half - r
        return np.array([[-h, 0.0], [h, 0.0]], np.float32), np.zeros((0, 3), np.uint32), h + r, r, h
    sides = int(rng.integers(3, 9))
    pts = _regular_polygon(rng, sides, half)
    # centroid of the polygon (area-weighted) so vertices are local to the centre of mass
    x, y = pts[:, 0], pts[:, 1]
    xn, yn = np.roll(x, -1), np.roll(y, -1)
    cr = x * yn - xn * y
    area = cr.sum() / 2.0
    cx = ((x + xn) * cr).sum() / (6.0 * area)
    cy = ((y + yn) * cr).sum() / (6.0 * area)
    local = (pts - np.array([cx, cy])).astype(np.float32)
    tris = np.array([[0, i, i + 1] for i in range(1, sides - 1)], np.uint32)
    bound = float(np.sqrt((local.astype(np.float64) ** 2).sum(axis=1)).max())
    return local, tris, bound, 0.0, 0.0


def add_bodies(rng, count, region, size_range, first_id, kinematic_fraction=0.25, speed=5.0, spin=0.2,
               horizon=5.0, clearance=80.0, gap=50.0, tries=40):
    """Random static / kinematic bodies (1/3 polygons, 1/3 circles, 1/3 capsules). Static polygons become one-sided
    edges (like NativePublicWorld.step); static circles / capsules and every kinematic body are obstacle bodies.
    Every body keeps `gap` (more than a bubble diameter) from other bodies and from the region edge, so no bubble is
    trapped in a narrow gap; a kinematic body keeps `clearance` plus its travel over `horizon` seconds, so it never
    closes a gap onto a bubble (a squeeze a world cannot survive). A body without such room is left out."""
    x0, y0, x1, y1 = region
    bodies, verts, tris, segs = [], [], [], []
    placed_pos = np.zeros((count, 2))  # placed bodies: position, bounding radius, keep-out radius
    placed_bound = np.zeros(count)
    placed_keep = np.zeros(count)
    nplaced = 0
    # placed bodies by cell of a coarse grid: a candidate only needs the bodies within its largest keep-out reach
    cell = 64.0
    buckets: dict = {}
    max_bound = max_keep = 0.0
    polygons = []  # world vertices of the static polygons
    vcount = tcount = 0
    seg_id = first_id * 16
    for k in range(count):
        kind = [N.BODY_POLYGON, N.BODY_CIRCLE, N.BODY_CAPSULE][k % 3]
        half = float(rng.uniform(*size_range))
        local, tri, bound, core, hl = _body_geometry(kind, rng, half)
        kinematic = rng.uniform() < kinematic_fraction
        keep = bound + gap + (clearance + speed * math.sqrt(2.0) * horizon if kinematic else 0.0)
        pos = None
        for _ in range(tries):
            if x1 - x0 <= 2 * keep or y1 - y0 <= 2 * keep:
                break
            cand = np.array([rng.uniform(x0 + keep, x1 - keep), rng.uniform(y0 + keep, y1 - keep)])
            if nplaced < 256:
                near = np.arange(nplaced)
            else:
                reach = max(keep + max_bound, max_keep + bound)
                gx0, gx1 = int(math.floor((cand[0] - reach) / cell)), int(math.floor((cand[0] + reach) / cell))
                gy0, gy1 = int(math.floor((cand[1] - reach) / cell)), int(math.floor((cand[1] + reach) / cell))
                near = [j for gx in range(gx0, gx1 + 1) for gy in range(gy0, gy1 + 1) for j in buckets.get((gx, gy), ())]
                near = np.array(near, np.int64)
            d = np.hypot(placed_pos[near, 0] - cand[0], placed_pos[near, 1] - cand[1])
            if np.all(d >= np.maximum(keep + placed_bound[near], placed_keep[near] + bound)):
                pos = cand
                break
        if pos is None:
            continue
        placed_pos[nplaced], placed_bound[nplaced], placed_keep[nplaced] = pos, bound, keep
        buckets.setdefault((int(math.floor(pos[0] / cell)), int(math.floor(pos[1] / cell))), []).append(nplaced)
        max_bound, max_keep = max(max_bound, bound), max(max_keep, keep)
        nplaced += 1
        angle = float(rng.uniform(0, 2 * math.pi))
        bid = first_id + k
        if kind == N.BODY_POLYGON and not kinematic:
            c, s = math.cos(angle), math.sin(angle)
            world = np.stack([local[:, 0] * c - local[:, 1] * s, local[:, 0] * s + local[:, 1] * c], 1) + pos
            e = polygon_edges(world.astype(np.float32), seg_id, bid)
            seg_id += len(e)
            segs.append(e)
            polygons.append(world)
            bodies.append(None)
            continue
        rec = np.zeros(1, N.BODY_DTYPE)[0]
        rec["id"] = bid
        rec["position"] = pos
        rec["angle"] = angle
        rec["bounding_radius"] = bound
        rec["kind"] = kind
        rec["core_radius"] = core
        rec["half_length"] = hl
        rec["flags"] = N.BODY_KINEMATIC if kinematic else N.BODY_STATIC
        if kinematic:
            rec["velocity"] = rng.uniform(-speed, speed, 2)
            rec["angular_velocity"] = float(rng.uniform(-spin, spin))
        rec["vertex_offset"] = vcount
        rec["vertex_count"] = local.shape[0]
        rec["triangle_offset"] = tcount
        rec["triangle_count"] = tri.shape[0]
        rec["category"] = 1
        rec["mask"] = 0xFFFFFFFF
        verts.append(local)
        tris.append(tri)
        vcount += local.shape[0]
        tcount += tri.shape[0]
        bodies.append(rec)
    recs = [b for b in bodies if b is not None]
    body_arr = np.array(recs, N.BODY_DTYPE) if recs else np.zeros(0, N.BODY_DTYPE)
    vert_arr = np.concatenate(verts).astype(np.float32) if verts else np.zeros((0, 2), np.float32)
    tri_arr = np.concatenate(tris).astype(np.uint32) if tris else np.zeros((0, 3), np.uint32)
    seg_arr = np.concatenate(segs) if segs else np.zeros(0, N.SEGMENT_DTYPE)
    return body_arr, vert_arr, tri_arr, seg_arr, polygons


def _clear_of_bodies(centers, radii, bodies, polygons):
    """Bubbles that start clear of every obstacle body and static polygon (more than r + 1 away). Each obstacle only
    tests the centres inside a box that holds every centre it could reject."""
    keep = np.ones(centers.shape[0], bool)
    if centers.shape[0] == 0:
        return keep
    rmax = float(radii.max()) + 1.0
    order = np.argsort(centers[:, 0], kind="stable")
    xs = centers[order, 0]

    def near(x, y, reach):
        lo, hi = np.searchsorted(xs, x - reach, "left"), np.searchsorted(xs, x + reach, "right")
        idx = order[lo:hi]
        return idx[np.abs(centers[idx, 1] - y) <= reach]

    for b in bodies:
        idx = near(b["position"][0], b["position"][1], float(b["bounding_radius"]) + rmax)
        d = np.hypot(centers[idx, 0] - b["position"][0], centers[idx, 1] - b["position"][1])
        keep[idx] &= d > b["bounding_radius"] + radii[idx] + 1.0
    for poly in polygons:
        # convex polygon: the largest signed distance to its edge lines bounds the distance to it from below
        p = np.asarray(poly, np.float64)
        q = np.roll(p, -1, axis=0)
        e = q - p
        area = np.sum(p[:, 0] * q[:, 1] - q[:, 0] * p[:, 1])
        normal = np.stack([e[:, 1], -e[:, 0]], 1) * (1.0 if area > 0 else -1.0)
        normal /= np.linalg.norm(normal, axis=1, keepdims=True)
        # a centre it rejects lies in the polygon offset by rmax: the hull of the vertices moved along the bisectors
        nprev = np.roll(normal, 1, axis=0)
        corner = p + rmax * (normal + nprev) / (1.0 + (normal * nprev).sum(axis=1, keepdims=True))
        lo, hi = corner.min(axis=0) - 1.0, corner.max(axis=0) + 1.0
        centre, half = (lo + hi) / 2.0, float((hi - lo).max()) / 2.0
        idx = near(centre[0], centre[1], half)
        rel = centers[idx, None, :] - p[None, :, :]
        signed = (rel * normal[None, :, :]).sum(-1).max(axis=1)
        keep[idx] &= signed > radii[idx] + 1.0
    return keep


def batched_world(rng, n_target: int, *, world_index: int = 0, max_bodies: int = 32, gravity=(0.0, 0.0)) -> WorldSpec:
    """One world of the batched workload: n ~ given, r ~ U[6,24], region sized to 40 % area fraction, 0-32 bodies
    (half-extents U[8,40]), jittered-grid placement, mass r^2/400, velocities N(0, 30^2), no gravity."""
    radii = rng.uniform(6.0, 24.0, n_target)
    area = math.pi * float(np.mean(radii ** 2)) * n_target / 0.4
    side = math.sqrt(area)
    region = (0.0, 0.0, side, side)
    nb = int(rng.integers(0, max_bodies + 1))
    bodies, bverts, btris, bsegs, polygons = add_bodies(rng, nb, region, (8.0, 40.0), first_id=10_000 + 64 * world_index)
    cols = int(math.ceil(math.sqrt(n_target)))
    spacing = side / cols
    ij = np.stack(np.divmod(np.arange(n_target), cols), axis=1)[:, ::-1].astype(np.float64)
    centers = (ij + 0.5) * spacing + rng.uniform(-0.2, 0.2, (n_target, 2)) * spacing
    keep = _clear_of_bodies(centers, radii, bodies, polygons)
    centers, radii = centers[keep], radii[keep]
    n = centers.shape[0]
    vel = rng.normal(0.0, 30.0, (n, 2))
    b = make_bubbles(centers, radii, velocities=vel, masses=radii * radii / 400.0, stiffness=K_C, damping=0.0,
                     flags=N.BUBBLE_FORCE_DRIVEN | N.BUBBLE_ENABLED)
    walls = wall_segments(region)
    segs = np.concatenate([walls, bsegs]) if bsegs.size else walls
    segs = np.sort(segs, order="id")
    return WorldSpec(bubbles=b, segments=segs, bodies=bodies, body_vertices=bverts, body_triangles=btris,
                     region=region, gravity=gravity, time_step=DT)


def rigid_world(seed: int = 4, n: int = 16384, bodies: int = 4096, side: float = 4096.0,
                size_range=(4.0, 48.0), kinematic_fraction: float = 0.25) -> WorldSpec:
    """Rigid-heavy single world: `bodies` static or kinematic bodies (1/3 polygons, 1/3 circles, 1/3 capsules, extent
    U[4,48], i.e. half-extent U[2,24]) and `n` bubbles (r ~ U[4,10], mass r^2/400, velocities N(0, 30^2)) in a
    side x side walled region. Static polygons become one-sided edges, so the world has thousands of segments and
    bodies: the rigid candidates go through the LBVH. Bodies keep 10 units from each other (18 + their travel when
    kinematic, drive speed <= 2 over 5 s); bubbles sit on a jittered grid in the free space."""
    rng = np.random.default_rng(seed)
    region = (0.0, 0.0, side, side)
    half = (size_range[0] / 2.0, size_range[1] / 2.0)
    body_arr, bverts, btris, bsegs, polygons = add_bodies(rng, bodies, region, half, first_id=3_000_000,
                                                          kinematic_fraction=kinematic_fraction, speed=2.0, spin=0.1,
                                                          horizon=5.0, clearance=8.0, gap=10.0, tries=1000)
    cols = int(math.ceil(math.sqrt(2.0 * n)))
    spacing = side / cols
    ij = np.stack(np.divmod(np.arange(cols * cols), cols), axis=1)[:, ::-1].astype(np.float64)
    centers = (ij + 0.5) * spacing + rng.uniform(-0.1, 0.1, (cols * cols, 2)) * spacing
    radii = rng.uniform(4.0, 10.0, cols * cols)
    inside = (centers.min(axis=1) > radii + 1.0) & (centers.max(axis=1) < side - radii - 1.0)
    keep = inside & _clear_of_bodies(centers, radii, body_arr, polygons)
    idx = np.flatnonzero(keep)
    idx = np.sort(rng.choice(idx, size=min(n, idx.size), replace=False))
    centers, radii = centers[idx], radii[idx]
    vel = rng.normal(0.0, 30.0, (idx.size, 2))
    b = make_bubbles(centers, radii, velocities=vel, masses=radii * radii / 400.0, stiffness=K_C, damping=0.0,
                     flags=N.BUBBLE_FORCE_DRIVEN | N.BUBBLE_ENABLED)
    walls = wall_segments(region)
    segs = np.concatenate([walls, bsegs]) if bsegs.size else walls
    segs = np.sort(segs, order="id")
    return WorldSpec(bubbles=b, segments=segs, bodies=body_arr, body_vertices=bverts, body_triangles=btris,
                     region=region, time_step=DT)


def serving_world(job) -> WorldSpec:
    """World `w` of the serving pool: its own seeded stream, n ~ LogUniform[n_min, n_max], batched-world
    distributions otherwise."""
    seed, w, n_min, n_max = job
    rng = np.random.default_rng([seed, w])
    n = int(math.exp(rng.uniform(math.log(n_min), math.log(n_max))))
    return batched_world(rng, n, world_index=w)


def serving_worlds(count: int = 8192, seed: int = 5, n_min: int = 16, n_max: int = 4096, processes: int = 0):
    """The serving pool: `count` worlds with bubble counts log-uniform in [n_min, n_max] (each world from its own seed,
    so the pool can be generated in parallel; processes > 1 uses a spawned process pool)."""
    jobs = [(seed, w, n_min, n_max) for w in range(count)]
    if processes > 1 and count > 64:
        import multiprocessing
        from concurrent.futures import ProcessPoolExecutor
        with ProcessPoolExecutor(processes, mp_context=multiprocessing.get_context("spawn")) as ex:
            return list(ex.map(serving_world, jobs, chunksize=64))
    return [serving_world(j) for j in jobs]


def batched_worlds(count: int = 4096, seed: int = 3, n_min: int = 16, n_max: int = 1024, max_bodies: int = 32,
                   limit: int | None = None):
    """The batched workload: `count` worlds, bubble counts log-uniform in [n_min, n_max]. `limit` returns only the
    first worlds of the same sequence (a bounded sample of the workload)."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(math.log(n_min), math.log(n_max), count)).astype(np.int64)
    take = count if limit is None else min(limit, count)
    return [batched_world(rng, int(sizes[w]), world_index=w, max_bodies=max_bodies) for w in range(take)]


# ---- rigid solver worlds -----------------------------------------------------------------------------------------

class RigidScene:
    """Records of a rigid-solver world: RIGID_BODY_DTYPE bodies, their vertices (local to the centre of mass),
    SEGMENT_DTYPE static segments, the public joints, the bodies' object ids, the region and the step."""

    def __init__(self, bodies, vertices, segments, joints, region, dt=DT, triangles=()):
        self.bodies = bodies
        self.vertices = np.asarray(vertices, np.float32).reshape(-1, 2)
        self.triangles = np.asarray(triangles, np.uint32).reshape(-1, 4)
        self.segments = segments
        self.joints = joints
        self.body_ids = [int(i) for i in bodies["id"]]
        self.region = tuple(float(v) for v in region)
        self.dt = dt

    def joint_arrays(self, bubble_ids=()):
        from .rigid import prepare_joints
        return prepare_joints(self.joints, list(bubble_ids), self.body_ids)


def _rigid_body(bid, pose, vertex_offset, vertex_count, inverse_mass, inverse_inertia, radius, *, velocity=(0.0, 0.0),
                spin=0.0, damping=0.0, static=False, kinematic=False, wrap=False, centroid=(0.0, 0.0),
                speed_limits=(0.0, 0.0), category=1, mask=0xFFFFFFFF, restitution=0.0, friction=0.5):
    b = np.zeros(1, N.RIGID_BODY_DTYPE)[0]
    b["id"] = bid
    b["pose"] = (pose[0], pose[1], pose[2], pose[2])
    b["previous"] = (pose[0], pose[1], centroid[0], centroid[1])
    b["motion"] = (velocity[0], velocity[1], spin, damping)
    b["physical"] = (0.0 if static or kinematic else inverse_mass, 0.0 if static or kinematic else inverse_inertia,
                     radius, friction)
    b["ranges"] = (vertex_offset, vertex_count, 0, 0)
    b["flags"] = (1 if static else 0, 1 if wrap else 0, 0, np.float32(restitution).view(np.uint32))
    b["filter"] = (category, mask, 1 if kinematic else 0, 0)
    b["limits"] = (speed_limits[0], speed_limits[1], 0.0, 0.0)
    return b


def _box(hx, hy, centroid=(0.0, 0.0)):
    return [(-hx - centroid[0], -hy - centroid[1]), (hx - centroid[0], -hy - centroid[1]),
            (hx - centroid[0], hy - centroid[1]), (-hx - centroid[0], hy - centroid[1])]


def jointed_chains(seed: int = 6, chains: int = 64, links: int = 16, spacing: float = 40.0) -> RigidScene:
    """Chains of box links hung from world points: every joint kind (hinges with and without limits and motors,
    soft damped distance joints, welds), random initial swing, some links with a centroid offset, speed limits and
    angular damping. The chains sit far inside the region and away from the floor segments, so no body meets
    another body: the reference's body contacts and wall guard do nothing here."""
    from .rigid import Joint
    rng = np.random.default_rng(seed)
    bodies, vertices, joints = [], [], []
    jid = 1
    for c in range(chains):
        ax, ay = (c % 16) * spacing * 2.0, 2000.0 + (c // 16) * spacing * 3.0
        prev = None
        for i in range(links):
            hx, hy = float(rng.uniform(0.8, 1.2)), float(rng.uniform(0.15, 0.3))
            centroid = (float(rng.uniform(-0.1, 0.1)), 0.0) if rng.random() < 0.2 else (0.0, 0.0)
            bid = 10_000 + c * links + i
            mass = 4.0 * hx * hy
            inertia = mass * ((2 * hx) ** 2 + (2 * hy) ** 2) / 12.0
            cx = ax + (2 * i + 1) * 1.05 + centroid[0]
            angle = float(rng.normal(0.0, 0.05))
            offset = len(vertices)
            vertices.extend(_box(hx, hy, centroid))
            limits = (float(rng.choice([0.0, 60.0])), float(rng.choice([0.0, 30.0])))
            bodies.append(_rigid_body(bid, (cx, ay, angle), offset, 4, 1.0 / mass, 1.0 / inertia,
                                      math.hypot(hx, hy) + 0.1, velocity=tuple(rng.normal(0.0, 3.0, 2)),
                                      spin=float(rng.normal(0.0, 1.0)), damping=float(rng.choice([0.0, 0.2])),
                                      centroid=centroid, speed_limits=limits))
            # anchors in the link's geometry frame (the centroid is subtracted inside the solver)
            left, right = (-1.05, 0.0), (1.05, 0.0)
            if prev is None:
                kind = ("hinge", "weld", "distance")[c % 3]
                joints.append(Joint(jid, bid, None, kind, anchor_a=left, anchor_b=(ax, ay), length=0.0,
                                    softness=1e-4 if kind == "distance" else 0.0,
                                    damping=2.0 if kind == "distance" else 0.0,
                                    limits=(-0.8, 0.8) if c % 6 == 0 else None))
            else:
                pick = (c + i) % 7
                if pick == 3:
                    joints.append(Joint(jid, prev, bid, "distance", anchor_a=(1.05, 0.0), anchor_b=left,
                                        length=0.05, softness=float(rng.choice([0.0, 1e-3])), damping=1.5))
                elif pick == 5:
                    joints.append(Joint(jid, prev, bid, "weld", anchor_a=(1.05, 0.0), anchor_b=left,
                                        reference_angle=float(rng.normal(0.0, 0.1))))
                else:
                    joints.append(Joint(jid, prev, bid, "hinge", anchor_a=(1.05, 0.0), anchor_b=left,
                                        limits=(-0.5, 0.5) if pick == 1 else None,
                                        motor=(2.0, 50.0) if pick == 2 else None))
            jid += 1
            prev = bid
    floor = polygon_edges([(-1000.0, -100.0), (4000.0, -100.0), (4000.0, -90.0), (-1000.0, -90.0)], 1_000_000)
    order = np.argsort([int(b["id"]) for b in bodies], kind="stable")
    return RigidScene(np.array([bodies[k] for k in order], N.RIGID_BODY_DTYPE), vertices, floor, joints,
                      (-2000.0, -2000.0, 6000.0, 6000.0))


def rigid_sweeps(seed: int = 7, movers: int = 96) -> RigidScene:
    """Dynamic bodies flung at thin static walls within one step: the predict sweep stops them before the wall
    (fast spins sample the rotation; one spin is over the 128-sample budget), kinematic bodies pass through,
    filtered bodies and bodies joined to a wall's owner without collideConnected ignore it; walls owned by static
    bodies leave a wall record. Some bodies start outside the region (removed or wrapped by the finish)."""
    from .rigid import Joint
    rng = np.random.default_rng(seed)
    bodies, vertices, segments, joints = [], [], [], []
    region = (0.0, 0.0, 1200.0, 1200.0)
    walls = []
    for w in range(6):
        x0, y0 = 100.0 + 180.0 * w, 100.0
        owner = 500 + w
        pts = [(x0, y0), (x0 + 4.0, y0), (x0 + 4.0, y0 + 900.0), (x0, y0 + 900.0)]
        offset = len(vertices)
        vertices.extend([(px - x0 - 2.0, py - y0 - 450.0) for px, py in pts])
        bodies.append(_rigid_body(owner, (x0 + 2.0, y0 + 450.0, 0.0), offset, 4, 0.0, 0.0, 451.0, static=True))
        segs = polygon_edges(pts, 100_000 + 10 * w, owner_id=owner if w % 3 else None)
        segments.extend(segs)
        walls.append((x0, owner))
    bid = 1000
    for m in range(movers):
        w = m % len(walls)
        x0, owner = walls[w]
        hx, hy = float(rng.uniform(2.0, 6.0)), float(rng.uniform(2.0, 6.0))
        mass = 4.0 * hx * hy
        inertia = mass * ((2 * hx) ** 2 + (2 * hy) ** 2) / 12.0
        side = -1.0 if m % 2 else 1.0
        start = (x0 + 2.0 - side * float(rng.uniform(10.0, 40.0)), float(rng.uniform(150.0, 950.0)))
        speed = float(rng.uniform(2000.0, 6000.0)) * side
        spin = float(rng.choice([0.0, rng.normal(0.0, 20.0), rng.normal(0.0, 150.0)]))
        if m == 7:
            spin = 450.0  # 7.5 rad in one step: over the 128-sample budget
        kinematic = m % 11 == 4
        category, mask = (2, 2) if m % 13 == 6 else (1, 0xFFFFFFFF)
        offset = len(vertices)
        vertices.extend(_box(hx, hy))
        bodies.append(_rigid_body(bid, (start[0], start[1], float(rng.uniform(-3, 3))), offset, 4, 1.0 / mass,
                                  1.0 / inertia, math.hypot(hx, hy), velocity=(speed, float(rng.normal(0, 200.0))),
                                  spin=spin, damping=float(rng.choice([0.0, 0.5])), kinematic=kinematic,
                                  category=category, mask=mask))
        if m % 17 == 9:  # joined to the wall's owner without collideConnected: that wall is transparent
            joints.append(Joint(len(joints) + 1, bid, owner, "distance", length=500.0, softness=1.0))
        bid += 1
    for k in range(8):  # outside the region: wrapped or removed by the finish
        offset = len(vertices)
        vertices.extend(_box(3.0, 3.0))
        pos = [(-50.0, 600.0), (1300.0, 600.0), (600.0, -40.0), (600.0, 1290.0)][k % 4]
        bodies.append(_rigid_body(bid, (pos[0], pos[1], 0.3 * k), offset, 4, 1.0 / 36.0, 1.0 / 216.0, 4.3,
                                  velocity=(0.0, 0.0), wrap=k % 2 == 0))
        bid += 1
    return RigidScene(np.array(bodies, N.RIGID_BODY_DTYPE), vertices, np.array(segments, N.SEGMENT_DTYPE), joints,
                      region, dt=DT)


def _shape_record(body, kind, core_radius=0.0, half_length=0.0):
    body["shape"] = (float(kind), core_radius, half_length, 0.0)
    return body


def rigid_pile(seed: int = 8, count: int = 256, columns: int = 16) -> RigidScene:
    """Dynamic boxes, circles and capsules dropped in columns onto a static floor and ramps, some pairs joined
    (with and without collideConnected): every part of the rigid step works here - body-pair rows, CCD of fast
    bodies, polygon / round contacts with friction and restitution, the wall guard against the static polygons, and
    the joint rounds. Bodies start just apart and fall at 60-240 units/s (the rigid predict applies no gravity)."""
    from .rigid import Joint
    rng = np.random.default_rng(seed)
    bodies, vertices, triangles, joints = [], [], [], []

    def polygon(points):
        offset, tri = len(vertices), len(triangles)
        vertices.extend(points)
        for k in range(1, len(points) - 1):
            triangles.append((0, k, k + 1, 0))
        return offset, len(points), tri, len(points) - 2

    def add_static_box(bid, cx, cy, hx, hy, angle=0.0):
        off, n, tri, nt = polygon(_box(hx, hy))
        b = _rigid_body(bid, (cx, cy, angle), off, n, 0.0, 0.0, math.hypot(hx, hy), static=True)
        b["ranges"] = (off, n, tri, nt)
        bodies.append(b)

    add_static_box(1, 0.0, -10.0, 600.0, 10.0)
    add_static_box(2, -300.0, 80.0, 120.0, 6.0, 0.35)
    add_static_box(3, 300.0, 80.0, 120.0, 6.0, -0.35)
    spacing = 18.0
    bid = 100
    for k in range(count):
        col, row = k % columns, k // columns
        cx = (col - columns / 2 + 0.5) * spacing + float(rng.uniform(-1.0, 1.0))
        cy = 40.0 + row * spacing + float(rng.uniform(0.0, 2.0))
        kind = k % 3
        vy = -float(rng.uniform(60.0, 240.0))
        vx = float(rng.normal(0.0, 20.0))
        spin = float(rng.normal(0.0, 2.0))
        if kind == 0:  # box
            hx, hy = float(rng.uniform(4.0, 7.0)), float(rng.uniform(3.0, 6.0))
            off, n, tri, nt = polygon(_box(hx, hy))
            mass = 4.0 * hx * hy
            inertia = mass * ((2 * hx) ** 2 + (2 * hy) ** 2) / 12.0
            b = _rigid_body(bid, (cx, cy, float(rng.uniform(-0.5, 0.5))), off, n, 1.0 / mass, 1.0 / inertia,
                            math.hypot(hx, hy), velocity=(vx, vy), spin=spin, restitution=float(rng.choice([0.0, 0.3])),
                            friction=float(rng.uniform(0.2, 0.8)))
            b["ranges"] = (off, n, tri, nt)
        elif kind == 1:  # circle
            r = float(rng.uniform(3.0, 6.0))
            off = len(vertices)
            vertices.append((0.0, 0.0))
            mass = math.pi * r * r
            b = _rigid_body(bid, (cx, cy, 0.0), off, 1, 1.0 / mass, 2.0 / (mass * r * r), r, velocity=(vx, vy),
                            spin=spin, friction=float(rng.uniform(0.2, 0.8)))
            _shape_record(b, 1, r)
        else:  # capsule
            r, h = float(rng.uniform(2.0, 4.0)), float(rng.uniform(2.0, 5.0))
            off = len(vertices)
            vertices.extend([(-h, 0.0), (h, 0.0)])
            mass = math.pi * r * r + 4.0 * h * r
            inertia = mass * ((2 * h) ** 2 / 12.0 + r * r / 2.0)
            b = _rigid_body(bid, (cx, cy, float(rng.uniform(-1.0, 1.0))), off, 2, 1.0 / mass, 1.0 / inertia, h + r,
                            velocity=(vx, vy), spin=spin, restitution=0.2, friction=0.5)
            _shape_record(b, 2, r, h)
        bodies.append(b)
        if k >= columns and k % 7 == 0:  # joined to the body below it
            joints.append(Joint(len(joints) + 1, bid - columns, bid, "distance", length=spacing, softness=1e-3,
                                collide_connected=k % 2 == 0))
        bid += 1
    return RigidScene(np.array(bodies, N.RIGID_BODY_DTYPE), vertices, np.zeros(0, N.SEGMENT_DTYPE), joints,
                      (-2000.0, -2000.0, 2000.0, 4000.0), triangles=triangles)
