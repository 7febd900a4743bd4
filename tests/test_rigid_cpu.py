"""Rigid solver passes on the CPU: the oracle (predict, joint rounds, finish) against an independent numpy float32
restatement of the joint rounds and the finish, the joint records against the reference's preparation rules
(NativeJointState.swift:61-141), the library's float sin / cos against double precision, and the physics the
reference's kernels promise (a sweep stops a body before a thin wall; rigid joints close their gap).

The reference's own tests hold no numbers for these kernels (they run on Metal), so the oracle is pinned by the
second restatement and by these properties."""
import numpy as np
import pytest

from bubblephysics_gb300 import _native as N
from bubblephysics_gb300 import scenes
from bubblephysics_gb300.rigid import Joint, prepare_joints
from oracle.oracle import OracleRigid, sincos

F = np.float32


# ---- the library's float sin / cos ---------------------------------------------------------------------------

def np_sincos(x):
    """numpy float32 restatement of the Cody-Waite / Taylor sin and cos (cos, sin)."""
    x = np.asarray(x, F)
    k = np.rint(x * F(float.fromhex("0x1.45f306p-1")))
    c1, c2, c3 = (F(float.fromhex(h)) for h in ("0x1.92p+0", "0x1.fb6p-12", "-0x1.777a5cp-25"))
    r = ((x - k * c1) - k * c2) - k * c3
    r2 = r * r
    s = [F(float.fromhex(h)) for h in ("-0x1.555556p-3", "0x1.111112p-7", "-0x1.a01a02p-13", "0x1.71de3ap-19",
                                       "-0x1.ae6456p-26")]
    c = [F(float.fromhex(h)) for h in ("-0x1.0p-1", "0x1.555556p-5", "-0x1.6c16c2p-10", "0x1.a01a02p-16",
                                       "-0x1.27e4fcp-22", "0x1.1eed8ep-29")]
    sr = r + r * r2 * (s[0] + r2 * (s[1] + r2 * (s[2] + r2 * (s[3] + r2 * s[4]))))
    cr = F(1) + r2 * (c[0] + r2 * (c[1] + r2 * (c[2] + r2 * (c[3] + r2 * (c[4] + r2 * c[5])))))
    q = k.astype(np.int64) & 3
    sn = np.select([q == 0, q == 1, q == 2], [sr, cr, -sr], -cr).astype(F)
    cs = np.select([q == 0, q == 1, q == 2], [cr, -sr, -cr], sr).astype(F)
    return cs, sn


def test_sincos_is_within_the_stated_error_and_matches_its_restatement():
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.uniform(-1000, 1000, 200_000), np.arange(-400, 400) * np.pi / 4]).astype(F)
    got = sincos(x)
    cs, sn = np_sincos(x)
    assert np.array_equal(got[:, 0], cs) and np.array_equal(got[:, 1], sn)
    for k, f in enumerate((np.cos, np.sin)):
        exact = f(x.astype(np.float64))
        err = np.abs(got[:, k].astype(np.float64) - exact)
        assert err.max() < 1e-7
        big = np.abs(exact) >= 0.25
        ulp = np.spacing(np.abs(exact[big]).astype(F)).astype(np.float64)
        assert (err[big] / ulp).max() <= 1.5
    assert np.isnan(sincos(np.array([np.inf, np.nan], F))).all()


# ---- joint records ---------------------------------------------------------------------------------------------

def test_joint_records_follow_the_reference_preparation():
    bubbles, bodies = [5, 6], [100, 200, 300]
    joints = [
        Joint(9, 200, 300, "hinge", anchor_a=(1, 0), anchor_b=(-1, 0), limits=(-1, 1), motor=(2, 3)),
        Joint(3, 100, None, "distance", anchor_a=(0.5, 0), anchor_b=(7, 8), length=2, softness=0.1, damping=4),
        Joint(4, 5, 100, "weld"),                           # a bubble end: only the no-collision exclusion stays
        Joint(5, 100, 999, "weld"),                         # unknown body: dropped
        Joint(7, 100, 200, "weld", reference_angle=0.25, collide_connected=True),
        Joint(8, 300, 100, "distance", length=1.0),
    ]
    a = prepare_joints(joints, bubbles, bodies)
    assert a.records["id"].tolist() == [3, 7, 8, 9]          # sorted by id
    world = a.records[0]
    assert world["ends"].tolist() == [N.JOINT_WORLD_END, 2, 0, 0]   # the world is end 0, the body end 1
    assert world["anchors"].tolist() == [7, 8, 0.5, 0]
    assert a.records[1]["ends"].tolist() == [2, 3, 2, 0] and a.records[1]["parameters"][3] == F(0.25)
    assert a.records[3]["ends"].tolist() == [3, 4, 1, 3] and a.records[3]["limits"].tolist() == [-1, 1, 2, 3]
    # body 100 (entity 2): joints 3 (side 1), 7 (side 0), 8 (side 1); partners: bubble 5 and body 300
    r = a.ranges[2]
    assert a.references[r[0]:r[0] + r[1]].tolist() == [[0, 1], [1, 0], [2, 1]]
    assert a.partners[r[2]:r[2] + r[3]].tolist() == [5, 300]
    assert a.partners[a.ranges[0][2]:a.ranges[0][2] + a.ranges[0][3]].tolist() == [100]   # bubble 5
    empty = prepare_joints([Joint(4, 5, 100, "weld")], bubbles, bodies)
    assert len(empty.records) == 0 and not empty.ranges.any() and empty.partners.size == 0


# ---- joint rounds: numpy restatement ------------------------------------------------------------------------------

def np_joint_rounds(bodies, joints, refs, ranges, bubble_count, dt, iteration_count, rounds):
    """Independent float32 restatement of nativeSolveJoints + nativeApplyJointBodies (NCK:446-562), every joint
    of a round from the same state (vectorised over joints), then each body's list summed in order."""
    bodies, joints = bodies.copy(), joints.copy()
    dt = max(F(dt), F(1e-6))
    ends, anchors, params, lims = joints["ends"], joints["anchors"], joints["parameters"], joints["limits"]
    kind, flags = ends[:, 2], ends[:, 3]
    tiny = np.finfo(F).tiny
    decay = np.exp((-params[:, 2] * dt / F(max(iteration_count, 1))).astype(np.float64)).astype(F)

    def end(e, anchor):
        world = e == N.JOINT_WORLD_END
        idx = np.where(world, 0, e.astype(np.int64) - bubble_count)
        b = bodies[idx]
        cs, sn = np_sincos(b["pose"][:, 2])
        lx, ly = anchor[:, 0] - b["previous"][:, 2], anchor[:, 1] - b["previous"][:, 3]
        ax, ay = lx * cs - ly * sn, lx * sn + ly * cs
        z = F(0)
        sel = lambda v, w=z: np.where(world, w, v).astype(F)
        return dict(px=sel(b["pose"][:, 0] + ax, anchor[:, 0]), py=sel(b["pose"][:, 1] + ay, anchor[:, 1]),
                    ax=sel(ax), ay=sel(ay), vx=sel(b["motion"][:, 0]), vy=sel(b["motion"][:, 1]),
                    w=sel(b["motion"][:, 2]), im=sel(b["physical"][:, 0]), ii=sel(b["physical"][:, 1]),
                    ang=sel(b["pose"][:, 2]))

    for _ in range(rounds):
        A, B = end(ends[:, 0], anchors[:, :2]), end(ends[:, 1], anchors[:, 2:])
        n_j = len(joints)
        mAx, mAy, mBx, mBy, tA, tB = (np.zeros(n_j, F) for _ in range(6))
        sAx, sAy, sBx, sBy, wA, wB = (np.zeros(n_j, F) for _ in range(6))
        pAx, pAy, pBx, pBy = -A["ay"], A["ax"], -B["ay"], B["ax"]
        for j in range(n_j):  # the scalar branches, per joint, in float32
            a = {k: v[j] for k, v in A.items()}
            b = {k: v[j] for k, v in B.items()}
            if kind[j] == 0:
                dx, dy = b["px"] - a["px"], b["py"] - a["py"]
                length = np.sqrt(dx * dx + dy * dy)
                nx, ny = (dx / length, dy / length) if length > F(1e-6) else (F(1), F(0))
                ca, cb = a["ax"] * ny - a["ay"] * nx, b["ax"] * ny - b["ay"] * nx
                w = a["im"] + b["im"] + a["ii"] * ca * ca + b["ii"] * cb * cb
                if w > tiny:
                    alpha = params[j, 1] / (dt * dt)
                    lam = (-(length - params[j, 0]) - alpha * joints[j]["state"][0]) / (w + alpha)
                    joints[j]["state"][0] = joints[j]["state"][0] + lam
                    mAx[j], mAy[j] = -nx * a["im"] * lam, -ny * a["im"] * lam
                    tA[j] = -ca * a["ii"] * lam
                    mBx[j], mBy[j] = nx * b["im"] * lam, ny * b["im"] * lam
                    tB[j] = cb * b["ii"] * lam
                    if params[j, 2] > 0:
                        rvx = (b["vx"] + pBx[j] * b["w"]) - (a["vx"] + pAx[j] * a["w"])
                        rvy = (b["vy"] + pBy[j] * b["w"]) - (a["vy"] + pAy[j] * a["w"])
                        rel = rvx * nx + rvy * ny
                        imp = -rel * (F(1) - decay[j]) / w
                        sAx[j], sAy[j] = F(0) - nx * a["im"] * imp, F(0) - ny * a["im"] * imp
                        wA[j] = F(0) - ca * a["ii"] * imp
                        sBx[j], sBy[j] = F(0) + nx * b["im"] * imp, F(0) + ny * b["im"] * imp
                        wB[j] = F(0) + cb * b["ii"] * imp
            else:
                weight = a["im"] + b["im"]
                k11 = weight + a["ii"] * pAx[j] * pAx[j] + b["ii"] * pBx[j] * pBx[j]
                k12 = a["ii"] * pAx[j] * pAy[j] + b["ii"] * pBx[j] * pBy[j]
                k22 = weight + a["ii"] * pAy[j] * pAy[j] + b["ii"] * pBy[j] * pBy[j]
                det = k11 * k22 - k12 * k12
                if det > tiny:
                    gx, gy = b["px"] - a["px"], b["py"] - a["py"]
                    ix, iy = -(k22 * gx - k12 * gy) / det, -(-k12 * gx + k11 * gy) / det
                    mAx[j], mAy[j] = -ix * a["im"], -iy * a["im"]
                    tA[j] = -a["ii"] * (pAx[j] * ix + pAy[j] * iy)
                    mBx[j], mBy[j] = ix * b["im"], iy * b["im"]
                    tB[j] = b["ii"] * (pBx[j] * ix + pBy[j] * iy)
                inertia = a["ii"] + b["ii"]
                if inertia > tiny:
                    ang = (b["ang"] + tB[j]) - (a["ang"] + tA[j]) - params[j, 3]
                    v = F(0)
                    if kind[j] == 2:
                        v = ang
                    elif flags[j] & 1:
                        v = ang - lims[j, 0] if ang < lims[j, 0] else (ang - lims[j, 1] if ang > lims[j, 1] else F(0))
                    if v != 0:
                        lam = -v / inertia
                        tA[j], tB[j] = tA[j] - a["ii"] * lam, tB[j] + b["ii"] * lam
                    if kind[j] == 1 and flags[j] & 2:
                        rel = (b["w"] + tB[j] / dt) - (a["w"] + tA[j] / dt) - lims[j, 2]
                        limit = lims[j, 3] * dt
                        total = min(max(joints[j]["state"][1] - rel / inertia, -limit), limit)
                        lam = total - joints[j]["state"][1]
                        joints[j]["state"][1] = total
                        wA[j], wB[j] = F(0) - a["ii"] * lam, F(0) + b["ii"] * lam
        first = np.stack([mAx, mAy, tA], 1)
        second = np.stack([mBx, mBy, tB], 1)
        vfirst = np.stack([mAx / dt + sAx, mAy / dt + sAy, tA / dt + wA], 1)
        vsecond = np.stack([mBx / dt + sBx, mBy / dt + sBy, tB / dt + wB], 1)
        for i in range(len(bodies)):
            start, count = ranges[bubble_count + i][:2]
            if count == 0:
                continue
            delta, vel = np.zeros(3, F), np.zeros(3, F)
            for ref in refs[start:start + count]:
                delta = delta + (second if ref[1] else first)[ref[0]]
                vel = vel + (vsecond if ref[1] else vfirst)[ref[0]]
            relax = F(1) / F(count)
            bodies[i]["pose"][:3] = bodies[i]["pose"][:3] + delta * relax
            bodies[i]["motion"][:3] = bodies[i]["motion"][:3] + vel * relax
    return bodies, joints


def test_joint_rounds_match_the_numpy_restatement_bit_for_bit():
    scene = scenes.jointed_chains(seed=11, chains=6, links=6)
    arrays = scene.joint_arrays()
    oracle = OracleRigid(scene.bodies, scene.vertices, scene.segments, arrays)
    for step in range(3):
        start = oracle.bodies()
        joints = oracle.joints()
        joints["state"] = 0  # the host clears the accumulated lambdas each step
        oracle.joint_records["state"] = 0
        want_b, want_j = np_joint_rounds(start, joints, arrays.references, arrays.ranges, 0, scene.dt, 8, 8)
        assert not np.array_equal(want_b["pose"], start["pose"])
        oracle.solve_joints(scene.dt, 8, 8)
        assert oracle.safety() == 0
        assert np.array_equal(oracle.bodies()["pose"], want_b["pose"]), step
        assert np.array_equal(oracle.bodies()["motion"], want_b["motion"]), step
        assert np.array_equal(oracle.joints()["state"], want_j["state"]), step
        oracle.predict(scene.dt)


def test_rigid_joints_close_their_gap():
    """One round of a rigid world hinge on a body without rotation inertia puts the anchor on the world point; a
    rigid distance joint restores its length; a motor's impulse stays within torque x dt."""
    body = scenes._rigid_body(1, (3.0, 1.0, 0.0), 0, 4, 1.0, 0.0, 1.0)
    verts = scenes._box(1.0, 0.5)
    for kind, length in (("hinge", 0.0), ("distance", 2.0)):
        arrays = prepare_joints([Joint(1, 1, None, kind, anchor_a=(-1.0, 0.0), anchor_b=(0.0, 0.0), length=length)],
                                [], [1])
        o = OracleRigid(np.array([body]), verts, None, arrays)
        o.solve_joints(1 / 60, 1, 8)
        p = o.bodies()[0]["pose"]
        gap = np.hypot(p[0] - 1.0, p[1])
        assert abs(gap - length) < 1e-6, (kind, gap)
    spinning = scenes._rigid_body(1, (0.0, 0.0, 0.0), 0, 4, 1.0, 2.0, 1.0, spin=10.0)
    arrays = prepare_joints([Joint(1, 1, None, "hinge", motor=(0.0, 3.0))], [], [1])
    o = OracleRigid(np.array([spinning]), verts, None, arrays)
    o.solve_joints(1 / 60, 8, 8)
    assert abs(o.joints()[0]["state"][1]) <= F(3.0) * F(1 / 60) * (1 + 1e-6)
    assert o.bodies()[0]["motion"][2] < 10.0


# ---- predict and finish --------------------------------------------------------------------------------------------

def test_predict_stops_bodies_before_thin_walls():
    scene = scenes.rigid_sweeps()
    arrays = scene.joint_arrays()
    o = OracleRigid(scene.bodies, scene.vertices, scene.segments, arrays)
    before = o.bodies()
    o.predict(scene.dt)
    after, walls = o.bodies(), o.walls()
    assert o.safety() & N.RIGID_SAFETY_ROTATION_BUDGET == N.RIGID_SAFETY_ROTATION_BUDGET
    excluded_owners = {(j.body_a, j.body_b) for j in scene.joints}
    wall_x = {500 + w: 100.0 + 180.0 * w for w in range(6)}
    checked = 0
    for k, (b0, b1) in enumerate(zip(before, after)):
        if b0["flags"][0] or b0["id"] < 1000 or b0["id"] >= 1000 + 96:
            continue
        m = int(b0["id"]) - 1000
        owner = 500 + m % 6
        x0 = wall_x[owner]
        if b0["filter"][2]:  # kinematic: straight through
            assert b1["pose"][0] == F(b0["pose"][0] + b0["motion"][0] * F(scene.dt))
            continue
        if m == 7 or b0["filter"][0] == 2 or (int(b0["id"]), owner) in excluded_owners:
            continue
        verts = scene.vertices[b1["ranges"][0]:b1["ranges"][0] + 4].astype(np.float64)
        c, s = np.cos(float(b1["pose"][2])), np.sin(float(b1["pose"][2]))
        xs = b1["pose"][0] + verts[:, 0] * c - verts[:, 1] * s
        if b0["motion"][0] > 0:
            assert xs.max() <= x0 + 1e-3, (m, xs.max(), x0)
        else:
            assert xs.min() >= x0 + 4.0 - 1e-3, (m, xs.min(), x0)
        assert not b1["motion"][:3].any()
        if m % 6 % 3:  # walls with an owner leave a record pointing back to the start side
            assert walls[k]["participants"].tolist() == [int(b0["id"]), owner]
            assert np.sign(walls[k]["geometry"][0]) == -np.sign(b0["motion"][0])
        checked += 1
    assert checked > 15


def np_finish(bodies, verts, region):
    """Independent restatement of nativeRigidFinish's region policy (NPK:172-198) for bodies at rest."""
    out = bodies.copy()
    rx0, ry0, rx1, ry1 = (F(v) for v in region)
    for b in out:
        if b["flags"][0]:
            continue
        v = verts[b["ranges"][0]:b["ranges"][0] + b["ranges"][1]]
        cs, sn = np_sincos(np.full(len(v), b["pose"][2], F))
        xs = b["pose"][0] + (v[:, 0] * cs - v[:, 1] * sn)
        ys = b["pose"][1] + (v[:, 0] * sn + v[:, 1] * cs)
        lo = np.array([xs.min(), ys.min()], F) - b["shape"][1]
        hi = np.array([xs.max(), ys.max()], F) + b["shape"][1]
        if hi[0] < rx0 or hi[1] < ry0 or lo[0] > rx1 or lo[1] > ry1:
            if not b["flags"][1]:
                b["flags"][2] = 1
            else:
                size = (rx1 - rx0, ry1 - ry0)
                shift = np.zeros(2, F)
                if hi[0] < rx0: shift[0] = np.ceil((rx0 - hi[0]) / size[0]) * size[0]
                if lo[0] > rx1: shift[0] = -np.ceil((lo[0] - rx1) / size[0]) * size[0]
                if hi[1] < ry0: shift[1] = np.ceil((ry0 - hi[1]) / size[1]) * size[1]
                if lo[1] > ry1: shift[1] = -np.ceil((lo[1] - ry1) / size[1]) * size[1]
                b["pose"][:2] = b["pose"][:2] + shift
                b["previous"][:2] = b["previous"][:2] + shift
                b["flags"][2] = 2
    return out


def test_finish_removes_or_wraps_bodies_outside_the_region():
    scene = scenes.rigid_sweeps()
    o = OracleRigid(scene.bodies, scene.vertices, scene.segments, None)
    start = o.bodies()
    o.finish(scene.region)
    got = o.bodies()
    want = np_finish(start, scene.vertices, scene.region)
    assert np.array_equal(got["pose"], want["pose"]) and np.array_equal(got["flags"], want["flags"])
    assert (got["flags"][:, 2] == 1).sum() == 4 and (got["flags"][:, 2] == 2).sum() == 4


# ---- body contacts, rows, CCD, wall guard ---------------------------------------------------------------------------

def pile_oracle(row_width=32, **kw):
    scene = scenes.rigid_pile(**kw)
    arrays = scene.joint_arrays()
    return scene, OracleRigid(scene.bodies, scene.vertices, scene.segments, arrays, triangles=scene.triangles,
                              row_width=row_width)


def test_body_pair_rows_are_sorted_and_symmetric():
    scene, o = pile_oracle()
    o.predict(scene.dt)
    o.body_candidates()
    rows, counts = o.candidates()
    assert counts[:, 1].sum() == 0 and counts[:, 0].sum() > 0
    pairs = set()
    for i, (row, n) in enumerate(zip(rows, counts[:, 0])):
        keys = [(int(c["metadata"][0]), int(c["participants"][0]), int(c["participants"][1])) for c in row[:n]]
        assert keys == sorted(keys)
        for c in row[:n]:
            low, high = int(c["metadata"][1]), int(c["metadata"][2])
            assert c["metadata"][0] == 3 and low < high and i in (low, high)
            pairs.add((low, high, i))
    full = {i for i, n in enumerate(counts[:, 0]) if n < o.row_width}  # rows that dropped nothing
    for low, high, owner in pairs:
        other = high if owner == low else low
        if other in full:
            assert (low, high, other) in pairs


def test_pile_settles_on_the_floor_without_tunnelling():
    scene, o = pile_oracle()
    for _ in range(60):
        o.step(scene.dt, scene.region)
    b = o.bodies()
    assert o.safety() == 0 and np.isfinite(b["pose"]).all()
    dynamic = b["flags"][:, 0] == 0
    # every dynamic body's centre stays above the floor's top face (y = 0) by more than a fraction of its size
    assert (b["pose"][dynamic, 1] > 0.5).all(), b["pose"][dynamic, 1].min()
    assert np.abs(b["motion"][dynamic, :2]).max() < 250.0
    assert (o.rows["metadata"][:, 3] != 0).sum() > 100  # contacts carried normal impulses


def test_ccd_stops_a_fast_body_before_it_passes_through_another():
    from bubblephysics_gb300.rigid import prepare_joints
    verts = scenes._box(20.0, 20.0) + scenes._box(2.0, 2.0)
    tris = [(0, 1, 2, 0), (0, 2, 3, 0)] * 2
    wall = scenes._rigid_body(1, (0.0, 0.0, 0.0), 0, 4, 0.0, 0.0, 28.3, static=True)
    wall["ranges"] = (0, 4, 0, 2)
    bullet = scenes._rigid_body(2, (-60.0, 0.0, 0.0), 4, 4, 1 / 16, 1 / 43, 2.9, velocity=(6000.0, 0.0))
    bullet["ranges"] = (4, 4, 2, 2)
    o = OracleRigid(np.array([wall, bullet]), verts, None, None, triangles=tris)
    o.predict(1 / 60)
    assert o.bodies()[1]["pose"][0] > 20.0  # the integration alone carries it through the wall
    o.body_candidates()
    o.ccd()
    x = float(o.bodies()[1]["pose"][0])
    assert -24.0 < x < -21.0, x  # stopped at the wall's near face (half widths 20 + 2)


# ---- pair contact: numpy restatement (NCK:248-373, NGK:444-581) ---------------------------------------------------

def _f(*v):
    return np.array(v, F)


def np_len(v):
    return np.sqrt(v[0] * v[0] + v[1] * v[1])


def np_dot(a, b):
    return a[0] * b[0] + a[1] * b[1]


def np_cross(a, b):
    return a[0] * b[1] - a[1] * b[0]


def np_closest(p, a, b):
    e = b - a
    sq = np_dot(e, e)
    t = min(max(np_dot(p - a, e) / sq, F(0)), F(1)) if sq > np.finfo(F).tiny else F(0)
    return a + e * t


def np_segment_distance(a, b, c, d):
    r, s = b - a, d - c
    den = np_cross(r, s)
    if abs(den) > F(1e-12):
        qp = c - a
        t, u = np_cross(qp, s) / den, np_cross(qp, r) / den
        if 0 <= t <= 1 and 0 <= u <= 1:
            pa = a + r * t
            return F(0), pa, pa
    best, pa, pb = F(np.inf), None, None
    for p, q, first in ((a, (c, d), True), (b, (c, d), True), (c, (a, b), False), (d, (a, b), False)):
        cp = np_closest(p, *q)
        v = np_len(p - cp)
        if v < best:
            best, pa, pb = v, (p if first else cp), (cp if first else p)
    return best, pa, pb


def np_vertex(body, verts, i):
    cs, sn = np_sincos(np.array([body["pose"][2]], F))
    v = verts[body["ranges"][0] + i]
    return _f(body["pose"][0] + (v[0] * cs[0] - v[1] * sn[0]), body["pose"][1] + (v[0] * sn[0] + v[1] * cs[0]))


def np_triangle_contact(a, b):
    depth, normal = F(np.inf), None
    for shape in (a, b):
        for e in range(3):
            delta = shape[(e + 1) % 3] - shape[e]
            m = np_len(delta)
            axis = _f(-delta[1], delta[0]) / m
            pa, pb = [np_dot(x, axis) for x in a], [np_dot(x, axis) for x in b]
            amin, amax, bmin, bmax = min(pa), max(pa), min(pb), max(pb)
            if amax < bmin or bmax < amin:
                return None
            plus, minus = amax - bmin, bmax - amin
            overlap = min(plus, minus)
            if overlap < depth:
                depth, normal = overlap, (axis if plus < minus else -axis)
    max_a = max(np_dot(x, normal) for x in a)
    min_b = min(np_dot(x, normal) for x in b)
    pa, pb, na, nb = _f(0, 0), _f(0, 0), 0, 0
    for k in range(3):
        if np_dot(a[k], normal) >= max_a - F(1e-5):
            pa, na = pa + a[k], na + 1
        if np_dot(b[k], normal) <= min_b + F(1e-5):
            pb, nb = pb + b[k], nb + 1
    return normal, depth, (pa / F(na) + pb / F(nb)) * F(0.5)


def np_round_contact(A, B):
    sep, pa, pb = np_segment_distance(A[0], A[1], B[0], B[1])
    assert sep > F(1e-4)  # the test pairs are apart at the cores
    n = (pb - pa) / sep
    return n, A[2] + B[2] - sep, ((pa + n * A[2]) + (pb - n * B[2])) * F(0.5)


def two_body_contact(a, b, verts, tris, full=False):
    """(normal, point, lambda) of the pair's first row slot after one contact round of the oracle (and the whole
    correction record with full=True)."""
    o = OracleRigid(np.array([a, b]), verts, None, None, triangles=tris, row_width=4)
    o.body_candidates()
    o.solve_contacts()
    c = o.contact_corrections[0]
    lam = o.rows[0]["metadata"][3].view(F)
    out = (_f(c["first"][3], c["second"][3]), _f(c["velocity_first"][3], c["velocity_second"][3]), lam)
    return out + (c,) if full else out


def np_contact_correction(a, b, n, point, depth):
    """The corrections of nativeRigidContacts (NCK:398-426) for a found contact: (first, second, velocity first,
    velocity second) xyz."""
    wa, wb, ia, ib = a["physical"][0], b["physical"][0], a["physical"][1], b["physical"][1]
    ra, rb = point - a["pose"][:2], point - b["pose"][:2]
    va, vb = a["motion"][:2], b["motion"][:2]
    spin_a, spin_b = a["motion"][2], b["motion"][2]
    ca, cb = np_cross(ra, n), np_cross(rb, n)
    denom = wa + wb + ia * ca * ca + ib * cb * cb
    lam = max(F(0), depth) / denom * F(0.5)
    first = np.append(-n * wa * lam, -ca * ia * lam)
    second = np.append(n * wb * lam, cb * ib * lam)
    closing = np_dot(vb - va, n) + spin_b * cb - spin_a * ca
    friction = np.sqrt(max(F(0), a["physical"][3] * b["physical"][3]))
    restitution = max(a["flags"][3:4].view(F)[0], b["flags"][3:4].view(F)[0])
    impulse = max(F(0), -closing) * (F(1) + restitution) / denom * F(0.5)
    tangent = _f(-n[1], n[0])
    tangent_speed = np_dot(vb - va, tangent) + spin_b * np_cross(rb, tangent) - spin_a * np_cross(ra, tangent)
    tangent_impulse = -tangent_speed * friction / denom * F(0.5)
    vfirst = np.append(-n * wa * impulse - tangent * wa * tangent_impulse,
                       -ca * ia * impulse - np_cross(ra, tangent) * ia * tangent_impulse)
    vsecond = np.append(n * wb * impulse + tangent * wb * tangent_impulse,
                        cb * ib * impulse + np_cross(rb, tangent) * ib * tangent_impulse)
    return lam, [x.astype(F) for x in (first, second, vfirst, vsecond)]


@pytest.mark.parametrize("seed", range(6))
def test_pair_contacts_match_the_numpy_restatement(seed):
    rng = np.random.default_rng(seed)
    tris = [(0, 1, 2, 0), (0, 2, 3, 0), (0, 1, 2, 0), (0, 2, 3, 0)]
    # two overlapping boxes: triangle SAT, the deepest piece
    verts = np.array(scenes._box(3.0, 2.0) + scenes._box(2.5, 1.5), F)
    a = scenes._rigid_body(1, (0.0, 0.0, float(rng.uniform(-0.3, 0.3))), 0, 4, 0.1, 0.01, 3.7,
                           velocity=tuple(rng.normal(0, 20, 2)), spin=float(rng.normal(0, 2)), friction=0.6,
                           restitution=0.25)
    b = scenes._rigid_body(2, (float(rng.uniform(3.5, 4.5)), float(rng.uniform(-1, 1)), float(rng.uniform(-0.3, 0.3))),
                           4, 4, 0.1, 0.01, 3.0, velocity=tuple(rng.normal(0, 20, 2)), spin=float(rng.normal(0, 2)),
                           friction=0.3, restitution=0.1)
    a["ranges"], b["ranges"] = (0, 4, 0, 2), (4, 4, 2, 2)
    n, point, lam, record = two_body_contact(a, b, verts, tris, full=True)
    best = None
    for ta in ((0, 1, 2), (0, 2, 3)):
        for tb in ((0, 1, 2), (0, 2, 3)):
            got = np_triangle_contact([np_vertex(a, verts, i) for i in ta], [np_vertex(b, verts, i) for i in tb])
            if got is not None and (best is None or got[1] > best[1]):
                best = got
    assert best is not None
    assert np.array_equal(n, best[0]) and np.array_equal(point, best[2])
    want_lam, want = np_contact_correction(a, b, best[0], best[2], best[1])
    assert lam == want_lam
    for field, expected in zip(("first", "second", "velocity_first", "velocity_second"), want):
        assert np.array_equal(record[field][:3], expected), field
    # two capsules whose cores are apart: segment distance of the cores
    verts = np.array([(-2.0, 0.0), (2.0, 0.0), (-1.5, 0.0), (1.5, 0.0)], F)
    rc = np.random.default_rng(500 + seed)  # cores tilted at most 0.2 rad, 1.2-1.8 apart: separated, overlapping radii
    a = scenes._shape_record(scenes._rigid_body(1, (0.0, 0.0, float(rc.uniform(-0.2, 0.2))), 0, 2, 0.2, 0.05, 3.0), 2,
                             1.0, 2.0)
    b = scenes._shape_record(scenes._rigid_body(2, (float(rc.uniform(0.5, 2.0)), float(rc.uniform(1.2, 1.8)),
                                                    float(rc.uniform(-0.2, 0.2))), 2, 2, 0.2, 0.05, 2.5), 2, 1.0, 1.5)
    n, point, lam = two_body_contact(a, b, verts, [])
    A = (np_vertex(a, verts, 0), np_vertex(a, verts, 1), F(1.0))
    B = (np_vertex(b, verts, 0), np_vertex(b, verts, 1), F(1.0))
    want_n, want_depth, want_point = np_round_contact(A, B)
    assert np.array_equal(n, want_n) and np.array_equal(point, want_point)
    assert want_depth > 0 and lam > 0


# ---- wall guard: numpy restatement (NPK:118-170) --------------------------------------------------------------------

def np_center_crossing_static(start, end, a, b):
    """nativeCenterCrossing (NGK:583-622) for a segment that does not move."""
    e0, de = b - a, _f(0, 0)
    r0, dr = start - a, end - start
    a_ = np_cross(de, dr)
    b_ = np_cross(e0, dr) + np_cross(de, r0)
    c = np_cross(e0, r0)
    if a_ == 0 and b_ == 0 and c == 0:
        q0 = np_dot(r0, r0 - e0)
        if q0 <= 0:
            return False
        qa = np_dot(dr, dr - de)
        qb = np_dot(dr, r0 - e0) + np_dot(r0, dr - de)
        minimum = min(q0, qa + qb + q0)
        if qa > 0:
            t = min(max(-qb / (F(2) * qa), F(0)), F(1))
            minimum = min(minimum, (qa * t + qb) * t + q0)
        return minimum <= 0
    roots = [F(-1), F(-1)]
    if abs(a_) <= np.finfo(F).eps * max(abs(b_), abs(c)):
        if abs(b_) > np.finfo(F).tiny:
            roots[0] = -c / b_
    for t in roots:
        if not (0 < t < 1):
            continue
        edge, rel = e0 + de * t, r0 + dr * t
        sq, along = np_dot(edge, edge), np_dot(rel, edge)
        if sq > np.finfo(F).tiny and 0 <= along <= sq:
            return True
    return False


def np_inside_polygon(p, body, verts, tris):
    cs, sn = np_sincos(np.array([-body["pose"][2]], F))
    d = p - body["pose"][:2]
    local = _f(d[0] * cs[0] - d[1] * sn[0], d[0] * sn[0] + d[1] * cs[0])
    for t in tris[body["ranges"][2]:body["ranges"][2] + body["ranges"][3]]:
        A, B, C = (verts[body["ranges"][0] + k] for k in t[:3])
        if np_cross(B - A, local - A) >= 0 and np_cross(C - B, local - B) >= 0 and np_cross(A - C, local - C) >= 0:
            return True
    return False


def np_guard(b, wall, verts, tris):
    """nativeRigidGuardWalls for one dynamic polygon body against one static polygon wall."""
    b = b.copy()
    wn = wall["ranges"][1]
    wv = [np_vertex(wall, verts, e) for e in range(wn)]
    for k in range(b["ranges"][1]):
        p = np_vertex(b, verts, k)
        cs, sn = np_sincos(np.array([b["pose"][3]], F))
        v = verts[b["ranges"][0] + k]
        start = _f(b["previous"][0] + (v[0] * cs[0] - v[1] * sn[0]), b["previous"][1] + (v[0] * sn[0] + v[1] * cs[0]))
        inside, started = np_inside_polygon(p, wall, verts, tris), np_inside_polygon(start, wall, verts, tris)
        if started and any(np_len(start - np_closest(start, wv[e], wv[(e + 1) % wn])) < F(1e-5) for e in range(wn)):
            started = False
        nearest, normal, depth = F(np.inf), None, F(0)
        for e in range(wn):
            ea, eb = wv[e], wv[(e + 1) % wn]
            direction = eb - ea
            raw = _f(direction[1], -direction[0])
            out = raw / np_len(raw)
            signed_start = np_dot(start - ea, out)
            on_boundary = np_len(start - np_closest(start, ea, eb)) < F(1e-5)
            crossing = signed_start >= F(-1e-5) and (np_center_crossing_static(start, p, ea, eb) or
                                                     (on_boundary and np_dot(p - ea, out) < 0))
            if not inside and not crossing:
                continue
            if inside and not started and signed_start < F(-1e-5):
                continue
            c = np_closest(p, ea, eb)
            d = np_len(start - np_closest(start, ea, eb)) if (crossing or not started) else np_len(p - c)
            if d < nearest:
                nearest, normal, depth = d, out, max(F(0), -np_dot(p - c, out))
        if np.isfinite(nearest) and depth > 0:
            shift = normal * (depth + F(1e-5))
            b["pose"][:2] = b["pose"][:2] + shift
            r = p - b["pose"][:2]
            lever = np_cross(r, normal)
            speed = np_dot(b["motion"][:2], normal) + b["motion"][2] * lever
            denom = b["physical"][0] + b["physical"][1] * lever * lever
            impulse = max(F(0), -speed) / max(denom, np.finfo(F).tiny)
            b["motion"][:2] = b["motion"][:2] + normal * b["physical"][0] * impulse
            b["motion"][2] = b["motion"][2] + lever * b["physical"][1] * impulse
    return b


@pytest.mark.parametrize("seed", range(8))
def test_wall_guard_matches_the_numpy_restatement(seed):
    rng = np.random.default_rng(100 + seed)
    verts = np.array(scenes._box(50.0, 5.0) + scenes._box(3.0, 2.0), F)
    tris = np.array([(0, 1, 2, 0), (0, 2, 3, 0)] * 2, np.uint32)
    floor = scenes._rigid_body(1, (0.0, 0.0, float(rng.uniform(-0.2, 0.2))), 0, 4, 0.0, 0.0, 50.3, static=True)
    floor["ranges"] = (0, 4, 0, 2)
    # a box that entered the floor's top face during the step (or started on it)
    y0 = float(rng.uniform(7.0, 9.0))
    y1 = float(rng.uniform(4.0, 6.5))
    box = scenes._rigid_body(2, (float(rng.uniform(-20, 20)), y1, float(rng.uniform(-0.4, 0.4))), 4, 4, 1 / 24, 1 / 104,
                             3.7, velocity=(float(rng.normal(0, 5)), -60.0), spin=float(rng.normal(0, 1)))
    box["previous"][:2] = (box["pose"][0], y0)
    box["pose"][3] = box["pose"][2] - F(rng.uniform(-0.05, 0.05))
    box["ranges"] = (4, 4, 2, 2)
    o = OracleRigid(np.array([floor, box]), verts, None, None, triangles=tris)
    o.guard_walls()
    got = o.bodies()[1]
    want = np_guard(box, floor, verts, tris)
    assert np.array_equal(got["pose"], want["pose"]) and np.array_equal(got["motion"], want["motion"])
    assert not np.array_equal(got["pose"], box["pose"])  # the guard pushed it out


# ---- CCD: numpy restatement (NPK:200-263) ---------------------------------------------------------------------------

def np_box_pair_depth(a, b, verts):
    """nativeRigidPairContact for two boxes of two triangles each: the deepest triangle pair's depth, or None."""
    best = None
    for ta in ((0, 1, 2), (0, 2, 3)):
        for tb in ((0, 1, 2), (0, 2, 3)):
            got = np_triangle_contact([np_vertex(a, verts, i) for i in ta], [np_vertex(b, verts, i) for i in tb])
            if got is not None and (best is None or got[1] > best):
                best = got[1]
    return best


def np_at(body, t):
    out = body.copy()
    out["pose"][0] = body["previous"][0] + (body["pose"][0] - body["previous"][0]) * t
    out["pose"][1] = body["previous"][1] + (body["pose"][1] - body["previous"][1]) * t
    out["pose"][2] = body["pose"][3] + (body["pose"][2] - body["pose"][3]) * t
    return out


def np_time_of_impact(a, b, verts):
    def overlap(t):
        d = np_box_pair_depth(np_at(a, t), np_at(b, t), verts)
        return d is not None and d > F(1e-3)
    da, db = a["pose"][:2] - a["previous"][:2], b["pose"][:2] - b["previous"][:2]
    travel = np_len(da - db) + abs(a["pose"][2] - a["pose"][3]) * a["physical"][2] + \
        abs(b["pose"][2] - b["pose"][3]) * b["physical"][2]
    if not travel > F(0.5) or overlap(F(0)):
        return F(2)
    samples = np.ceil(travel / F(0.5))
    steps = 64 if samples >= 64 else max(2, int(samples))
    last = F(0)
    for step in range(1, steps + 1):
        t = F(step) / F(steps)
        if not overlap(t):
            last = t
            continue
        low, high = last, t
        for _ in range(12):
            middle = F(0.5) * (low + high)
            if overlap(middle):
                high = middle
            else:
                low = middle
        return low
    return F(2)


@pytest.mark.parametrize("seed", range(4))
def test_ccd_matches_the_numpy_restatement(seed):
    rng = np.random.default_rng(200 + seed)
    verts = np.array(scenes._box(20.0, 20.0) + scenes._box(2.0, 2.0), F)
    tris = [(0, 1, 2, 0), (0, 2, 3, 0)] * 2
    wall = scenes._rigid_body(1, (0.0, 0.0, float(rng.uniform(-0.3, 0.3))), 0, 4, 0.0, 0.0, 28.3, static=True)
    wall["ranges"] = (0, 4, 0, 2)
    bullet = scenes._rigid_body(2, (-60.0, float(rng.uniform(-10, 10)), float(rng.uniform(-1, 1))), 4, 4, 1 / 16,
                                1 / 43, 2.9, velocity=(float(rng.uniform(4000, 7000)), float(rng.normal(0, 300))),
                                spin=float(rng.normal(0, 2)))
    bullet["ranges"] = (4, 4, 2, 2)
    o = OracleRigid(np.array([wall, bullet]), verts, None, None, triangles=tris)
    o.predict(1 / 60)
    moved = o.bodies()
    o.body_candidates()
    o.ccd()
    t = np_time_of_impact(moved[0], moved[1], verts)  # the pair (lower index, higher index) of the bullet's row
    assert t <= 1
    want = np_at(moved[1], t)
    got = o.bodies()[1]
    assert np.array_equal(got["pose"][:3], want["pose"][:3]) and got["limits"][2] == 0


# ---- body-pair rows and predict: numpy restatements -----------------------------------------------------------------

def test_body_pair_rows_match_the_numpy_restatement():
    """nativeEmitBodyCandidates, body pairs (NGK:394-415): every row equals the sorted, truncated list built here."""
    scene, o = pile_oracle(row_width=8)
    o.predict(scene.dt)
    o.body_candidates()
    rows, counts = o.candidates()
    b = o.bodies()
    arrays = scene.joint_arrays()
    excluded = {}
    for e, (_, _, start, n) in enumerate(arrays.ranges):
        excluded[e] = set(int(x) for x in arrays.partners[start:start + n])
    immovable = (b["flags"][:, 0] != 0) | (b["filter"][:, 2] != 0)
    dropped_total, wanted_max = 0, 0
    for i in range(len(b)):
        keys = []
        for other in range(len(b)):
            if other == i:
                continue
            lo, hi = min(i, other), max(i, other)
            A, C = b[lo], b[hi]
            if immovable[lo] and immovable[hi]:
                continue
            if not ((A["filter"][0] & C["filter"][1]) and (C["filter"][0] & A["filter"][1])):
                continue
            if int(b[other]["id"]) in excluded.get(i, ()):
                continue
            start = A["previous"][:2] - C["previous"][:2]
            travel = (A["pose"][:2] - C["pose"][:2]) - start
            ts = np_dot(travel, travel)
            t = min(max(-np_dot(start, travel) / ts, F(0)), F(1)) if ts > np.finfo(F).tiny else F(0)
            radius = F(1.25) * (A["physical"][2] + C["physical"][2])
            closest = start + travel * t
            if not np_dot(closest, closest) <= radius * radius:
                continue
            keys.append((3, int(np.int64(A["id"])), int(np.int64(C["id"])), lo, hi))
        keys.sort()
        kept = keys[:8]
        dropped_total += len(keys) - len(kept)
        wanted_max = max(wanted_max, len(keys))
        assert counts[i, 0] == len(kept)
        got = [(int(c["metadata"][0]), int(c["participants"][0]), int(c["participants"][1]), int(c["metadata"][1]),
                int(c["metadata"][2])) for c in rows[i, :counts[i, 0]]]
        assert got == kept, i
    assert o.overflow_counts().tolist() == [dropped_total, wanted_max]


def np_center_crossing(start, end, pa, pb, ca, cb):
    """nativeCenterCrossing (NGK:583-622): the point moving start -> end against the segment moving (pa, pb) ->
    (ca, cb)."""
    e0 = pb - pa
    de = (cb - ca) - e0
    r0 = start - pa
    dr = (end - start) - (ca - pa)
    a, b, c = np_cross(de, dr), np_cross(e0, dr) + np_cross(de, r0), np_cross(e0, r0)
    if a == 0 and b == 0 and c == 0:
        q0 = np_dot(r0, r0 - e0)
        if q0 <= 0:
            return False
        qa = np_dot(dr, dr - de)
        qb = np_dot(dr, r0 - e0) + np_dot(r0, dr - de)
        minimum = min(q0, qa + qb + q0)
        if qa > 0:
            t = min(max(-qb / (F(2) * qa), F(0)), F(1))
            minimum = min(minimum, (qa * t + qb) * t + q0)
        return minimum <= 0
    roots = [F(-1), F(-1)]
    if abs(a) <= np.finfo(F).eps * max(abs(b), abs(c)):
        if abs(b) > np.finfo(F).tiny:
            roots[0] = -c / b
    else:
        d = b * b - F(4) * a * c
        if d > 0:
            q = F(-0.5) * (b + np.copysign(np.sqrt(d), b))
            roots = [q / a, c / q if abs(q) > np.finfo(F).tiny else F(-1)]
    for t in roots:
        if not (0 < t < 1):
            continue
        edge, rel = e0 + de * t, r0 + dr * t
        sq, along = np_dot(edge, edge), np_dot(rel, edge)
        if sq > np.finfo(F).tiny and 0 <= along <= sq:
            return True
    return False


def np_sweep(body, p, q, verts, segs, excluded):
    """nativeRigidSweepCrossing (NPK:30-63): (point, normal, owner) of the first crossing, or None."""
    n = body["ranges"][1]
    (cp,), (sp,) = np_sincos(np.array([p[2]], F))
    (cq,), (sq_,) = np_sincos(np.array([q[2]], F))
    at_p = lambda v: p[:2] + _f(v[0] * cp - v[1] * sp, v[0] * sp + v[1] * cp)
    at_q = lambda v: q[:2] + _f(v[0] * cq - v[1] * sq_, v[0] * sq_ + v[1] * cq)
    for s in segs:
        has_owner = bool(s["flags"] & N.SEGMENT_HAS_OWNER)
        if has_owner and (int(np.uint64(s["owner_id"])) == int(body["id"]) or int(s["owner_id"]) in excluded):
            continue
        if not ((body["filter"][0] & s["mask"]) and (s["category"] & body["filter"][1])):
            continue
        A, B = s["a"].astype(F), s["b"].astype(F)
        for k in range(n):
            v, w = verts[body["ranges"][0] + k], verts[body["ranges"][0] + (k + 1) % n]
            sv, ev = at_p(v), at_q(v)
            hit = np_center_crossing(sv, ev, A, B, A, B)
            if not hit:
                ps, pe = at_p(v), at_p(w)
                qs, qe = at_q(v), at_q(w)
                hit = np_center_crossing(A, A, ps, pe, qs, qe) or np_center_crossing(B, B, ps, pe, qs, qe)
            if hit:
                edge = B - A
                raw = _f(edge[1], -edge[0])
                normal = raw / np_len(raw)
                if np_dot(sv - A, normal) < 0:
                    normal = -normal
                return np_closest(ev, A, B), normal, int(s["owner_id"])
    return None


def test_predict_sweep_matches_the_numpy_restatement():
    """nativeRigidPredict (NPK:66-115) for the movers of the sweep scene: damping, limits, integration, the sampled
    sweep with its bisection, the stop and the wall record, against the oracle bit for bit."""
    scene = scenes.rigid_sweeps()
    arrays = scene.joint_arrays()
    o = OracleRigid(scene.bodies, scene.vertices, scene.segments, arrays)
    start_state = o.bodies()
    o.predict(scene.dt)
    got, walls = o.bodies(), o.walls()
    dt = F(scene.dt)
    statics = {int(b["id"]) for b in start_state if b["flags"][0]}
    checked = 0
    for i, b0 in enumerate(start_state[:40]):  # the walls' owners and the first 34 movers
        if b0["flags"][0] or b0["filter"][2] or b0["ranges"][1] == 0:
            continue
        b = b0.copy()
        b["previous"][:2] = b["pose"][:2]
        b["pose"][3] = b["pose"][2]
        b["motion"][2] = b["motion"][2] * F(np.exp(np.float64(-b["motion"][3] * dt)))
        start = b["pose"][:3].copy()
        end = start + b["motion"][:3] * dt
        span = np.ceil(abs(end[2] - start[2]) / F(0.05))
        if span > 128:
            continue  # the rotation budget: checked by the safety bits elsewhere
        steps = max(1, int(span))
        r = arrays.ranges[i]
        excluded = set(int(x) for x in arrays.partners[r[2]:r[2] + r[3]])
        lerp = lambda t: start + (end - start) * t
        stop, hit = start, None
        for sample in range(steps):
            p, q = lerp(F(sample) / F(steps)), lerp(F(sample + 1) / F(steps))
            hit = np_sweep(b, p, q, scene.vertices, scene.segments, excluded)
            if hit is None:
                continue
            last, high = p, q
            for _ in range(12):
                middle = F(0.5) * (last + high)
                if np_sweep(b, p, middle, scene.vertices, scene.segments, excluded) is not None:
                    high = middle
                else:
                    last = middle
            stop = last
            break
        if hit is None:
            assert np.array_equal(got[i]["pose"][:3], end), i
            continue
        assert np.array_equal(got[i]["pose"][:3], stop), i
        assert not got[i]["motion"][:3].any()
        point, normal, owner = hit
        if owner in statics:
            closing = max(F(0), -np_dot(b["motion"][:2], normal))
            stopped = closing / b["physical"][0] * dt
            assert walls[i]["participants"].tolist() == [int(b["id"]), owner]
            assert np.array_equal(walls[i]["geometry"], np.concatenate([normal, point]).astype(F))
            assert walls[i]["extra"][0] == stopped
        checked += 1
    assert checked > 15
