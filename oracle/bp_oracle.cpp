// bp_oracle.cpp - CPU ORACLE for the bubble step. TEST INFRASTRUCTURE ONLY.
//
// This file restates, in plain scalar C++ and in the reference's operation order, the per-step bubble simulation
// of BubblePhysics v4 (Metal kernels under Sources/BubblePhysicsNativeMetal/Shaders/). It is the checker the CUDA
// path is compared against; the product never links, loads or calls it. Only tests/, __graft_entry__.smoke() and the
// cpu_baseline / reference legs of bench.py use it.
//
// It is templated on the arithmetic type: T = float is the parity build (bit-for-bit the same formulas the GPU
// runs), T = double is the FP64 rerun used to report the FP32 error. Build with -ffp-contract=off so no
// multiply-add is fused behind our back; the one explicit fma of the reference (nativePastSegmentEnd) is kept.
//
// Abbreviations in citations: NFK = NativeForceKernels.metal-source, NGK = NativeGeometryKernels.metal-source,
// NCK = NativeContactKernels.metal-source, NPK = NativePostSolveKernels.metal-source (all under
// Sources/BubblePhysicsNativeMetal/Shaders/).
//
// Deliberate, documented differences from the reference (both the oracle and the CUDA path follow them):
//  - gravity: an acceleration added to the non-contact acceleration of force-driven bubbles (the reference only has a
//    per-bubble global force; with gravity = 0 nothing changes);
//  - adjacency overflow keeps the first k neighbours in (kind, neighbour) order; the reference keeps an
//    atomic-order-dependent subset (NCK:186-195 says so itself), the dropped count is the same;
//  - the contact assertion reports the violation of the lowest bubble index (the reference: whichever thread wins a
//    compare-and-swap, NFK:848-854).

#include "../include/bubblephysics.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <new>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

template <typename T> struct V2 {
    T x, y;
};
template <typename T> inline V2<T> mk(T x, T y) { return V2<T>{x, y}; }
template <typename T> inline V2<T> operator+(V2<T> a, V2<T> b) { return {a.x + b.x, a.y + b.y}; }
template <typename T> inline V2<T> operator-(V2<T> a, V2<T> b) { return {a.x - b.x, a.y - b.y}; }
template <typename T> inline V2<T> operator*(V2<T> a, T s) { return {a.x * s, a.y * s}; }
template <typename T> inline V2<T> operator*(T s, V2<T> a) { return {s * a.x, s * a.y}; }
template <typename T> inline V2<T> operator/(V2<T> a, T s) { return {a.x / s, a.y / s}; }
template <typename T> inline V2<T> operator-(V2<T> a) { return {-a.x, -a.y}; }
template <typename T> inline T dot(V2<T> a, V2<T> b) { return a.x * b.x + a.y * b.y; }
template <typename T> inline T len(V2<T> a) { return std::sqrt(a.x * a.x + a.y * a.y); }
template <typename T> inline V2<T> vmin(V2<T> a, V2<T> b) { return {std::fmin(a.x, b.x), std::fmin(a.y, b.y)}; }
template <typename T> inline V2<T> vmax(V2<T> a, V2<T> b) { return {std::fmax(a.x, b.x), std::fmax(a.y, b.y)}; }
template <typename T> inline V2<T> vclamp(V2<T> a, V2<T> lo, V2<T> hi) { return vmin(vmax(a, lo), hi); }
template <typename T> inline T clampv(T v, T lo, T hi) { return std::fmin(std::fmax(v, lo), hi); }
template <typename T> inline bool finite2(V2<T> a) { return std::isfinite(a.x) && std::isfinite(a.y); }
template <typename T> inline T cross(V2<T> a, V2<T> b) { return a.x * b.y - a.y * b.x; }

template <typename T> struct Lim {
    static T tiny() { return std::numeric_limits<T>::min(); }  // FLT_MIN of the reference
    static T inf() { return std::numeric_limits<T>::infinity(); }
    static T big() { return std::numeric_limits<T>::max(); }   // FLT_MAX
};

constexpr uint32_t kFrameLimit = 1024;  // nativeSubstepFrameLimit, NFK:384
constexpr uint32_t kNewtonSteps = 12;   // nativePairNewtonSteps, NFK:39
constexpr uint32_t kRemovedFlag = 0x80000000u;

// ---------------------------------------------------------------------------------------------------------------
// Contact law (NFK:36-102)
// ---------------------------------------------------------------------------------------------------------------
template <typename T> struct Law {
    T force, epsA, epsB, stiffness;
};

// nativeEpsilonFromForceRatio, NFK:50-53
template <typename T> T epsilon_from_ratio(T q) {
    if (!(q > 0)) return 0;
    return T(2) * q / ((T(2) * q + T(1)) + std::sqrt(T(4) * q + T(1)));
}
// nativeRestFromForceRatio, NFK:55-57
template <typename T> T rest_from_ratio(T q) { return T(2) / (T(1) + std::sqrt(std::fmax(T(4) * q, T(0)) + T(1))); }

// nativeWallContactLaw, NFK:60-69
template <typename T> Law<T> wall_law(T K, T r, T distance) {
    Law<T> law{0, 0, 0, 0};
    T d = std::fmax(distance, r * T(1e-6));
    if (!(K > 0) || !(r > 0) || !(d < r)) return law;
    T rest = d / r;
    law.epsA = (r - d) / r;
    law.force = K * (r - d) * r / (d * d);
    law.stiffness = K * (T(1) + law.epsA) / (r * rest * rest * rest);
    return law;
}

// nativePairContactLaw, NFK:75-102
template <typename T> Law<T> pair_law(T Ka, T ra, T Kb, T rb, T distance) {
    Law<T> law{0, 0, 0, 0};
    T R = ra + rb;
    T d = std::fmax(distance, R * T(1e-6));
    T overlap = R - d;
    if (!(Ka > 0) || !(Kb > 0) || !(overlap > 0)) return law;
    T lowest = std::fmin(Ka, Kb) * overlap * R / (d * d);
    T force = lowest;
    if (Ka != Kb) {
        for (uint32_t step = 0; step < kNewtonSteps; ++step) {
            T qa = force / Ka, qb = force / Kb;
            T ea = epsilon_from_ratio(qa), eb = epsilon_from_ratio(qb);
            T rsa = rest_from_ratio(qa), rsb = rest_from_ratio(qb);
            T residual = ra * ea + rb * eb - overlap;
            T slope = ra * rsa * rsa * rsa / ((T(1) + ea) * Ka) + rb * rsb * rsb * rsb / ((T(1) + eb) * Kb);
            if (!(slope > Lim<T>::tiny())) break;
            force = std::fmax(force - residual / slope, lowest);
        }
    }
    T qa = force / Ka, qb = force / Kb;
    T ea = epsilon_from_ratio(qa), eb = epsilon_from_ratio(qb);
    T rsa = rest_from_ratio(qa), rsb = rest_from_ratio(qb);
    T compliance = ra * rsa * rsa * rsa / ((T(1) + ea) * Ka) + rb * rsb * rsb * rsb / ((T(1) + eb) * Kb);
    law.force = force;
    law.epsA = ea;
    law.epsB = eb;
    law.stiffness = compliance > Lim<T>::tiny() ? T(1) / compliance : T(0);
    return law;
}

// ---------------------------------------------------------------------------------------------------------------
// World state
// ---------------------------------------------------------------------------------------------------------------
template <typename T> struct Body {
    int64_t id;
    V2<T> pos, prev;          // end-of-step pose (after the kinematic advance) and start-of-step pose
    T angle, prevAngle;
    V2<T> vel;
    T omega;
    T radius;                 // bounding radius (physical.z)
    T coreRadius;
    uint32_t kind, flags, voff, vcount, toff, tcount, cat, mask, layer;
    T cosPrev, sinPrev, cosEnd, sinEnd;  // host-computed rotation of both poses (same in the CUDA path)
};

template <typename T> struct Field {
    V2<T> pos;
    T cosr, sinr, falloff;
    V2<T> dir;
    T strength, radius;
    uint32_t kind, voff, vcount, foff, fcount, hasFilter;
};

template <typename T> struct World {
    // configuration
    T dt, sepTol, contactTol, split;
    V2<T> rmin, rmax, globalForce, gravity;
    uint32_t limit, flags;
    int64_t injectObject;
    uint32_t injectSubstep;
    V2<T> injectPos;
    bool failed = false;

    // bubbles (sorted by id)
    uint32_t n;
    std::vector<int64_t> id;
    std::vector<V2<T>> pos, start, vel, acc, a0, ref, force;
    std::vector<T> rot, omega, mass, invMass, radius, K, gamma, margin;
    std::vector<uint32_t> flags_, cat, mask, result, layer;

    // published copy (a failed step publishes nothing)
    std::vector<V2<T>> pPos, pStart, pVel;
    std::vector<T> pRot, pOmega;
    std::vector<uint32_t> pResult, pFlags;

    // segments
    uint32_t s;
    std::vector<int64_t> sid, sowner;
    std::vector<V2<T>> sa, sb, sprev;
    std::vector<T> soutward, sallowed;
    std::vector<uint32_t> sflags, scat, smask, slayer;

    // bodies
    std::vector<Body<T>> bodies;
    std::vector<Body<T>> pBodies;
    std::vector<V2<T>> bverts;
    std::vector<uint32_t> btris;

    // forces
    std::vector<Field<T>> fields;
    std::vector<V2<T>> fverts;
    std::vector<int64_t> fids;
    std::vector<bp_band> bands;
    std::vector<bp_motor> motors;
    std::vector<uint32_t> jranges;
    std::vector<int64_t> jpartners;

    // step control (NativeSubstepControl, NFK:22-26)
    T timeX, timeY, timeZ, timeW;
    uint32_t countsX, countsY, countsZ, countsW;
    int64_t limiterObject;
    uint32_t limiterTerm;
    std::vector<T> history;
    bool traceOn = false;       // record every bubble's state after each substep (NativeMetalConfiguration.captureSubsteps)
    std::vector<T> trace;       // per substep: h, then x, y, vx, vy per bubble

    // broadphase products of the last build
    T cellWidth;
    std::vector<int64_t> cellX, cellY;
    std::vector<uint8_t> cellValid;
    // forward candidate row per bubble: pair neighbours (index > i) then segment indices, both ascending
    std::vector<std::vector<uint32_t>> rowPairs, rowSegs;
    // body rows: bubble indices ascending
    std::vector<std::vector<uint32_t>> bodyRows;
    // adjacency (kind << 30 | neighbour), sorted, capped at k
    std::vector<std::vector<uint32_t>> adj;
    uint32_t overflowBuild = 0, overflowMax = 0, maxPerObject = 0, rebuilds = 0;

    // end-of-step
    std::vector<bp_contact> contacts;
    bp_step_report lastReport{};
};

template <typename T> inline bool is_removed(const World<T>& w, uint32_t i) { return (w.flags_[i] & kRemovedFlag) != 0; }
// nativeIsStatic / nativeInverseMass / nativeIsForceDriven / nativeEffectiveVelocity, NFK:388-392
template <typename T> inline bool is_static(const World<T>& w, uint32_t i) {
    return !(w.invMass[i] > 0) || ((w.flags_[i] & BP_BUBBLE_ENABLED) && (w.flags_[i] & BP_BUBBLE_STATIC));
}
template <typename T> inline T inv_mass(const World<T>& w, uint32_t i) { return is_static(w, i) ? T(0) : w.invMass[i]; }
template <typename T> inline bool force_driven(const World<T>& w, uint32_t i) { return (w.flags_[i] & BP_BUBBLE_FORCE_DRIVEN) != 0; }
template <typename T> inline V2<T> eff_vel(const World<T>& w, uint32_t i) { return is_static(w, i) ? mk<T>(0, 0) : w.vel[i]; }

// nativeFilterAccepts, NGK:124-126
inline bool filter_accepts(uint32_t ca, uint32_t ma, uint32_t cb, uint32_t mb) { return (ca & mb) != 0 && (cb & ma) != 0; }

// nativeJointExcluded, NGK:254-258
template <typename T> bool joint_excluded(const World<T>& w, uint32_t entity, int64_t partner) {
    if (entity >= w.jranges.size() / 2) return false;
    uint32_t start = w.jranges[2 * entity], count = w.jranges[2 * entity + 1];
    for (uint32_t i = 0; i < count; ++i)
        if (w.jpartners[start + i] == partner) return true;
    return false;
}

// ---------------------------------------------------------------------------------------------------------------
// Geometry helpers (NGK:430-500, 660-681)
// ---------------------------------------------------------------------------------------------------------------
// nativeClosestPoint, NGK:437-441
template <typename T> V2<T> closest_point(V2<T> p, V2<T> a, V2<T> b) {
    V2<T> edge = b - a;
    T square = dot(edge, edge);
    T t = square > Lim<T>::tiny() ? clampv(dot(p - a, edge) / square, T(0), T(1)) : T(0);
    return a + edge * t;
}
// nativePastSegmentEnd, NGK:665-668 (explicit fma)
template <typename T> bool past_segment_end(V2<T> center, V2<T> from, V2<T> to) {
    V2<T> edge = to - from, rel = center - from;
    return std::fma(rel.x, edge.x, rel.y * edge.y) >= std::fma(edge.x, edge.x, edge.y * edge.y);
}
template <typename T> V2<T> rotate_cs(V2<T> p, T c, T s) { return {p.x * c - p.y * s, p.x * s + p.y * c}; }

// nativeWallRegion, NFK:112-136
template <typename T> bool wall_region(const World<T>& w, uint32_t si, V2<T> center, V2<T>& normal, T& distance) {
    V2<T> start = w.sa[si], end = w.sb[si], edge = end - start;
    T edgeLength = len(edge);
    V2<T> base = edgeLength > 0 ? mk(-edge.y, edge.x) / edgeLength : mk<T>(0, 1);
    if (w.sflags[si] & BP_SEGMENT_POLYGON_EDGE) {
        V2<T> outward = base * w.soutward[si];
        T along = dot(center - start, edge);
        bool convexStart = (w.sflags[si] & BP_SEGMENT_CONVEX_START) != 0;
        if (convexStart && along <= 0 && past_segment_end(center, w.sprev[si], start)) {
            V2<T> delta = center - start;
            distance = len(delta);
            normal = distance > 0 ? delta / distance : outward;
        } else if (along > 0 && !past_segment_end(center, start, end) && dot(center - start, outward) >= 0) {
            normal = outward;
            distance = dot(center - start, outward);
        } else {
            return false;
        }
    } else {
        V2<T> delta = center - closest_point(center, start, end);
        distance = len(delta);
        normal = distance > 0 ? delta / distance : base;
    }
    return true;
}
template <typename T> bool wall_contact(const World<T>& w, uint32_t si, V2<T> center, T radius, V2<T>& normal, T& d) {
    return wall_region(w, si, center, normal, d) && d < radius;
}

// Body pose at a fraction of the step (nativeBodyAtFraction, NFK:155-159) with its rotation.
template <typename T> struct Pose {
    V2<T> pos;
    T c, s;
};
template <typename T> Pose<T> body_at(const Body<T>& b, T fraction) {
    Pose<T> p;
    p.pos = b.prev + (b.pos - b.prev) * fraction;
    T angle = b.prevAngle + (b.angle - b.prevAngle) * fraction;
    if (angle == b.prevAngle) { p.c = b.cosPrev; p.s = b.sinPrev; }
    else if (angle == b.angle) { p.c = b.cosEnd; p.s = b.sinEnd; }
    else { p.c = std::cos(angle); p.s = std::sin(angle); }
    return p;
}
template <typename T> V2<T> body_vertex(const World<T>& w, const Body<T>& b, const Pose<T>& p, uint32_t i) {
    return p.pos + rotate_cs(w.bverts[b.voff + i], p.c, p.s);
}
// nativeRigidInside, NGK:477-490
template <typename T> bool rigid_inside(const World<T>& w, V2<T> pt, const Body<T>& b, const Pose<T>& p) {
    if (b.kind != BP_BODY_POLYGON) {
        V2<T> ca = body_vertex(w, b, p, 0), cb = b.vcount > 1 ? body_vertex(w, b, p, 1) : ca;
        return len(pt - closest_point(pt, ca, cb)) <= b.coreRadius;
    }
    V2<T> local = rotate_cs(pt - p.pos, p.c, -p.s);
    for (uint32_t i = 0; i < b.tcount; ++i) {
        const uint32_t* t = &w.btris[3 * (b.toff + i)];
        V2<T> a = w.bverts[b.voff + t[0]], bb = w.bverts[b.voff + t[1]], c = w.bverts[b.voff + t[2]];
        if (cross(bb - a, local - a) >= 0 && cross(c - bb, local - bb) >= 0 && cross(a - c, local - c) >= 0) return true;
    }
    return false;
}

template <typename T> struct Obstacle {
    V2<T> normal;
    T distance;
    V2<T> velocity;
    T speedBound;
};
// nativeBodyObstacle, NFK:170-210
template <typename T> Obstacle<T> body_obstacle(const World<T>& w, const Body<T>& b, T fraction, V2<T> center) {
    Pose<T> p = body_at(b, fraction);
    Obstacle<T> o;
    V2<T> point, normal;
    T distance;
    if (b.kind != BP_BODY_POLYGON) {
        V2<T> ca = body_vertex(w, b, p, 0), cb = b.vcount > 1 ? body_vertex(w, b, p, 1) : ca;
        point = closest_point(center, ca, cb);
        V2<T> delta = center - point;
        T away = len(delta);
        V2<T> axis = cb - ca;
        T axisLength = len(axis);
        V2<T> fallback = axisLength > T(1e-6) ? mk(-axis.y, axis.x) / axisLength : mk<T>(0, 1);
        normal = away > T(1e-7) ? delta / away : fallback;
        distance = away - b.coreRadius;
        point = point + normal * b.coreRadius;
    } else {
        T best = Lim<T>::inf();
        V2<T> nearest = mk<T>(0, 0), outward = mk<T>(0, 1);
        for (uint32_t e = 0; e < b.vcount; ++e) {
            V2<T> pp = body_vertex(w, b, p, e), q = body_vertex(w, b, p, (e + 1) % b.vcount);
            V2<T> cand = closest_point(center, pp, q);
            T d = len(center - cand);
            if (d < best) {
                best = d;
                nearest = cand;
                V2<T> edge = q - pp;
                T size = len(edge);
                outward = size > Lim<T>::tiny() ? mk(edge.y, -edge.x) / size : mk<T>(0, 1);
            }
        }
        bool inside = rigid_inside(w, center, b, p);
        normal = inside ? outward : (best > T(1e-7) ? (center - nearest) / best : outward);
        distance = inside ? -best : best;
        point = nearest;
    }
    V2<T> arm = point - p.pos;
    o.normal = normal;
    o.distance = distance;
    o.velocity = b.vel + mk(-arm.y, arm.x) * b.omega;
    o.speedBound = len(b.vel) + std::fabs(b.omega) * len(arm);
    return o;
}

// ---------------------------------------------------------------------------------------------------------------
// Non-contact acceleration (NFK:389-470)
// ---------------------------------------------------------------------------------------------------------------
template <typename T> V2<T> field_force(const World<T>& w, const Field<T>& f, V2<T> point) {
    V2<T> delta = point - f.pos;
    T c = f.cosr, s = f.sinr;
    V2<T> local = mk(c * delta.x + s * delta.y, -s * delta.x + c * delta.y);
    T distance = len(local), radius = f.radius;
    if (f.vcount == 0) {
        if (!(distance <= radius)) return mk<T>(0, 0);
    } else {
        bool inside = false;
        for (uint32_t i = 0; i < f.vcount; ++i) {
            V2<T> a = w.fverts[f.voff + i], b = w.fverts[f.voff + (i + 1) % f.vcount];
            if ((a.y > local.y) != (b.y > local.y) && local.x < (b.x - a.x) * (local.y - a.y) / (b.y - a.y) + a.x) inside = !inside;
        }
        if (!inside) return mk<T>(0, 0);
    }
    if (f.kind == 0) return mk(c * f.dir.x - s * f.dir.y, s * f.dir.x + c * f.dir.y);
    if (!(distance > 0)) return mk<T>(0, 0);
    T profile = f.falloff == 0 ? T(1) : std::pow(std::fmax(T(0), T(1) - distance / radius), f.falloff);
    T scale = f.strength * profile / distance;
    return f.kind == 2 ? mk(-delta.y, delta.x) * scale : delta * scale;
}
template <typename T> bool field_affects(const World<T>& w, const Field<T>& f, int64_t id) {
    if (!f.hasFilter) return true;
    uint32_t low = f.foff, end = f.foff + f.fcount, high = end;
    while (low < high) {
        uint32_t mid = low + (high - low) / 2;
        if (w.fids[mid] < id) low = mid + 1; else high = mid;
    }
    return low < end && w.fids[low] == id;
}
template <typename R> const R* find_by_bubble(const std::vector<R>& v, int64_t id) {
    uint32_t low = 0, high = (uint32_t)v.size();
    while (low < high) {
        uint32_t mid = low + (high - low) / 2;
        if (v[mid].bubble_id < id) low = mid + 1; else high = mid;
    }
    return low < v.size() && v[low].bubble_id == id ? &v[low] : nullptr;
}
// nativeNonContactAcceleration, NFK:450-470 (+ the gravity acceleration of this framework)
template <typename T> V2<T> non_contact_acc(const World<T>& w, uint32_t i, V2<T> position) {
    T im = inv_mass(w, i);
    if (!force_driven(w, i) || !(im > 0)) return mk<T>(0, 0);
    V2<T> f = w.globalForce;
    int64_t id = w.id[i];
    for (const Field<T>& fl : w.fields)
        if (field_affects(w, fl, id)) f = f + field_force(w, fl, position);
    if (!w.bands.empty()) {
        const bp_band* band = find_by_bubble(w.bands, id);
        if (band) {
            V2<T> bf = (mk<T>(band->target[0], band->target[1]) - position) * T(band->stiffness);
            T lim = band->maximum_force, magnitude = len(bf);
            if (lim > 0 && magnitude > lim) bf = bf * (lim / magnitude);
            f = f + bf;
        }
    }
    if (!w.motors.empty()) {
        const bp_motor* motor = find_by_bubble(w.motors, id);
        if (motor) f = f + mk<T>(motor->force[0], motor->force[1]);
    }
    V2<T> a = f * im;
    if (w.gravity.x != 0 || w.gravity.y != 0) a = a + w.gravity;
    return a;
}

// ---------------------------------------------------------------------------------------------------------------
// Broadphase (NFK:492-506, NGK:163-426, NCK:181-246, NFK:298-331)
// ---------------------------------------------------------------------------------------------------------------
template <typename T> void broadphase(World<T>& w) {
    const uint32_t n = w.n, k = w.limit;
    // a0, margin, x0 (nativeBubbleAcceleration + nativeBubbleMargin, NFK:472-499)
    T t = std::fmax(w.timeX - w.timeY, T(0));
    for (uint32_t i = 0; i < n; ++i) {
        w.a0[i] = non_contact_acc(w, i, w.pos[i]);
        T travel = len(eff_vel(w, i)) * t + T(0.5) * len(w.a0[i]) * t * t;
        w.margin[i] = (w.flags & BP_WORLD_MINIMUM_MARGIN_ONLY) ? T(0.25) * w.radius[i]
                                                              : std::fmax(T(1.05) * travel, T(0.25) * w.radius[i]);
        w.ref[i] = w.pos[i];
    }
    // cell width (nativePrepareGrid, NGK:163-177)
    T cw = w.sepTol;
    for (uint32_t i = 0; i < n; ++i) {
        if (is_removed(w, i)) continue;
        cw = std::fmax(cw, T(2) * (w.radius[i] + w.margin[i]) + w.sepTol);
    }
    cw = std::fmax(cw, Lim<T>::tiny());
    w.cellWidth = cw;
    // cells (nativeBuildGrid, NGK:179-189)
    std::vector<uint32_t> order;
    order.reserve(n);
    for (uint32_t i = 0; i < n; ++i) {
        bool valid = !is_removed(w, i) && finite2(w.pos[i]);
        w.cellValid[i] = valid;
        if (valid) {
            T fx = std::floor(w.pos[i].x / cw), fy = std::floor(w.pos[i].y / cw);
            const T lim = T(4.0e18);
            w.cellX[i] = (int64_t)clampv(fx, -lim, lim);
            w.cellY[i] = (int64_t)clampv(fy, -lim, lim);
            order.push_back(i);
        } else {
            w.cellX[i] = 0;
            w.cellY[i] = 0;
        }
    }
    // sort by (cell.x, cell.y, index) (nativeGridLess, NGK:191-196)
    std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
        if (w.cellX[a] != w.cellX[b]) return w.cellX[a] < w.cellX[b];
        if (w.cellY[a] != w.cellY[b]) return w.cellY[a] < w.cellY[b];
        return a < b;
    });
    uint32_t buildOverflow = 0;
    // candidate rows (nativeEmitBubbleCandidates + nativeFinishBubbleRow, NGK:262-330)
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : buildOverflow) if (n > 4096)
    for (uint32_t i = 0; i < n; ++i) {
        std::vector<uint32_t>& rp = w.rowPairs[i];
        std::vector<uint32_t>& rs = w.rowSegs[i];
        rp.clear();
        rs.clear();
        if (!w.cellValid[i] || !finite2(w.start[i])) continue;
        int64_t cx = w.cellX[i], cy = w.cellY[i];
        for (int dx = -1; dx <= 1; ++dx) {
            int64_t tx = cx + dx, ty = cy - 1;
            // lower bound of (tx, ty) in the sorted grid
            uint32_t low = 0, high = (uint32_t)order.size();
            while (low < high) {
                uint32_t mid = low + (high - low) / 2;
                uint32_t e = order[mid];
                if (w.cellX[e] < tx || (w.cellX[e] == tx && w.cellY[e] < ty)) low = mid + 1; else high = mid;
            }
            for (uint32_t q = low; q < order.size() && w.cellX[order[q]] == tx && w.cellY[order[q]] <= ty + 2; ++q) {
                uint32_t j = order[q];
                if (j <= i) continue;
                // nativeBubblePairCandidate, NGK:262-273
                if (!filter_accepts(w.cat[i], w.mask[i], w.cat[j], w.mask[j])) continue;
                if (joint_excluded(w, i, w.id[j])) continue;
                T reach = w.radius[i] + w.radius[j] + w.margin[i] + w.margin[j] + w.sepTol;
                if (std::fabs(w.pos[i].x - w.pos[j].x) <= reach && std::fabs(w.pos[i].y - w.pos[j].y) <= reach) rp.push_back(j);
            }
        }
        std::sort(rp.begin(), rp.end());
        // segments (nativeFinishBubbleRow, NGK:276-290)
        for (uint32_t j = 0; j < w.s; ++j) {
            if (!filter_accepts(w.cat[i], w.mask[i], w.scat[j], w.smask[j])) continue;
            if ((w.sflags[j] & BP_SEGMENT_HAS_OWNER) && joint_excluded(w, i, w.sowner[j])) continue;
            T reach = w.radius[i] + w.margin[i] + w.sepTol;
            V2<T> lower = vmin(w.sa[j], w.sb[j]) - mk(reach, reach);
            V2<T> upper = vmax(w.sa[j], w.sb[j]) + mk(reach, reach);
            V2<T> p = w.pos[i];
            if (p.x >= lower.x && p.y >= lower.y && p.x <= upper.x && p.y <= upper.y) rs.push_back(j);
        }
        // keep the k smallest keys (nativeInsertCandidate, NGK:238-251): pairs sort before segments
        uint32_t total = (uint32_t)(rp.size() + rs.size());
        if (total > k) {
            buildOverflow += total - k;
            if (rp.size() >= k) { rp.resize(k); rs.clear(); }
            else rs.resize(k - rp.size());
        }
#pragma omp critical
        w.maxPerObject = std::max(w.maxPerObject, total);
    }
    // body rows (nativeEmitBodyCandidates, NGK:350-415, mode bit 1 = no body pairs)
    for (size_t b = 0; b < w.bodies.size(); ++b) {
        const Body<T>& body = w.bodies[b];
        std::vector<uint32_t>& row = w.bodyRows[b];
        row.clear();
        bool obstacle = (body.flags & BP_BODY_STATIC) ? body.kind != BP_BODY_POLYGON : (body.flags & BP_BODY_KINEMATIC) != 0;
        if (!obstacle) continue;
        V2<T> bodyLow = vmin(body.pos, body.prev) - mk(body.radius, body.radius);
        V2<T> bodyHigh = vmax(body.pos, body.prev) + mk(body.radius, body.radius);
        uint32_t entity = n + (uint32_t)b;
        uint32_t total = 0;
        for (uint32_t a = 0; a < n; ++a) {
            if (is_removed(w, a)) continue;
            if (!filter_accepts(w.cat[a], w.mask[a], body.cat, body.mask)) continue;
            if (joint_excluded(w, entity, w.id[a])) continue;
            T reach = w.radius[a] + std::fmax(w.margin[a], T(0));
            V2<T> lo = w.pos[a] - mk(reach, reach), hi = w.pos[a] + mk(reach, reach);
            bool hit = !(hi.x < bodyLow.x || hi.y < bodyLow.y || bodyHigh.x < lo.x || bodyHigh.y < lo.y);
            if (!hit) continue;
            ++total;
            if (row.size() < k) row.push_back(a);
        }
        if (total > k) buildOverflow += total - k;
        w.maxPerObject = std::max(w.maxPerObject, total);
    }
    // adjacency (nativeEmitCandidateEdges + nativeEmitBodyEdges + nativeBuildAdjacencyRow)
    for (uint32_t i = 0; i < n; ++i) w.adj[i].clear();
    for (uint32_t i = 0; i < n; ++i) {
        for (uint32_t j : w.rowPairs[i]) {
            w.adj[i].push_back(j);
            w.adj[j].push_back(i);
        }
        for (uint32_t sg : w.rowSegs[i]) w.adj[i].push_back((1u << 30) | sg);
    }
    for (size_t b = 0; b < w.bodies.size(); ++b)
        for (uint32_t a : w.bodyRows[b]) w.adj[a].push_back((2u << 30) | (uint32_t)b);
    for (uint32_t i = 0; i < n; ++i) {
        std::vector<uint32_t>& row = w.adj[i];
        std::sort(row.begin(), row.end());  // (kind, neighbour) order: kind is in the top bits
        uint32_t demanded = (uint32_t)row.size();
        if (demanded > k) {
            buildOverflow += demanded - k;
            row.resize(k);
        }
        w.maxPerObject = std::max(w.maxPerObject, demanded);
    }
    w.overflowBuild = buildOverflow;
}

// ---------------------------------------------------------------------------------------------------------------
// Substep functions
// ---------------------------------------------------------------------------------------------------------------
template <typename T> T step_fraction(const World<T>& w) {
    return w.timeX > 0 ? clampv(w.timeY / w.timeX, T(0), T(1)) : T(1);  // nativeStepFraction, NFK:150-152
}

// nativeBubbleContactForce, NFK:216-243
template <typename T> V2<T> contact_force(const World<T>& w, uint32_t i, T fraction) {
    V2<T> total = mk<T>(0, 0);
    T radius = w.radius[i], K = w.K[i];
    for (uint32_t e : w.adj[i]) {
        uint32_t kind = e >> 30, j = e & 0x3fffffffu;
        if (kind == 0) {
            uint32_t low = std::min(i, j), high = std::max(i, j);
            V2<T> delta = w.pos[high] - w.pos[low];
            T d = len(delta);
            V2<T> normal = d > 0 ? delta / d : mk<T>(1, 0);
            Law<T> law = pair_law(w.K[low], w.radius[low], w.K[high], w.radius[high], d);
            total = total + normal * (i == low ? -law.force : law.force);
        } else if (kind == 1) {
            V2<T> normal;
            T d;
            if (!wall_contact(w, j, w.pos[i], radius, normal, d)) continue;
            total = total + normal * wall_law(K, radius, d).force;
        } else {
            Obstacle<T> o = body_obstacle(w, w.bodies[j], fraction, w.pos[i]);
            total = total + o.normal * wall_law(K, radius, o.distance).force;
        }
    }
    return total;
}

// nativeBubbleOmegaSquared, NFK:510-541
template <typename T> T omega_squared(const World<T>& w, uint32_t i, T fraction) {
    T im = inv_mass(w, i);
    if (!(im > 0)) return 0;
    T radius = w.radius[i], K = w.K[i], total = 0;
    if (!w.bands.empty()) {
        const bp_band* band = find_by_bubble(w.bands, w.id[i]);
        if (band) total = total + T(band->stiffness) * im;
    }
    for (uint32_t e : w.adj[i]) {
        uint32_t kind = e >> 30, j = e & 0x3fffffffu;
        if (kind == 0) {
            uint32_t low = std::min(i, j), high = std::max(i, j);
            T d = len(w.pos[high] - w.pos[low]);
            Law<T> law = pair_law(w.K[low], w.radius[low], w.K[high], w.radius[high], d);
            total = total + law.stiffness * (im + std::sqrt(im * inv_mass(w, j)));
        } else if (kind == 1) {
            V2<T> normal;
            T d;
            if (!wall_contact(w, j, w.pos[i], radius, normal, d)) continue;
            total = total + wall_law(K, radius, d).stiffness * im;
        } else {
            Obstacle<T> o = body_obstacle(w, w.bodies[j], fraction, w.pos[i]);
            total = total + wall_law(K, radius, o.distance).stiffness * im;
        }
    }
    return total;
}

// nativeBubbleDistanceBound, NFK:550-598
template <typename T> T distance_bound(const World<T>& w, uint32_t i, T hMax, T fraction) {
    if (!(inv_mass(w, i) > 0)) return Lim<T>::inf();
    V2<T> velocity = w.vel[i];
    T radius = w.radius[i], best = Lim<T>::inf();
    for (uint32_t e : w.adj[i]) {
        uint32_t kind = e >> 30, j = e & 0x3fffffffu;
        T distance, approach, accSum, reach, bodySpeed = 0;
        if (kind == 0) {
            V2<T> delta = w.pos[j] - w.pos[i];
            distance = len(delta);
            V2<T> normal = distance > 0 ? delta / distance : mk<T>(1, 0);
            approach = dot(velocity - eff_vel(w, j), normal);
            accSum = len(w.acc[i]) + len(w.acc[j]);
            reach = radius + w.radius[j];
        } else if (kind == 1) {
            V2<T> normal;
            if (!wall_region(w, j, w.pos[i], normal, distance)) continue;
            approach = -dot(velocity, normal);
            accSum = len(w.acc[i]);
            reach = radius;
        } else {
            Obstacle<T> o = body_obstacle(w, w.bodies[j], fraction, w.pos[i]);
            distance = o.distance;
            approach = -dot(velocity, o.normal);
            bodySpeed = o.speedBound;
            accSum = len(w.acc[i]);
            reach = radius;
        }
        bool active = distance < reach;
        T d = std::fmax(distance, reach * T(1e-6));
        T speed;
        if (active) speed = std::fabs(approach) + bodySpeed;
        else {
            if (approach + bodySpeed + accSum * hMax * T(0.5) <= 0) continue;
            speed = approach + bodySpeed;
        }
        T sq = std::sqrt(speed * speed + accSum * d * T(0.5));
        T denominator = sq + speed;
        if (!(denominator > 0)) continue;
        best = std::fmin(best, d / (T(2) * denominator));
    }
    return best;
}

// nativeBubbleMarginBound, NFK:604-614
template <typename T> T margin_bound(const World<T>& w, uint32_t i) {
    if (!(inv_mass(w, i) > 0)) return Lim<T>::inf();
    T left = w.margin[i] - len(w.pos[i] - w.ref[i]);
    if (std::isnan(left)) return Lim<T>::inf();
    if (left <= 0) return 0;
    T speed = len(w.vel[i]), a = len(w.acc[i]);
    T denominator = speed + std::sqrt(speed * speed + T(2) * a * left);
    return denominator > 0 ? T(2) * left / denominator : Lim<T>::inf();
}

// nativeHalfImpulseFactor, NFK:754-758
template <typename T> T half_impulse(T gamma, T halfStep) {
    T x = gamma * halfStep;
    if (x < T(0.05))
        return halfStep * (T(1) - x * T(0.5) + x * x * (T(1) / T(6)) - x * x * x * (T(1) / T(24)) + x * x * x * x * (T(1) / T(120)));
    return (T(1) - std::exp(-x)) / gamma;
}

// All bubble-level phases skip removed bubbles: the reference host drops them from the world.
template <typename T> void contact_forces_all(World<T>& w) {
    T fraction = step_fraction(w);
#pragma omp parallel for schedule(static) if (w.n > 4096)
    for (uint32_t i = 0; i < w.n; ++i) w.force[i] = is_removed(w, i) ? mk<T>(0, 0) : contact_force(w, i, fraction);
}

// nativeIntegratePhase, NFK:765-802
template <typename T> void integrate(World<T>& w, uint32_t phase) {
#pragma omp parallel for schedule(static) if (w.n > 4096)
    for (uint32_t i = 0; i < w.n; ++i) {
        if (is_removed(w, i)) continue;
        T im = inv_mass(w, i);
        if (phase == 2) {
            w.acc[i] = w.force[i] * im + w.a0[i];
            continue;
        }
        T h = w.timeZ;
        if (!(h > 0)) continue;
        T halfStep = T(0.5) * h;
        T gamma = force_driven(w, i) ? std::fmax(w.gamma[i], T(0)) : T(0);
        T decay = std::exp(-gamma * halfStep), factor = half_impulse(gamma, halfStep);
        if (phase == 0) {
            if (!(im > 0)) continue;
            V2<T> velocity = w.vel[i] * decay + w.acc[i] * factor;
            T angular = w.omega[i] * std::exp(-gamma * h);
            if (!w.motors.empty() && force_driven(w, i)) {
                const bp_motor* motor = find_by_bubble(w.motors, w.id[i]);
                if (motor && motor->inertia > 0) angular = angular + T(motor->torque) / T(motor->inertia) * half_impulse(gamma, h);
            }
            w.pos[i] = w.pos[i] + velocity * h;
            w.rot[i] = w.rot[i] + w.omega[i] * h;
            w.vel[i] = velocity;
            w.omega[i] = angular;
            continue;
        }
        if (im > 0) {
            V2<T> a = w.force[i] * im + non_contact_acc(w, i, w.pos[i]);
            w.vel[i] = w.vel[i] * decay + a * factor;
            w.acc[i] = a;
        }
    }
}

// nativeReduceSubstepInGroup, NFK:625-736 (reductions: max / min with the lower index winning ties)
template <typename T> void reduce(World<T>& w) {
    T remaining = w.timeX - w.timeY;
    bool over = !(remaining > 0), stopped = w.countsZ != 0 || w.countsW != 0;
    bool limited = w.countsY >= kFrameLimit;
    if (over || stopped || limited) {
        if (limited && !over && !stopped) w.countsW = 1;
        w.timeZ = 0;
        return;
    }
    const uint32_t n = w.n;
    T fraction = step_fraction(w);
    std::vector<T> v1(n), v2(n), v3(n);
#pragma omp parallel for schedule(static) if (n > 4096)
    for (uint32_t i = 0; i < n; ++i) {
        v1[i] = is_removed(w, i) ? T(-1) : omega_squared(w, i, fraction);
        v3[i] = is_removed(w, i) ? Lim<T>::inf() : margin_bound(w, i);
    }
    T best = -1;
    uint32_t owner = 0;
    for (uint32_t i = 0; i < n; ++i)
        if (v1[i] > best) { best = v1[i]; owner = i; }
    T omegaSq = best;
    uint32_t omegaOwner = owner;
    T stiffnessBound = omegaSq > 0 ? T(1) / std::sqrt(omegaSq) : Lim<T>::inf();
    T hMax = std::fmin(remaining, stiffnessBound);
#pragma omp parallel for schedule(static) if (n > 4096)
    for (uint32_t i = 0; i < n; ++i) v2[i] = is_removed(w, i) ? Lim<T>::inf() : distance_bound(w, i, hMax, fraction);
    best = Lim<T>::inf();
    owner = 0;
    for (uint32_t i = 0; i < n; ++i)
        if (v2[i] < best) { best = v2[i]; owner = i; }
    T distanceBound = best;
    uint32_t distanceOwner = owner;
    best = Lim<T>::inf();
    owner = 0;
    for (uint32_t i = 0; i < n; ++i)
        if (v3[i] < best) { best = v3[i]; owner = i; }
    T marginBound = best;
    uint32_t marginOwner = owner;
    if (marginBound <= 0) {
        w.countsZ = 1;
        w.timeZ = 0;
        w.limiterObject = w.id[marginOwner];
        w.limiterTerm = BP_TERM_MARGIN;
        return;
    }
    T split = std::fmax(w.timeW, T(1));
    T h = remaining;
    uint32_t term = BP_TERM_REMAINING;
    int64_t object = 0;
    if (split > 1 && w.timeX / split < h) h = w.timeX / split;
    if (stiffnessBound / split < h) { h = stiffnessBound / split; term = BP_TERM_STIFFNESS; object = w.id[omegaOwner]; }
    if (distanceBound / split < h) { h = distanceBound / split; term = BP_TERM_DISTANCE; object = w.id[distanceOwner]; }
    if (marginBound < h) { h = marginBound; term = BP_TERM_MARGIN; object = w.id[marginOwner]; w.countsZ = 1; }
    h = std::fmax(h, w.timeX * T(1e-7));
    uint32_t frameSubstep = w.countsY;
    if (h >= remaining || remaining - h <= w.timeX * T(1e-5)) { h = remaining; w.timeY = w.timeX; }
    else w.timeY = w.timeY + h;
    w.timeZ = h;
    w.countsX += 1;
    w.countsY = frameSubstep + 1;
    w.limiterObject = object;
    w.limiterTerm = term;
    w.history.push_back(h);
}

// ---------------------------------------------------------------------------------------------------------------
// Contact assertion (NFK:865-918): violation of the lowest bubble index.
// ---------------------------------------------------------------------------------------------------------------
struct Violation {
    uint32_t kind = 0;
    uint32_t index = 0xffffffffu;
    int64_t a = 0, b = 0, edge = 0;
    double distance = 0;
};

template <typename T> bool assert_bubble(const World<T>& w, uint32_t i, const std::vector<uint32_t>* sameCell, Violation& v) {
    V2<T> center = w.pos[i], start = w.start[i];
    if (!finite2(center) || w.result[i] == 1 || is_removed(w, i)) return false;
    bool movable = inv_mass(w, i) > 0;
    auto checkPair = [&](uint32_t other) -> bool {
        if (is_removed(w, other) || w.result[other] == 1) return false;
        if (!filter_accepts(w.cat[i], w.mask[i], w.cat[other], w.mask[other])) return false;
        if (!movable && !(inv_mass(w, other) > 0)) return false;
        T d = len(w.pos[other] - center);
        if (d <= 0) {
            v.kind = BP_VIOLATION_PAIR; v.index = i; v.a = w.id[i]; v.b = w.id[other]; v.distance = (double)d;
            return true;
        }
        return false;
    };
    if (sameCell) {
        for (uint32_t other : *sameCell)
            if (other > i && checkPair(other)) return true;
    } else {
        for (uint32_t other = i + 1; other < w.n; ++other)
            if (checkPair(other)) return true;
    }
    if (!movable) return false;
    T fraction = step_fraction(w);
    for (const Body<T>& b : w.bodies) {
        if (!filter_accepts(w.cat[i], w.mask[i], b.cat, b.mask)) continue;
        if (rigid_inside(w, center, b, body_at(b, fraction))) {
            v.kind = BP_VIOLATION_INSIDE_BODY; v.index = i; v.a = w.id[i]; v.b = b.id;
            return true;
        }
    }
    for (uint32_t e = 0; e < w.s; ++e) {
        if (!(w.sflags[e] & BP_SEGMENT_POLYGON_EDGE) || !filter_accepts(w.cat[i], w.mask[i], w.scat[e], w.smask[e])) continue;
        V2<T> edge = w.sb[e] - w.sa[e];
        T lsq = dot(edge, edge);
        if (!(lsq > 0)) continue;
        V2<T> outward = mk(-edge.y, edge.x) / std::sqrt(lsq) * w.soutward[e];
        T before = dot(start - w.sa[e], outward), after = dot(center - w.sa[e], outward);
        if (!(before > 0) || !(after <= 0)) continue;
        V2<T> crossing = start + (center - start) * (before / (before - after));
        T along = dot(crossing - w.sa[e], edge) / lsq;
        if (along < 0 || along > 1) continue;
        v.kind = BP_VIOLATION_EDGE_SIDE; v.index = i; v.a = w.id[i]; v.b = w.sowner[e]; v.edge = w.sid[e]; v.distance = (double)after;
        return true;
    }
    return false;
}

// Pairs with d <= 0 have (numerically) coincident centres, so only bubbles of the same exact centre bit pattern or
// within 1e-18 can violate. Large worlds group candidates by a coarse cell of the final positions first.
template <typename T> Violation assert_contacts(const World<T>& w) {
    Violation v;
    const uint32_t n = w.n;
    if (n <= 8192) {
        for (uint32_t i = 0; i < n; ++i)
            if (assert_bubble(w, i, nullptr, v)) return v;
        return v;
    }
    // coarse grid of final centres (cell 1.0); a pair with |delta| < 1 is in the same or an adjacent cell
    std::vector<std::pair<std::pair<int64_t, int64_t>, uint32_t>> cells;
    cells.reserve(n);
    for (uint32_t i = 0; i < n; ++i)
        if (finite2(w.pos[i]))
            cells.push_back({{(int64_t)clampv(std::floor((double)w.pos[i].x), -4.0e18, 4.0e18),
                              (int64_t)clampv(std::floor((double)w.pos[i].y), -4.0e18, 4.0e18)}, i});
    std::sort(cells.begin(), cells.end());
    std::vector<std::vector<uint32_t>> near(n);
    for (size_t a = 0; a < cells.size(); ++a) {
        for (int dx = -1; dx <= 1; ++dx)
            for (int dy = -1; dy <= 1; ++dy) {
                std::pair<int64_t, int64_t> key{cells[a].first.first + dx, cells[a].first.second + dy};
                auto it = std::lower_bound(cells.begin(), cells.end(), std::make_pair(key, 0u));
                for (; it != cells.end() && it->first == key; ++it) near[cells[a].second].push_back(it->second);
            }
        std::sort(near[cells[a].second].begin(), near[cells[a].second].end());
    }
    for (uint32_t i = 0; i < n; ++i)
        if (assert_bubble(w, i, &near[i], v)) return v;
    return v;
}

// ---------------------------------------------------------------------------------------------------------------
// End of step: region (NPK:536-568), contact records (NGK:683-728, NCK:146-160, NFK:261-280), finite check (NPK:5-27)
// ---------------------------------------------------------------------------------------------------------------
template <typename T> bool apply_region(World<T>& w, uint32_t& removed, uint32_t& wrapped) {
    bool finite = true;
    for (uint32_t i = 0; i < w.n; ++i) {
        if (is_removed(w, i)) continue;
        uint32_t f = w.flags_[i];
        if (!(f & BP_BUBBLE_ENABLED) || (f & BP_BUBBLE_STATIC)) continue;
        V2<T> nearest = vclamp(w.pos[i], w.rmin, w.rmax);
        T r = w.radius[i];
        if (len(w.pos[i] - nearest) <= r) continue;
        if (!(f & BP_BUBBLE_WRAP)) { w.result[i] = 1; ++removed; continue; }
        V2<T> delta = mk<T>(0, 0);
        V2<T> span = (w.rmax - w.rmin) + mk(T(2) * r, T(2) * r);
        T p[2] = {w.pos[i].x, w.pos[i].y}, lo[2] = {w.rmin.x, w.rmin.y}, hi[2] = {w.rmax.x, w.rmax.y}, sp[2] = {span.x, span.y};
        T dl[2] = {0, 0};
        for (int axis = 0; axis < 2; ++axis) {
            if (p[axis] > hi[axis]) dl[axis] = -sp[axis] * std::fmax(T(1), std::ceil((p[axis] - r - hi[axis]) / sp[axis]));
            else if (p[axis] < lo[axis]) dl[axis] = sp[axis] * std::fmax(T(1), std::ceil((lo[axis] - r - p[axis]) / sp[axis]));
        }
        delta = mk(dl[0], dl[1]);
        V2<T> wrappedPos = w.pos[i] + delta;
        V2<T> nearestWrapped = vclamp(wrappedPos, w.rmin, w.rmax);
        if (len(wrappedPos - nearestWrapped) > r) delta = delta + (nearestWrapped - wrappedPos);
        w.pos[i] = w.pos[i] + delta;
        w.start[i] = w.start[i] + delta;
        if (!finite2(w.pos[i]) || !finite2(w.start[i])) { finite = false; continue; }
        w.result[i] = 2;
        ++wrapped;
    }
    return finite;
}

template <typename T> void build_contacts(World<T>& w) {
    w.contacts.clear();
    T dt = w.timeX;
    auto record = [&](uint32_t ai, uint32_t kind, uint32_t other) {
        V2<T> apos = w.pos[ai];
        T ar = w.radius[ai];
        V2<T> normal, point;
        T pen, allowed = 0;
        uint32_t feature = 0;
        int64_t second;
        if (kind == 0) {
            V2<T> delta = w.pos[other] - apos;
            T d = len(delta);
            normal = d > 0 ? delta / d : mk<T>(1, 0);
            point = apos + normal * ar;
            pen = ar + w.radius[other] - d;
            second = w.id[other];
        } else {
            uint32_t s = other;
            second = w.sid[s];
            V2<T> edge = w.sb[s] - w.sa[s];
            T lsq = dot(edge, edge);
            T t = lsq > 0 ? clampv(dot(apos - w.sa[s], edge) / lsq, T(0), T(1)) : T(0);
            point = w.sa[s] + edge * t;
            V2<T> delta = apos - point;
            T d = len(delta), edgeLength = len(edge);
            V2<T> base = edgeLength > 0 ? mk(-edge.y, edge.x) / edgeLength : mk<T>(0, 1);
            T sign = ((w.id[ai] ^ w.sid[s]) & 1) == 0 ? T(1) : T(-1);
            bool fixedSide = (w.sflags[s] & BP_SEGMENT_ALLOWED_SIDE) != 0;
            normal = fixedSide ? base * w.sallowed[s] : (d > 0 ? delta / d : base * sign);
            allowed = fixedSide ? w.sallowed[s] : T(0);
            pen = ar - d;
            if (w.sflags[s] & BP_SEGMENT_POLYGON_EDGE) {
                V2<T> outward = base * w.soutward[s];
                // nativePolygonEdgeFeature, NGK:674-681
                V2<T> start = w.sa[s], end = w.sb[s];
                T along = dot(apos - start, end - start);
                bool convexStart = (w.sflags[s] & BP_SEGMENT_CONVEX_START) != 0;
                if (convexStart && along <= 0 && past_segment_end(apos, w.sprev[s], start)) feature = 2;
                else {
                    bool interior = along > 0 && !past_segment_end(apos, start, end);
                    feature = dot(apos - start, outward) >= 0 && interior ? 1 : 0;
                }
                if (feature == 1) {
                    normal = outward;
                    point = apos - outward * dot(apos - w.sa[s], outward);
                    pen = ar - dot(apos - w.sa[s], outward);
                } else if (feature == 2) {
                    point = w.sa[s];
                    delta = apos - point;
                    d = len(delta);
                    normal = d > 0 ? delta / d : outward;
                    pen = ar - d;
                } else {
                    normal = outward;
                    point = w.sa[s];
                    pen = -Lim<T>::big();
                }
            }
        }
        // nativePrepareContactFlags / nativeCompactActiveContacts: active = penetration > -sepTol
        if (!(pen > -w.sepTol)) return;
        // nativeContactImpulses, NFK:261-280
        T f;
        if (kind == 0) f = pair_law(w.K[ai], ar, w.K[other], w.radius[other], ar + w.radius[other] - pen).force;
        else f = wall_law(w.K[ai], ar, ar - pen).force;
        bp_contact c{};
        c.participants[0] = w.id[ai];
        c.participants[1] = second;
        c.kind = kind;
        c.feature = feature;
        c.normal[0] = (float)normal.x; c.normal[1] = (float)normal.y;
        c.point[0] = (float)point.x; c.point[1] = (float)point.y;
        c.impulse = (float)(f * dt * dt);
        c.penetration = (float)pen;
        c.allowed_side = (float)allowed;
        w.contacts.push_back(c);
    };
    for (uint32_t i = 0; i < w.n; ++i)
        for (uint32_t j : w.rowPairs[i]) record(i, 0, j);
    for (uint32_t i = 0; i < w.n; ++i)
        for (uint32_t sg : w.rowSegs[i]) record(i, 1, sg);
}

template <typename T> bool finite_state(const World<T>& w) {
    for (uint32_t i = 0; i < w.n; ++i) {
        if (is_removed(w, i)) continue;
        if (!finite2(w.pos[i]) || !finite2(w.start[i]) || !finite2(w.vel[i]) || !std::isfinite(w.rot[i]) ||
            !std::isfinite(w.omega[i]))
            return false;
    }
    for (const bp_contact& c : w.contacts)
        if (!std::isfinite(c.normal[0]) || !std::isfinite(c.normal[1]) || !std::isfinite(c.point[0]) ||
            !std::isfinite(c.point[1]) || !std::isfinite(c.impulse) || !std::isfinite(c.penetration))
            return false;
    return true;
}

// ---------------------------------------------------------------------------------------------------------------
// One step (NativeMetalSolver.executeSnapshot + nativeSubstepLoopSingleGroup, NFK:1236-1307)
// ---------------------------------------------------------------------------------------------------------------
template <typename T> void kinematic_advance(World<T>& w) {
    // nativeRigidPredict for static and kinematic bodies (NPK:65-80): previous <- pose; pose += velocity * dt.
    for (Body<T>& b : w.bodies) {
        b.prev = b.pos;
        b.prevAngle = b.angle;
        b.cosPrev = b.cosEnd;
        b.sinPrev = b.sinEnd;
        if (b.flags & BP_BODY_STATIC) {
            b.vel = mk<T>(0, 0);
            b.omega = 0;
            continue;
        }
        b.pos = b.pos + b.vel * w.dt;
        b.angle = b.angle + b.omega * w.dt;
        if (b.angle != b.prevAngle) {
            b.cosEnd = std::cos(b.angle);
            b.sinEnd = std::sin(b.angle);
        }
    }
}

template <typename T> int step(World<T>& w, bp_step_report& rep) {
    std::memset(&rep, 0, sizeof(rep));
    if (w.failed) { rep.status = BP_E_WORLD_FAILED; return BP_E_WORLD_FAILED; }
    const uint32_t n = w.n;
    // nativeBeginStep, NFK:285-293
    for (uint32_t i = 0; i < n; ++i) {
        if (is_removed(w, i)) continue;
        w.result[i] = 0;
        w.start[i] = w.pos[i];
        if ((w.flags_[i] & BP_BUBBLE_ENABLED) && (w.flags_[i] & BP_BUBBLE_STATIC)) {
            w.vel[i] = mk<T>(0, 0);
            w.omega[i] = 0;
        }
    }
    kinematic_advance(w);
    uint32_t live = 0;
    for (uint32_t i = 0; i < n; ++i) live += is_removed(w, i) ? 0 : 1;
    w.timeX = w.dt;
    w.timeY = live == 0 ? w.dt : T(0);
    w.timeZ = 0;
    w.timeW = w.split;
    w.countsX = w.countsY = w.countsZ = w.countsW = 0;
    w.limiterObject = 0;
    w.limiterTerm = 0;
    w.history.clear();
    w.trace.clear();
    w.overflowMax = 0;
    w.maxPerObject = 0;
    w.rebuilds = 0;
    Violation substepViolation;
    broadphase(w);
    contact_forces_all(w);
    integrate(w, 2);
    for (uint32_t iteration = 0; iteration < 2 * kFrameLimit + 2; ++iteration) {
        reduce(w);
        T h = w.timeZ;
        bool limited = w.countsW != 0, finished = !(w.timeX - w.timeY > 0), rebuild = w.countsZ != 0;
        if (!(h > 0)) {
            if (limited || finished || !rebuild) break;
            w.countsX = 0;
            w.countsZ = 0;
            w.overflowMax = std::max(w.overflowMax, w.overflowBuild);
            w.rebuilds += 1;
            broadphase(w);
            contact_forces_all(w);
            integrate(w, 2);
            continue;
        }
        integrate(w, 0);
        contact_forces_all(w);
        integrate(w, 1);
        if (w.flags & BP_WORLD_INJECT_STATE) {
            if (w.countsY == w.injectSubstep + 1)
                for (uint32_t i = 0; i < n; ++i)
                    if (w.id[i] == w.injectObject) w.pos[i] = w.injectPos;
        }
        if ((w.flags & BP_WORLD_ASSERT_EVERY_SUBSTEP) && substepViolation.kind == 0) substepViolation = assert_contacts(w);
        if (w.traceOn) {
            w.trace.push_back(h);
            for (uint32_t i = 0; i < n; ++i) {
                w.trace.push_back(w.pos[i].x); w.trace.push_back(w.pos[i].y);
                w.trace.push_back(w.vel[i].x); w.trace.push_back(w.vel[i].y);
            }
        }
    }
    w.overflowMax = std::max(w.overflowMax, w.overflowBuild);
    // end of step
    uint32_t removed = 0, wrapped = 0;
    bool finite = true;
    if (w.countsW == 0 && (w.flags & BP_WORLD_HAS_REGION)) finite = apply_region(w, removed, wrapped);
    build_contacts(w);
    finite = finite && finite_state(w);
    Violation v = substepViolation;
    if (v.kind == 0 && w.countsW == 0 && !(w.flags & BP_WORLD_NO_END_ASSERTION)) v = assert_contacts(w);

    rep.substep_count = w.countsY;
    rep.rebuild_count = w.rebuilds;
    uint32_t cand = 0;
    for (uint32_t i = 0; i < n; ++i) cand += (uint32_t)(w.rowPairs[i].size() + w.rowSegs[i].size());
    rep.candidate_count = cand;
    uint32_t bodyCand = 0;
    for (auto& row : w.bodyRows) bodyCand += (uint32_t)row.size();
    rep.body_candidate_count = bodyCand;
    rep.candidate_overflow = w.overflowMax;
    rep.max_candidates_per_object = w.maxPerObject;
    rep.contact_count = (uint32_t)w.contacts.size();
    rep.limiter_term = w.limiterTerm;
    rep.limiter_object = w.limiterObject;
    rep.cell_width = (float)w.cellWidth;
    rep.removed_count = removed;
    rep.wrapped_count = wrapped;
    rep.violation_kind = v.kind;
    rep.violation_objects[0] = v.a;
    rep.violation_objects[1] = v.b;
    rep.violation_edge = v.edge;
    rep.violation_distance = (float)v.distance;
    // failure order (NativeMetalSolver.swift:1026-1040): substep limit, non-finite, contact violation
    int status = BP_OK;
    if (w.countsW != 0) status = BP_E_SUBSTEP_LIMIT;
    else if (!finite) status = BP_E_NONFINITE;
    else if (v.kind != 0) status = BP_E_CONTACT_VIOLATION;
    rep.status = status;
    if (status != BP_OK) {
        // publish nothing: restore the last published state, the world is stopped
        w.pos = w.pPos; w.start = w.pStart; w.vel = w.pVel; w.rot = w.pRot; w.omega = w.pOmega;
        w.result = w.pResult; w.flags_ = w.pFlags; w.bodies = w.pBodies;
        w.failed = true;
        return status;
    }
    for (uint32_t i = 0; i < n; ++i)
        if (w.result[i] == 1) w.flags_[i] |= kRemovedFlag;
    w.pPos = w.pos; w.pStart = w.start; w.pVel = w.vel; w.pRot = w.rot; w.pOmega = w.omega;
    w.pResult = w.result; w.pFlags = w.flags_; w.pBodies = w.bodies;
    w.lastReport = rep;
    return BP_OK;
}

// ---------------------------------------------------------------------------------------------------------------
// Construction from the C records
// ---------------------------------------------------------------------------------------------------------------
template <typename T> World<T>* create(const bp_world_desc* d, const bp_world_input* in) {
    World<T>* w = new (std::nothrow) World<T>();
    if (!w) return nullptr;
    w->dt = d->time_step;
    w->sepTol = d->separation_tolerance;
    w->contactTol = d->contact_tolerance;
    w->split = d->substep_split_multiplier;
    w->rmin = mk<T>(d->region[0], d->region[1]);
    w->rmax = mk<T>(d->region[2], d->region[3]);
    w->globalForce = mk<T>(d->global_force[0], d->global_force[1]);
    w->gravity = mk<T>(d->gravity[0], d->gravity[1]);
    w->limit = d->candidate_limit == 0 ? 128u : std::min(d->candidate_limit, 128u);
    w->flags = d->flags;
    w->injectObject = d->inject_object;
    w->injectSubstep = 0;
    w->injectPos = mk<T>(0, 0);
    const uint32_t n = in->bubble_count;
    w->n = n;
    auto resize = [&](auto& v) { v.resize(n); };
    resize(w->id); resize(w->pos); resize(w->start); resize(w->vel); resize(w->acc); resize(w->a0); resize(w->ref);
    resize(w->force); resize(w->rot); resize(w->omega); resize(w->mass); resize(w->invMass); resize(w->radius);
    resize(w->K); resize(w->gamma); resize(w->margin); resize(w->flags_); resize(w->cat); resize(w->mask);
    resize(w->result); resize(w->layer); resize(w->cellX); resize(w->cellY); resize(w->cellValid); resize(w->rowPairs);
    resize(w->rowSegs); resize(w->adj);
    for (uint32_t i = 0; i < n; ++i) {
        const bp_bubble& b = in->bubbles[i];
        w->id[i] = b.id;
        w->pos[i] = mk<T>(b.center[0], b.center[1]);
        w->start[i] = mk<T>(b.previous_center[0], b.previous_center[1]);
        w->vel[i] = mk<T>(b.velocity[0], b.velocity[1]);
        w->acc[i] = mk<T>(0, 0);
        w->rot[i] = b.rotation;
        w->omega[i] = b.angular_velocity;
        w->mass[i] = b.mass;
        w->invMass[i] = b.inverse_mass;
        w->radius[i] = b.radius;
        w->K[i] = b.contact_stiffness;
        w->gamma[i] = b.damping;
        w->flags_[i] = b.flags & 0xffu;
        w->cat[i] = b.category;
        w->mask[i] = b.mask;
        w->result[i] = 0;
        w->layer[i] = b.layer;
    }
    w->s = in->segment_count;
    const uint32_t s = w->s;
    w->sid.resize(s); w->sowner.resize(s); w->sa.resize(s); w->sb.resize(s); w->sprev.resize(s);
    w->soutward.resize(s); w->sallowed.resize(s); w->sflags.resize(s); w->scat.resize(s); w->smask.resize(s);
    w->slayer.resize(s);
    for (uint32_t j = 0; j < s; ++j) {
        const bp_segment& g = in->segments[j];
        w->sid[j] = g.id;
        w->sowner[j] = g.owner_id;
        w->sa[j] = mk<T>(g.a[0], g.a[1]);
        w->sb[j] = mk<T>(g.b[0], g.b[1]);
        w->sprev[j] = mk<T>(g.previous_start[0], g.previous_start[1]);
        w->soutward[j] = g.outward_sign;
        w->sallowed[j] = g.allowed_side;
        w->sflags[j] = g.flags;
        w->scat[j] = g.category;
        w->smask[j] = g.mask;
        w->slayer[j] = g.layer;
    }
    w->bverts.resize(in->body_vertex_count);
    for (uint32_t v = 0; v < in->body_vertex_count; ++v)
        w->bverts[v] = mk<T>(in->body_vertices[2 * v], in->body_vertices[2 * v + 1]);
    w->btris.assign(in->body_triangles, in->body_triangles + 3 * (size_t)in->body_triangle_count);
    for (uint32_t b = 0; b < in->body_count; ++b) {
        const bp_body& r = in->bodies[b];
        Body<T> body;
        body.id = r.id;
        body.pos = mk<T>(r.position[0], r.position[1]);
        body.prev = body.pos;
        body.angle = r.angle;
        body.prevAngle = r.angle;
        body.vel = mk<T>(r.velocity[0], r.velocity[1]);
        body.omega = r.angular_velocity;
        body.radius = r.bounding_radius;
        body.coreRadius = r.core_radius;
        body.kind = r.kind;
        body.flags = r.flags;
        body.voff = r.vertex_offset;
        body.vcount = r.vertex_count;
        body.toff = r.triangle_offset;
        body.tcount = r.triangle_count;
        body.cat = r.category;
        body.mask = r.mask;
        body.layer = r.layer;
        body.cosEnd = std::cos((T)r.angle);
        body.sinEnd = std::sin((T)r.angle);
        body.cosPrev = body.cosEnd;
        body.sinPrev = body.sinEnd;
        w->bodies.push_back(body);
    }
    w->bodyRows.resize(in->body_count);
    w->fverts.resize(in->field_vertex_count);
    for (uint32_t v = 0; v < in->field_vertex_count; ++v)
        w->fverts[v] = mk<T>(in->field_vertices[2 * v], in->field_vertices[2 * v + 1]);
    w->fids.assign(in->field_object_ids, in->field_object_ids + in->field_object_id_count);
    for (uint32_t f = 0; f < in->field_count; ++f) {
        const bp_force_field& r = in->fields[f];
        Field<T> fl;
        fl.pos = mk<T>(r.position[0], r.position[1]);
        fl.cosr = std::cos((T)r.rotation);
        fl.sinr = std::sin((T)r.rotation);
        fl.falloff = r.falloff;
        fl.dir = mk<T>(r.direction[0], r.direction[1]);
        fl.strength = r.strength;
        fl.radius = r.radius;
        fl.kind = r.kind;
        fl.voff = r.vertex_offset;
        fl.vcount = r.vertex_count;
        fl.foff = r.filter_offset;
        fl.fcount = r.filter_count;
        fl.hasFilter = r.has_filter;
        w->fields.push_back(fl);
    }
    w->bands.assign(in->bands, in->bands + in->band_count);
    w->motors.assign(in->motors, in->motors + in->motor_count);
    if (in->joint_ranges && in->joint_entity_count)
        w->jranges.assign(in->joint_ranges, in->joint_ranges + 2 * (size_t)in->joint_entity_count);
    if (in->joint_partners && in->joint_partner_count)
        w->jpartners.assign(in->joint_partners, in->joint_partners + in->joint_partner_count);
    w->pPos = w->pos; w->pStart = w->start; w->pVel = w->vel; w->pRot = w->rot; w->pOmega = w->omega;
    w->pResult = w->result; w->pFlags = w->flags_; w->pBodies = w->bodies;
    w->cellWidth = 0;
    return w;
}

struct Handle {
    int precision;
    void* world;
};

template <typename T> void write_bubbles(const World<T>& w, bp_bubble* out, uint32_t count) {
    for (uint32_t i = 0; i < count && i < w.n; ++i) {
        bp_bubble& b = out[i];
        std::memset(&b, 0, sizeof(b));
        b.id = w.id[i];
        b.center[0] = (float)w.pPos[i].x; b.center[1] = (float)w.pPos[i].y;
        b.previous_center[0] = (float)w.pStart[i].x; b.previous_center[1] = (float)w.pStart[i].y;
        b.velocity[0] = (float)w.pVel[i].x; b.velocity[1] = (float)w.pVel[i].y;
        b.mass = (float)w.mass[i];
        b.inverse_mass = (float)w.invMass[i];
        b.radius = (float)w.radius[i];
        b.rotation = (float)w.pRot[i];
        b.angular_velocity = (float)w.pOmega[i];
        b.contact_stiffness = (float)w.K[i];
        b.damping = (float)w.gamma[i];
        b.flags = w.pFlags[i] & 0xffu;
        b.category = w.cat[i];
        b.mask = w.mask[i];
        b.region_result = w.pResult[i];
    }
}

template <typename T> uint32_t candidate_keys(const World<T>& w, bp_candidate_key* out, uint32_t capacity) {
    std::vector<bp_candidate_key> keys;
    for (uint32_t i = 0; i < w.n; ++i) {
        for (uint32_t j : w.rowPairs[i]) keys.push_back({0, 0, w.id[i], w.id[j]});
        for (uint32_t sg : w.rowSegs[i]) keys.push_back({1, 0, w.id[i], w.sid[sg]});
    }
    for (size_t b = 0; b < w.bodies.size(); ++b)
        for (uint32_t a : w.bodyRows[b]) keys.push_back({2, 0, w.id[a], w.bodies[b].id});
    std::sort(keys.begin(), keys.end(), [](const bp_candidate_key& a, const bp_candidate_key& b) {
        if (a.kind != b.kind) return a.kind < b.kind;
        if (a.first != b.first) return a.first < b.first;
        return a.second < b.second;
    });
    uint32_t count = (uint32_t)keys.size();
    for (uint32_t i = 0; i < count && i < capacity; ++i) out[i] = keys[i];
    return count;
}

}  // namespace

// ---------------------------------------------------------------------------------------------------------------
// C entry points of the oracle (loaded by tests and by bench.py's CPU legs through ctypes)
// ---------------------------------------------------------------------------------------------------------------
// ---------------------------------------------------------------------------------------------------------------
// LBVH keys of the rigid leaves for the step just taken. The reference has no tree (its rigid candidates are brute
// force, NGK:279-290 and NGK:350-415), so this restates the key rule of the CUDA path, in float, to check it bit for
// bit: leaves are the segments then the bodies; a leaf box is the segment's [min(a,b), max(a,b)] or the body's swept
// box [min(pos, prev) - R, max(pos, prev) + R]; centre = (lo + hi) * 0.5; q = trunc(clamp((c - min c) * (32767 /
// extent), 0, 32767)) per axis (scale 0 for a zero extent); code = q.x in the even bits, q.y in the odd bits; key =
// code << 32 | leaf, sorted ascending. No keys when a leaf box is not finite.
// ---------------------------------------------------------------------------------------------------------------
static uint32_t spread_bits15(uint32_t v) {
    v &= 0x7fffu;
    v = (v | (v << 8)) & 0x00ff00ffu;
    v = (v | (v << 4)) & 0x0f0f0f0fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}

template <typename T> std::vector<uint64_t> rigid_keys(const World<T>& w) {
    struct Box { float lx, ly, hx, hy; };
    std::vector<Box> boxes;
    for (uint32_t j = 0; j < w.s; ++j) {
        float ax = (float)w.sa[j].x, ay = (float)w.sa[j].y, bx = (float)w.sb[j].x, by = (float)w.sb[j].y;
        boxes.push_back({std::fmin(ax, bx), std::fmin(ay, by), std::fmax(ax, bx), std::fmax(ay, by)});
    }
    for (const Body<T>& b : w.bodies) {
        float r = (float)b.radius;
        float px = (float)b.pos.x, py = (float)b.pos.y, qx = (float)b.prev.x, qy = (float)b.prev.y;
        boxes.push_back({std::fmin(px, qx) - r, std::fmin(py, qy) - r, std::fmax(px, qx) + r, std::fmax(py, qy) + r});
    }
    std::vector<uint64_t> keys;
    if (boxes.empty()) return keys;
    float lox = 0, loy = 0, hix = 0, hiy = 0;
    for (size_t p = 0; p < boxes.size(); ++p) {
        const Box& b = boxes[p];
        if (!std::isfinite(b.lx) || !std::isfinite(b.ly) || !std::isfinite(b.hx) || !std::isfinite(b.hy)) return {};
        float cx = (b.lx + b.hx) * 0.5f, cy = (b.ly + b.hy) * 0.5f;
        if (p == 0) { lox = hix = cx; loy = hiy = cy; continue; }
        lox = std::fmin(lox, cx); hix = std::fmax(hix, cx);
        loy = std::fmin(loy, cy); hiy = std::fmax(hiy, cy);
    }
    float ex = hix - lox, ey = hiy - loy;
    float sx = ex > 0.0f ? 32767.0f / ex : 0.0f, sy = ey > 0.0f ? 32767.0f / ey : 0.0f;
    for (size_t p = 0; p < boxes.size(); ++p) {
        const Box& b = boxes[p];
        float cx = (b.lx + b.hx) * 0.5f, cy = (b.ly + b.hy) * 0.5f;
        uint32_t qx = (uint32_t)std::fmin(std::fmax((cx - lox) * sx, 0.0f), 32767.0f);
        uint32_t qy = (uint32_t)std::fmin(std::fmax((cy - loy) * sy, 0.0f), 32767.0f);
        uint32_t code = spread_bits15(qx) | (spread_bits15(qy) << 1);
        keys.push_back(((uint64_t)code << 32) | (uint64_t)p);
    }
    std::sort(keys.begin(), keys.end());
    return keys;
}

// ---------------------------------------------------------------------------------------------------------------
// Contours of the published state (NativePostSolveKernels:268-527: nativeContourRayLimit,
// nativeAccumulateContactPressure, nativeGenerateContoursFused, nativePrepareRenderDataGrouped), in float.
// ---------------------------------------------------------------------------------------------------------------
static float contour_ray_limit(float cx, float cy, float dx, float dy, float ax, float ay, float bx, float by,
                               float radius, float clearance) {
    float ex = bx - ax, ey = by - ay, ox = ax - cx, oy = ay - cy;
    float denominator = dx * ey - dy * ex;
    if (std::fabs(denominator) < 1e-6f) return radius;
    float distance = (ox * ey - oy * ex) / denominator;
    float fraction = (ox * dy - oy * dx) / denominator;
    return distance >= 0.0f && fraction >= 0.0f && fraction <= 1.0f ? std::fmin(radius, std::fmax(0.0f, distance - clearance))
                                                                      : radius;
}

static uint32_t contour_samples(float r, float maxEdge, uint32_t stride) {
    const float pi = 3.14159265358979323846f;
    uint32_t want = (uint32_t)std::ceil((r / maxEdge) * (4.0f * pi));
    uint32_t count = std::max(want, 64u);
    return std::min(count, stride);
}

static void world_contours(const World<float>& w, float maxEdge, float tension, float clearance, uint32_t stride,
                           float* points, uint32_t* counts, float* level, float* shape) {
    const float pi = 3.14159265358979323846f;
    for (uint32_t i = 0; i < w.n; ++i) {
        const float r = w.radius[i];
        uint32_t count = (is_removed(w, i) || !(r > 0.0f)) ? 0u : contour_samples(r, maxEdge, stride);
        counts[i] = count;
        if (!count) continue;
        const float cx = w.pPos[i].x, cy = w.pPos[i].y;
        std::vector<float> dirx(count), diry(count), hard(count), lvl(count);
        for (uint32_t s = 0; s < count; ++s) {
            // the CUDA path's host table: cosine and sine of the float angle in double precision, rounded to float
            float angle = 2.0f * pi * (float)s / (float)count;
            dirx[s] = (float)std::cos((double)angle);
            diry[s] = (float)std::sin((double)angle);
            float limit = r;
            for (uint32_t j = 0; j < w.s; ++j) {
                if (!filter_accepts(w.cat[i], w.mask[i], w.scat[j], w.smask[j])) continue;
                limit = contour_ray_limit(cx, cy, dirx[s], diry[s], w.sa[j].x, w.sa[j].y, w.sb[j].x, w.sb[j].y, limit, clearance);
            }
            for (uint32_t key : w.adj[i]) {
                if (key >> 30) continue;
                uint32_t j = key & 0x3fffffffu;
                float ddx = w.pPos[j].x - cx, ddy = w.pPos[j].y - cy;
                float distance = std::sqrt(ddx * ddx + ddy * ddy);
                if (distance <= 1.1920929e-7f || distance >= r + w.radius[j]) continue;
                float nx = ddx / distance, ny = ddy / distance;
                bool lowIsSelf = i < j;
                uint32_t lo = lowIsSelf ? i : j, hi = lowIsSelf ? j : i;
                Law<float> law = pair_law(w.K[lo], w.radius[lo], w.K[hi], w.radius[hi], distance);
                float eps = lowIsSelf ? law.epsA : law.epsB;
                float plane = std::fmin(std::fmax(r * (1.0f - eps), 0.0f), r);
                float half = std::sqrt(std::fmax(0.0f, r * r - plane * plane));
                float tx = -ny, ty = nx;
                float px = cx + nx * plane, py = cy + ny * plane;
                limit = contour_ray_limit(cx, cy, dirx[s], diry[s], px - tx * half, py - ty * half, px + tx * half,
                                          py + ty * half, limit, clearance);
            }
            float deficit = std::fmin(std::fmax(1.0f - limit / r, 0.0f), 1.0f);
            hard[s] = deficit;
            lvl[s] = deficit;
        }
        const float weight = std::fmin(0.8f, tension / (tension + 10.0f));
        std::vector<float> next(count);
        for (int pass = 0; pass < 13; ++pass) {
            for (uint32_t s = 0; s < count; ++s) {
                float neighbour = (lvl[(s + count - 1) % count] + lvl[(s + 1) % count]) * 0.5f;
                next[s] = std::fmin(std::fmax(std::fmax(hard[s], lvl[s] + (neighbour - lvl[s]) * weight), 0.0f), 1.0f);
            }
            lvl.swap(next);
        }
        float maximum = 0.0f;
        uint32_t anchor = 0;
        for (uint32_t s = 0; s < count; ++s)
            if (lvl[s] > maximum) { maximum = lvl[s]; anchor = s; }
        const float slope = maxEdge / (2.0f * r);
        float previous = maximum;
        for (uint32_t step = 1; step < count; ++step) {
            uint32_t s = (anchor + step) % count;
            float v = std::fmax(lvl[s], previous - slope);
            lvl[s] = v;
            previous = v;
        }
        previous = maximum;
        for (uint32_t step = 1; step < count; ++step) {
            uint32_t s = (anchor + count - step) % count;
            float v = std::fmax(lvl[s], previous - slope);
            lvl[s] = v;
            previous = v;
        }
        float effective = r, top = maximum, bx0 = cx, by0 = cy, bx1 = cx, by1 = cy;
        for (uint32_t s = 0; s < count; ++s) {
            float scale = r * (1.0f - lvl[s]);
            float px = cx + dirx[s] * scale, py = cy + diry[s] * scale;
            uint64_t at = (uint64_t)i * stride + s;
            points[2 * at] = px;
            points[2 * at + 1] = py;
            level[at] = lvl[s];
            float ex = px - cx, ey = py - cy;
            effective = std::fmin(effective, std::sqrt(ex * ex + ey * ey));
            top = std::fmax(top, lvl[s]);
            bx0 = std::fmin(bx0, px); by0 = std::fmin(by0, py);
            bx1 = std::fmax(bx1, px); by1 = std::fmax(by1, py);
        }
        float* out = shape + 6ull * i;
        out[0] = top; out[1] = effective; out[2] = bx0; out[3] = by0; out[4] = bx1; out[5] = by1;
    }
}

// Hit test (nativeHitTest, NativeGeometryKernels:501-541) over the contours of world_contours, the bodies at their
// end-of-step pose and the static polygons (even-odd over each owner's consecutive polygon edges): the highest
// (layer as int32, then id as uint64) wins.
static void world_hit_test(const World<float>& w, float maxEdge, float tension, float clearance, const float* queries,
                           uint32_t count, int64_t* ids, uint32_t* layers, uint32_t* found) {
    uint32_t stride = 64;
    for (uint32_t i = 0; i < w.n; ++i) stride = std::max(stride, contour_samples(w.radius[i], maxEdge, 0xffffffffu));
    std::vector<float> points(2ull * w.n * stride), level((size_t)w.n * stride), shape(6ull * w.n);
    std::vector<uint32_t> counts(w.n);
    world_contours(w, maxEdge, tension, clearance, stride, points.data(), counts.data(), level.data(), shape.data());
    for (uint32_t q = 0; q < count; ++q) {
        const float qx = queries[2 * q], qy = queries[2 * q + 1];
        bool any = false;
        uint32_t bestLayer = 0;
        uint64_t bestId = 0;
        auto offer = [&](uint32_t bits, int64_t id) {  // layers order like Int32
            const int32_t layer = (int32_t)bits, best = (int32_t)bestLayer;
            uint64_t u = (uint64_t)id;
            if (!any || layer > best || (layer == best && u > bestId)) { any = true; bestLayer = bits; bestId = u; }
        };
        for (uint32_t i = 0; i < w.n; ++i) {
            if (is_removed(w, i)) continue;
            const float* box = &shape[6ull * i];
            if (qx < box[2] || qy < box[3] || qx > box[4] || qy > box[5]) continue;
            uint32_t c = std::min(counts[i], stride);
            if (c < 3) continue;
            bool inside = false;
            const float* ring = &points[2ull * i * stride];
            for (uint32_t k = 0, j = c - 1; k < c; j = k++) {
                float ax = ring[2 * k], ay = ring[2 * k + 1], bx = ring[2 * j], by = ring[2 * j + 1];
                bool crosses = ((ay > qy) != (by > qy)) && (qx <= (bx - ax) * (qy - ay) / (by - ay) + ax);
                inside = crosses ? !inside : inside;
            }
            if (inside) offer(w.layer[i], w.id[i]);
        }
        for (const Body<float>& b : w.bodies)
            if (rigid_inside(w, mk<float>(qx, qy), b, body_at(b, 1.0f))) offer(b.layer, b.id);
        bool inside = false;
        const uint32_t edge = BP_SEGMENT_POLYGON_EDGE | BP_SEGMENT_HAS_OWNER;
        for (uint32_t j = 0; j < w.s; ++j) {
            if ((w.sflags[j] & edge) != edge) continue;
            float ax = w.sb[j].x, ay = w.sb[j].y, bx = w.sa[j].x, by = w.sa[j].y;
            if (((ay > qy) != (by > qy)) && (qx <= (bx - ax) * (qy - ay) / (by - ay) + ax)) inside = !inside;
            bool last = j + 1 == w.s || w.sowner[j + 1] != w.sowner[j];
            if (last) {
                if (inside) offer(w.slayer[j], w.sowner[j]);
                inside = false;
            }
        }
        ids[q] = (int64_t)bestId;
        layers[q] = bestLayer;
        found[q] = any ? 1u : 0u;
    }
}

// Sensor geometry (NativePostSolveKernels:650-738), each helper restating the reference function named beside it.
struct SensorFrame {
    float px, py, c, s;
    const bp_sensor* sn;
    const float* verts;
    V2<float> vertex(uint32_t j) const {  // world-frame ring vertex
        uint32_t k = sn->vertex_offset + j;
        V2<float> v = mk<float>(verts[2 * k], verts[2 * k + 1]);
        return mk<float>(px, py) + rotate_cs(v, c, s);
    }
};
// nativePointInPolygon
template <typename F> static bool inside_ring(V2<float> p, uint32_t count, F vertex) {
    bool inside = false;
    for (uint32_t i = 0; i < count; ++i) {
        V2<float> a = vertex(i), b = vertex((i + 1) % count);
        if ((a.y > p.y) != (b.y > p.y) && p.x < (b.x - a.x) * (p.y - a.y) / (b.y - a.y) + a.x) inside = !inside;
    }
    return inside;
}
// nativePointSegmentDistanceSquared
static float point_segment_d2(V2<float> p, V2<float> a, V2<float> b) {
    V2<float> ab = b - a;
    float t = std::fmin(std::fmax(dot(p - a, ab) / std::fmax(dot(ab, ab), 1e-20f), 0.0f), 1.0f);
    V2<float> d = p - (a + ab * t);
    return dot(d, d);
}
// nativeSegmentsCross
static bool segments_cross(V2<float> a, V2<float> b, V2<float> c, V2<float> d) {
    if (std::fmax(std::fmin(a.x, b.x), std::fmin(c.x, d.x)) > std::fmin(std::fmax(a.x, b.x), std::fmax(c.x, d.x)) ||
        std::fmax(std::fmin(a.y, b.y), std::fmin(c.y, d.y)) > std::fmin(std::fmax(a.y, b.y), std::fmax(c.y, d.y)))
        return false;
    V2<float> ab = b - a, cd = d - c;
    float p = cross(ab, c - a), q = cross(ab, d - a), r = cross(cd, a - c), s = cross(cd, b - c);
    return ((p <= 0 && q >= 0) || (p >= 0 && q <= 0)) && ((r <= 0 && s >= 0) || (r >= 0 && s <= 0));
}
// nativeSegmentDistance, NativeGeometryKernels:444-462
static float segment_distance(V2<float> a, V2<float> b, V2<float> c, V2<float> d) {
    V2<float> r = b - a, s = d - c;
    float denominator = cross(r, s);
    if (std::fabs(denominator) > 1e-12f) {
        V2<float> qp = c - a;
        float t = cross(qp, s) / denominator, u = cross(qp, r) / denominator;
        if (t >= 0 && t <= 1 && u >= 0 && u <= 1) return 0.0f;
    }
    float best = INFINITY;
    best = std::fmin(best, len(a - closest_point(a, c, d)));
    best = std::fmin(best, len(b - closest_point(b, c, d)));
    best = std::fmin(best, len(c - closest_point(c, a, b)));
    best = std::fmin(best, len(d - closest_point(d, a, b)));
    return best;
}

// A bubble against a sensor, in the sensor's frame (nativeCompactSensorEvents, :610-632).
static bool bubble_overlaps_sensor(const SensorFrame& f, V2<float> center, float radius) {
    const bp_sensor& sn = *f.sn;
    float dx = center.x - f.px, dy = center.y - f.py;
    float lx = f.c * dx + f.s * dy, ly = -f.s * dx + f.c * dy;
    if (sn.vertex_count == 0) {
        float reach = sn.radius + radius;
        return lx * lx + ly * ly <= reach * reach;
    }
    bool inside = false, near = false;
    for (uint32_t j = 0; j < sn.vertex_count; ++j) {
        uint32_t ia = sn.vertex_offset + j, ib = sn.vertex_offset + (j + 1) % sn.vertex_count;
        float ax = f.verts[2 * ia], ay = f.verts[2 * ia + 1], bx = f.verts[2 * ib], by = f.verts[2 * ib + 1];
        if ((ay > ly) != (by > ly) && lx < (bx - ax) * (ly - ay) / (by - ay) + ax) inside = !inside;
        float abx = bx - ax, aby = by - ay;
        float t = std::fmin(std::fmax(((lx - ax) * abx + (ly - ay) * aby) / std::fmax(abx * abx + aby * aby, 1e-20f), 0.0f), 1.0f);
        float ex = lx - (ax + abx * t), ey = ly - (ay + aby * t);
        if (ex * ex + ey * ey <= radius * radius) near = true;
    }
    return near || inside;
}

// A body at its end-of-step pose against a sensor (nativeRoundOverlapsSensor, nativeRigidOverlapsSensor, :677-738).
static bool body_overlaps_sensor(const World<float>& w, const SensorFrame& f, const Body<float>& b) {
    const bp_sensor& sn = *f.sn;
    if (b.vcount == 0) return false;
    Pose<float> pose;
    pose.pos = b.pos;
    pose.c = b.cosEnd;
    pose.s = b.sinEnd;
    auto bodyVertex = [&](uint32_t i) { return body_vertex(w, b, pose, i); };
    auto sensorVertex = [&](uint32_t j) { return f.vertex(j); };
    const V2<float> centre = mk<float>(f.px, f.py);
    if (b.kind != BP_BODY_POLYGON) {
        V2<float> a = bodyVertex(0), e = b.vcount > 1 ? bodyVertex(1) : a;
        if (sn.vertex_count == 0) {
            float reach = b.coreRadius + sn.radius;
            return point_segment_d2(centre, a, e) <= reach * reach;
        }
        if (inside_ring(a, sn.vertex_count, sensorVertex)) return true;
        for (uint32_t j = 0; j < sn.vertex_count; ++j)
            if (segment_distance(a, e, f.vertex(j), f.vertex((j + 1) % sn.vertex_count)) <= b.coreRadius) return true;
        return false;
    }
    if (sn.vertex_count == 0 && inside_ring(centre, b.vcount, bodyVertex)) return true;
    for (uint32_t i = 0; i < b.vcount; ++i) {
        V2<float> a = bodyVertex(i), e = bodyVertex((i + 1) % b.vcount);
        if (sn.vertex_count == 0) {
            if (point_segment_d2(centre, a, e) <= sn.radius * sn.radius) return true;
        } else {
            if (inside_ring(a, sn.vertex_count, sensorVertex)) return true;
            for (uint32_t j = 0; j < sn.vertex_count; ++j)
                if (segments_cross(a, e, f.vertex(j), f.vertex((j + 1) % sn.vertex_count))) return true;
        }
    }
    if (sn.vertex_count) return inside_ring(f.vertex(0), b.vcount, bodyVertex);
    return false;
}

// Sensor events of the published state against the overlap state of the previous evaluation, in pair order: for each
// sensor its bubbles, then its bodies (nativeCompactSensorEvents and nativeCompactPolygonSensorEvents,
// NativePostSolveKernels:601-648 and 740-775). `allowed` (may be null) and `state` hold one byte per pair,
// sensor-major; `state` is updated in place. The rotation is cosf / sinf of the angle, as the CUDA path's host takes
// it. Returns the number of events (written up to `capacity`).
static uint32_t world_sensor_events(const World<float>& w, const bp_sensor* sensors, uint32_t count, const float* verts,
                                    const uint8_t* allowed, uint8_t* state, bp_sensor_event* out, uint32_t capacity) {
    uint32_t events = 0;
    const uint32_t nb = (uint32_t)w.bodies.size(), objects = w.n + nb;
    for (uint32_t si = 0; si < count; ++si) {
        const bp_sensor& sn = sensors[si];
        SensorFrame f{sn.position[0], sn.position[1], std::cos(sn.angle), std::sin(sn.angle), &sn, verts};
        for (uint32_t j = 0; j < objects; ++j) {
            const uint64_t pair = (uint64_t)si * objects + j;
            bool overlapping = false;
            if (!allowed || allowed[pair]) {
                if (j < w.n) overlapping = !is_removed(w, j) && bubble_overlaps_sensor(f, w.pPos[j], w.radius[j]);
                else overlapping = body_overlaps_sensor(w, f, w.bodies[j - w.n]);
            }
            uint8_t& was = state[pair];
            uint32_t kind = overlapping && !was && (sn.flags & BP_SENSOR_ENTER_EVENTS) ? 1u
                          : !overlapping && was && (sn.flags & BP_SENSOR_EXIT_EVENTS) ? 2u : 0u;
            was = overlapping ? 1 : 0;
            if (!kind) continue;
            if (events < capacity) {
                bp_sensor_event& e = out[events];
                e.sensor = sn.id;
                e.kind = kind;
                if (j < w.n) {
                    e.object = w.id[j];
                    e.point[0] = w.pPos[j].x;
                    e.point[1] = w.pPos[j].y;
                    e.object_kind = 0;
                } else {
                    const Body<float>& b = w.bodies[j - w.n];
                    e.object = b.id;
                    e.point[0] = b.pos.x;
                    e.point[1] = b.pos.y;
                    e.object_kind = 1;
                }
            }
            ++events;
        }
    }
    return events;
}

extern "C" {

int bpo_world_create(const bp_world_desc* desc, const bp_world_input* input, int precision, void** out) {
    if (!desc || !input || !out) return BP_E_INVALID;
    Handle* h = new Handle{precision, nullptr};
    h->world = precision == 64 ? (void*)create<double>(desc, input) : (void*)create<float>(desc, input);
    if (!h->world) { delete h; return BP_E_ALLOC; }
    *out = h;
    return BP_OK;
}

void bpo_world_destroy(void* handle) {
    Handle* h = (Handle*)handle;
    if (!h) return;
    if (h->precision == 64) delete (World<double>*)h->world; else delete (World<float>*)h->world;
    delete h;
}

int bpo_world_set_injection(void* handle, uint32_t substep, float x, float y) {
    Handle* h = (Handle*)handle;
    if (h->precision == 64) { auto* w = (World<double>*)h->world; w->injectSubstep = substep; w->injectPos = mk<double>(x, y); }
    else { auto* w = (World<float>*)h->world; w->injectSubstep = substep; w->injectPos = mk<float>(x, y); }
    return BP_OK;
}

int bpo_world_step(void* handle, uint32_t steps, bp_step_report* reports) {
    Handle* h = (Handle*)handle;
    bp_step_report rep;
    int status = BP_OK;
    for (uint32_t s = 0; s < steps; ++s) {
        status = h->precision == 64 ? step(*(World<double>*)h->world, rep) : step(*(World<float>*)h->world, rep);
        if (reports) reports[s] = rep;
        if (status != BP_OK) break;
    }
    return status;
}

// Steps many independent worlds, OpenMP over worlds (the CPU baseline of the batched path).
int bpo_worlds_step(void** handles, uint32_t count, uint32_t steps, int threads, uint64_t* bubble_substeps) {
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
    uint64_t total = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total)
    for (uint32_t wi = 0; wi < count; ++wi) {
        Handle* h = (Handle*)handles[wi];
        bp_step_report rep;
        for (uint32_t s = 0; s < steps; ++s) {
            int status = h->precision == 64 ? step(*(World<double>*)h->world, rep) : step(*(World<float>*)h->world, rep);
            uint32_t n = h->precision == 64 ? ((World<double>*)h->world)->n : ((World<float>*)h->world)->n;
            total += (uint64_t)rep.substep_count * n;
            if (status != BP_OK) break;
        }
    }
    if (bubble_substeps) *bubble_substeps = total;
    return BP_OK;
}

// The same, keeping every world's report of every step: reports[step * count + world] (steps after a failure keep
// the failing report's status and no substeps). Used by the full-size batched parity checks.
int bpo_worlds_step_reports(void** handles, uint32_t count, uint32_t steps, int threads, bp_step_report* reports) {
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
#pragma omp parallel for schedule(dynamic, 1)
    for (uint32_t wi = 0; wi < count; ++wi) {
        Handle* h = (Handle*)handles[wi];
        bp_step_report rep{};
        int status = BP_OK;
        for (uint32_t s = 0; s < steps; ++s) {
            if (status == BP_OK)
                status = h->precision == 64 ? step(*(World<double>*)h->world, rep) : step(*(World<float>*)h->world, rep);
            else
                rep.substep_count = 0;
            reports[(uint64_t)s * count + wi] = rep;
        }
    }
    return BP_OK;
}

// Sorted LBVH keys of the rigid leaves for the last step (see rigid_keys); returns the number of keys.
uint32_t bpo_world_rigid_keys(void* handle, uint64_t* out, uint32_t capacity) {
    Handle* h = (Handle*)handle;
    std::vector<uint64_t> keys = h->precision == 64 ? rigid_keys(*(World<double>*)h->world) : rigid_keys(*(World<float>*)h->world);
    for (uint32_t i = 0; i < keys.size() && i < capacity; ++i) out[i] = keys[i];
    return (uint32_t)keys.size();
}

// Contours of a float world's published state (see world_contours); returns BP_E_INVALID for a double world.
int bpo_world_contours(void* handle, float max_edge, float tension, float clearance, uint32_t stride, float* points,
                       uint32_t* counts, float* level, float* shape) {
    Handle* h = (Handle*)handle;
    if (h->precision == 64) return BP_E_INVALID;
    world_contours(*(World<float>*)h->world, max_edge, tension, clearance, stride, points, counts, level, shape);
    return BP_OK;
}

int bpo_world_hit_test(void* handle, float max_edge, float tension, float clearance, const float* queries,
                       uint32_t count, int64_t* ids, uint32_t* layers, uint32_t* found) {
    Handle* h = (Handle*)handle;
    if (h->precision == 64) return BP_E_INVALID;
    world_hit_test(*(World<float>*)h->world, max_edge, tension, clearance, queries, count, ids, layers, found);
    return BP_OK;
}

uint32_t bpo_world_sensor_events(void* handle, const bp_sensor* sensors, uint32_t count, const float* verts,
                                 const uint8_t* allowed, uint8_t* state, bp_sensor_event* out, uint32_t capacity) {
    Handle* h = (Handle*)handle;
    if (h->precision == 64) return 0;
    return world_sensor_events(*(World<float>*)h->world, sensors, count, verts, allowed, state, out, capacity);
}

int bpo_set_threads(int threads) {
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
    return omp_get_max_threads();
#else
    (void)threads;
    return 1;
#endif
}

int bpo_world_read_bubbles(void* handle, bp_bubble* out, uint32_t capacity, uint32_t* count) {
    Handle* h = (Handle*)handle;
    if (h->precision == 64) { auto* w = (World<double>*)h->world; write_bubbles(*w, out, capacity); if (count) *count = w->n; }
    else { auto* w = (World<float>*)h->world; write_bubbles(*w, out, capacity); if (count) *count = w->n; }
    return BP_OK;
}

// Double-precision state of the FP64 rerun (center.xy, velocity.xy) for error reporting.
int bpo_world_read_state64(void* handle, double* out, uint32_t capacity) {
    Handle* h = (Handle*)handle;
    if (h->precision == 64) {
        auto* w = (World<double>*)h->world;
        for (uint32_t i = 0; i < w->n && i < capacity; ++i) {
            out[4 * i] = w->pPos[i].x; out[4 * i + 1] = w->pPos[i].y; out[4 * i + 2] = w->pVel[i].x; out[4 * i + 3] = w->pVel[i].y;
        }
    } else {
        auto* w = (World<float>*)h->world;
        for (uint32_t i = 0; i < w->n && i < capacity; ++i) {
            out[4 * i] = w->pPos[i].x; out[4 * i + 1] = w->pPos[i].y; out[4 * i + 2] = w->pVel[i].x; out[4 * i + 3] = w->pVel[i].y;
        }
    }
    return BP_OK;
}

int bpo_world_read_contacts(void* handle, bp_contact* out, uint32_t capacity, uint32_t* count) {
    Handle* h = (Handle*)handle;
    const std::vector<bp_contact>& c = h->precision == 64 ? ((World<double>*)h->world)->contacts : ((World<float>*)h->world)->contacts;
    for (uint32_t i = 0; i < c.size() && i < capacity; ++i) out[i] = c[i];
    if (count) *count = (uint32_t)c.size();
    return BP_OK;
}

int bpo_world_read_candidates(void* handle, bp_candidate_key* out, uint32_t capacity, uint32_t* count) {
    Handle* h = (Handle*)handle;
    uint32_t c = h->precision == 64 ? candidate_keys(*(World<double>*)h->world, out, capacity)
                                    : candidate_keys(*(World<float>*)h->world, out, capacity);
    if (count) *count = c;
    return BP_OK;
}

int bpo_world_read_cells(void* handle, int64_t* out, uint32_t capacity, uint32_t* count) {
    Handle* h = (Handle*)handle;
    auto fill = [&](auto* w) {
        for (uint32_t i = 0; i < w->n && i < capacity; ++i) { out[2 * i] = w->cellX[i]; out[2 * i + 1] = w->cellY[i]; }
        if (count) *count = w->n;
    };
    if (h->precision == 64) fill((World<double>*)h->world); else fill((World<float>*)h->world);
    return BP_OK;
}

int bpo_world_read_substeps(void* handle, double* out, uint32_t capacity, uint32_t* count) {
    Handle* h = (Handle*)handle;
    auto fill = [&](auto* w) {
        for (uint32_t i = 0; i < w->history.size() && i < capacity; ++i) out[i] = (double)w->history[i];
        if (count) *count = (uint32_t)w->history.size();
    };
    if (h->precision == 64) fill((World<double>*)h->world); else fill((World<float>*)h->world);
    return BP_OK;
}

// Substep trace of the last step: per substep its h, then x, y, vx, vy of every bubble.
int bpo_world_set_trace(void* handle, int on) {
    Handle* h = (Handle*)handle;
    if (h->precision == 64) ((World<double>*)h->world)->traceOn = on != 0; else ((World<float>*)h->world)->traceOn = on != 0;
    return BP_OK;
}
int bpo_world_read_trace(void* handle, double* out, uint32_t capacity, uint32_t* count) {
    Handle* h = (Handle*)handle;
    auto fill = [&](auto* w) {
        for (uint32_t i = 0; i < w->trace.size() && i < capacity; ++i) out[i] = (double)w->trace[i];
        if (count) *count = (uint32_t)w->trace.size();
    };
    if (h->precision == 64) fill((World<double>*)h->world); else fill((World<float>*)h->world);
    return BP_OK;
}

// Contact began / ended events of one step (NativePublicWorld.contactTransitions, NativePublicWorld.swift:347-391) over
// a step's contact records in id form (bp_contact, as bp_world_read_contacts gives them; kind 1 participants[1] is a
// segment id, reported as its owner when it has one, else skipped; other kinds are id pairs with the normal from the
// first). A record counts when penetration > 0 or impulse > 0 (:373) and either object is interested (:354). Per key
// (ids ordered as unsigned 64-bit values) the sums run in record order in float (:357-359): point * weight with weight
// = max(penetration, 0) + 1e-4, weight, normal from the key's first object (a segment record's normal is negated,
// :375-376), impulse / step. Events: began for keys not in the history, ascending (:384-389), then ended for history
// keys not current, ascending (:390-392); with `removed` ids the host world's rule: a pair that lost one object ends,
// a pair that lost both reports nothing, and the new history drops pairs with a removed object.
int bpo_contact_events(const bp_contact* records, uint32_t count, const int64_t* seg_ids, const int64_t* seg_owners,
                       const uint8_t* seg_has_owner, uint32_t seg_count, const int64_t* interested, uint32_t ni,
                       const uint64_t* history, uint32_t nh, const int64_t* removed, uint32_t nr, float step,
                       bp_contact_event* out, uint32_t capacity, uint32_t* event_count, uint64_t* next_history,
                       uint32_t* next_count) {
    struct Sum { float px = 0, py = 0, w = 0, nx = 0, ny = 0, imp = 0; };
    typedef std::pair<uint64_t, uint64_t> Key;
    std::vector<int64_t> in(interested, interested + ni), rm(removed, removed + nr);
    std::sort(in.begin(), in.end());
    std::sort(rm.begin(), rm.end());
    auto has = [](const std::vector<int64_t>& v, int64_t id) { return std::binary_search(v.begin(), v.end(), id); };
    std::vector<std::pair<Key, Sum>> sums;  // keys in first-seen order; looked up linearly through an index
    std::vector<std::pair<Key, size_t>> index;
    for (uint32_t r = 0; r < count; ++r) {
        const bp_contact& c = records[r];
        const int64_t first = c.participants[0];
        int64_t second = c.participants[1];
        float nfx = c.normal[0], nfy = c.normal[1];
        if (c.kind == 1u) {
            bool found = false;
            for (uint32_t q = 0; q < seg_count; ++q)
                if (seg_ids[q] == second) { found = seg_has_owner[q] != 0; second = seg_owners[q]; break; }
            if (!found) continue;
            nfx = -nfx;
            nfy = -nfy;
        }
        if (!(c.penetration > 0.0f || c.impulse > 0.0f)) continue;
        if (!has(in, first) && !has(in, second)) continue;
        const uint64_t uf = (uint64_t)first, us = (uint64_t)second;
        const bool firstLow = uf <= us;
        const Key key = firstLow ? Key(uf, us) : Key(us, uf);
        size_t at = sums.size();
        for (const auto& e : index)
            if (e.first == key) { at = e.second; break; }
        if (at == sums.size()) { sums.push_back({key, Sum()}); index.push_back({key, at}); }
        Sum& m = sums[at].second;
        const float w = std::fmax(c.penetration, 0.0f) + 1e-4f;
        m.px = m.px + c.point[0] * w;
        m.py = m.py + c.point[1] * w;
        m.w = m.w + w;
        m.nx = m.nx + (firstLow ? nfx : -nfx);
        m.ny = m.ny + (firstLow ? nfy : -nfy);
        m.imp = m.imp + c.impulse / step;
    }
    std::sort(sums.begin(), sums.end(), [](const std::pair<Key, Sum>& a, const std::pair<Key, Sum>& b) { return a.first < b.first; });
    std::vector<Key> hist;
    for (uint32_t q = 0; q < nh; ++q) hist.push_back(Key(history[2 * q], history[2 * q + 1]));
    std::sort(hist.begin(), hist.end());
    uint32_t n = 0;
    auto emit = [&](const bp_contact_event& e) {
        if (n < capacity) out[n] = e;
        ++n;
    };
    std::vector<Key> current;
    for (const auto& kv : sums) {
        current.push_back(kv.first);
        if (std::binary_search(hist.begin(), hist.end(), kv.first)) continue;
        const Sum& m = kv.second;
        bp_contact_event e;
        std::memset(&e, 0, sizeof(e));
        e.kind = 0u;
        e.objects[0] = (int64_t)kv.first.first;
        e.objects[1] = (int64_t)kv.first.second;
        e.point[0] = m.px / m.w;
        e.point[1] = m.py / m.w;
        const float length = std::sqrt(m.nx * m.nx + m.ny * m.ny);
        e.normal[0] = length > 0.0f ? m.nx / length : 0.0f;
        e.normal[1] = length > 0.0f ? m.ny / length : 0.0f;
        e.impulse = m.imp;
        emit(e);
    }
    for (const Key& k : hist) {
        const bool r0 = has(rm, (int64_t)k.first), r1 = has(rm, (int64_t)k.second);
        if (r0 && r1) continue;
        if (!r0 && !r1 && std::binary_search(current.begin(), current.end(), k)) continue;
        bp_contact_event e;
        std::memset(&e, 0, sizeof(e));
        e.kind = 1u;
        e.objects[0] = (int64_t)k.first;
        e.objects[1] = (int64_t)k.second;
        emit(e);
    }
    uint32_t kept = 0;
    for (const Key& k : current) {
        if (has(rm, (int64_t)k.first) || has(rm, (int64_t)k.second)) continue;
        next_history[2 * kept] = k.first;
        next_history[2 * kept + 1] = k.second;
        ++kept;
    }
    *event_count = n;
    *next_count = kept;
    return BP_OK;
}

// Contact law known-answer entry (same layout as bp_device_contact_law): 8 floats in and out per case.
int bpo_contact_law(uint32_t mode, int precision, const double* in, double* out, uint32_t count) {
    for (uint32_t c = 0; c < count; ++c) {
        const double* a = in + 8 * c;
        double* o = out + 8 * c;
        for (int q = 0; q < 8; ++q) o[q] = 0;
        if (precision == 64) {
            if (mode == 0) o[0] = epsilon_from_ratio<double>(a[0]);
            else if (mode == 1) { Law<double> l = wall_law<double>(a[0], a[1], a[2]); o[0] = l.force; o[1] = l.epsA; o[2] = l.stiffness; }
            else { Law<double> l = pair_law<double>(a[0], a[1], a[2], a[3], a[4]); o[0] = l.force; o[1] = l.epsA; o[2] = l.epsB; o[3] = l.stiffness; }
        } else {
            if (mode == 0) o[0] = epsilon_from_ratio<float>((float)a[0]);
            else if (mode == 1) { Law<float> l = wall_law<float>((float)a[0], (float)a[1], (float)a[2]); o[0] = l.force; o[1] = l.epsA; o[2] = l.stiffness; }
            else {
                Law<float> l = pair_law<float>((float)a[0], (float)a[1], (float)a[2], (float)a[3], (float)a[4]);
                o[0] = l.force; o[1] = l.epsA; o[2] = l.epsB; o[3] = l.stiffness;
            }
        }
    }
    return BP_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------------------------
// Rigid body solver: predict (NPK:66-115), joints (NCK:446-562) and finish (NPK:172-198), scalar float, one body or
// joint after the other. sin and cos are the library's own float functions (sincos_cw), exp the float of the
// double-precision exp of the float argument.
// ---------------------------------------------------------------------------------------------------------------
namespace rigid {

const float kMin = std::numeric_limits<float>::min();
const float kEps = std::numeric_limits<float>::epsilon();

struct P2 { float x, y; };
inline P2 p2(float x, float y) { return P2{x, y}; }
inline P2 operator+(P2 a, P2 b) { return p2(a.x + b.x, a.y + b.y); }
inline P2 operator-(P2 a, P2 b) { return p2(a.x - b.x, a.y - b.y); }
inline P2 operator*(P2 a, float s) { return p2(a.x * s, a.y * s); }
inline P2 operator/(P2 a, float s) { return p2(a.x / s, a.y / s); }
inline P2 neg(P2 a) { return p2(-a.x, -a.y); }
inline float dot(P2 a, P2 b) { return a.x * b.x + a.y * b.y; }
inline float cross(P2 a, P2 b) { return a.x * b.y - a.y * b.x; }
inline float length(P2 a) { return std::sqrt(a.x * a.x + a.y * a.y); }
inline float clampf(float v, float lo, float hi) { return std::fmin(std::fmax(v, lo), hi); }

// The library's float sin / cos: Cody-Waite reduction by pi/2 in three float parts (1.5703125, 11 and 24 more
// bits), Taylor series of sin and cos on |r| <= pi/4 to r^11 / r^12, Horner; (cos, sin) of x.
inline P2 sincos_cw(float x) {
    if (!std::isfinite(x)) return p2(std::numeric_limits<float>::quiet_NaN(), std::numeric_limits<float>::quiet_NaN());
    const float k = std::rint(x * 0x1.45f306p-1f);
    const float r = ((x - k * 0x1.92p+0f) - k * 0x1.fb6p-12f) - k * -0x1.777a5cp-25f;
    const float r2 = r * r;
    const float sr = r + r * r2 * (-0x1.555556p-3f + r2 * (0x1.111112p-7f + r2 * (-0x1.a01a02p-13f +
                                   r2 * (0x1.71de3ap-19f + r2 * -0x1.ae6456p-26f))));
    const float cr = 1.0f + r2 * (-0x1.0p-1f + r2 * (0x1.555556p-5f + r2 * (-0x1.6c16c2p-10f +
                                   r2 * (0x1.a01a02p-16f + r2 * (-0x1.27e4fcp-22f + r2 * 0x1.1eed8ep-29f)))));
    const int q = (int)k & 3;
    const float sn = q == 0 ? sr : q == 1 ? cr : q == 2 ? -sr : -cr;
    const float cs = q == 0 ? cr : q == 1 ? -sr : q == 2 ? -cr : sr;
    return p2(cs, sn);
}

// nativeRotate (NGK:136-138)
inline P2 rotate(P2 p, float angle) {
    const P2 cs = sincos_cw(angle);
    return p2(p.x * cs.x - p.y * cs.y, p.x * cs.y + p.y * cs.x);
}
// nativeClosestPoint (NGK:436-440)
inline P2 closest(P2 p, P2 a, P2 b) {
    const P2 edge = b - a;
    const float square = dot(edge, edge);
    return a + edge * (square > kMin ? clampf(dot(p - a, edge) / square, 0.0f, 1.0f) : 0.0f);
}
// nativeClampLinearSpeed / nativeClampAngularSpeed (NGK:151-158)
inline P2 clamp_speed(P2 v, float limit) {
    const float speed = length(v);
    return limit > 0 && speed > limit ? v * (limit / speed) : v;
}
inline float clamp_spin(float w, float limit) { return limit > 0 ? clampf(w, -limit, limit) : w; }
inline bool finite4(const float* v) { return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]) && std::isfinite(v[3]); }

// nativeCenterCrossing (NGK:583-622); the segment moves from (pa, pb) to (ca, cb).
bool center_crossing(P2 start, P2 end, P2 pa, P2 pb, P2 ca, P2 cb) {
    const P2 e0 = pb - pa, de = (cb - ca) - e0, r0 = start - pa, dr = (end - start) - (ca - pa);
    const float a = cross(de, dr), b = cross(e0, dr) + cross(de, r0), c = cross(e0, r0);
    if (a == 0 && b == 0 && c == 0) {
        const float q0 = dot(r0, r0 - e0);
        if (q0 <= 0) return false;
        const float qa = dot(dr, dr - de);
        const float qb = dot(dr, r0 - e0) + dot(r0, dr - de);
        float minimum = std::fmin(q0, qa + qb + q0);
        if (qa > 0) {
            const float t = clampf(-qb / (2 * qa), 0.0f, 1.0f);
            minimum = std::fmin(minimum, (qa * t + qb) * t + q0);
        }
        return minimum <= 0;
    }
    float roots[2] = {-1, -1};
    if (std::fabs(a) <= kEps * std::fmax(std::fabs(b), std::fabs(c))) {
        if (std::fabs(b) > kMin) roots[0] = -c / b;
    } else {
        const float d = b * b - 4 * a * c;
        if (d > 0) {
            const float q = -0.5f * (b + std::copysign(std::sqrt(d), b));
            roots[0] = q / a;
            roots[1] = std::fabs(q) > kMin ? c / q : -1;
        }
    }
    for (int k = 0; k < 2; ++k) {
        const float t = roots[k];
        if (!(t > 0 && t < 1)) continue;
        const P2 edge = e0 + de * t, relative = r0 + dr * t;
        const float square = dot(edge, edge), along = dot(relative, edge);
        if (square > kMin && along >= 0 && along <= square) return true;
    }
    return false;
}

// nativeJointExcluded (NGK:254-258)
bool excluded(const uint32_t* ranges, const uint64_t* partners, uint32_t partnerCount, uint32_t entity, uint64_t partner) {
    if (!ranges) return false;
    const uint32_t* r = ranges + 4 * (size_t)entity;
    for (uint32_t i = 0; i < r[3]; ++i) {
        if (r[2] + i >= partnerCount) break;
        if (partners[r[2] + i] == partner) return true;
    }
    return false;
}

struct Pose { float x, y, a; };
inline Pose lerp(Pose s, Pose e, float t) { return Pose{s.x + (e.x - s.x) * t, s.y + (e.y - s.y) * t, s.a + (e.a - s.a) * t}; }

struct Sweep {
    const float* verts;
    const bp_segment* segs;
    uint32_t segmentCount, entity, partnerCount;
    const uint32_t* ranges;
    const uint64_t* partners;
};

P2 hit_normal(P2 a, P2 b, P2 startVertex) {
    const P2 edge = b - a;
    const P2 raw = p2(edge.y, -edge.x);
    P2 n = raw / length(raw);
    if (dot(startVertex - a, n) < 0) n = neg(n);
    return n;
}

// nativeRigidSweepCrossing (NPK:30-63)
bool sweep_crossing(const bp_rigid_body& b, Pose p, Pose q, const Sweep& in, P2& point, P2& normal, int64_t& owner) {
    for (uint32_t j = 0; j < in.segmentCount; ++j) {
        const bp_segment& wall = in.segs[j];
        const bool hasOwner = (wall.flags & BP_SEGMENT_HAS_OWNER) != 0;
        if ((uint64_t)wall.owner_id == b.id && hasOwner) continue;
        if (hasOwner && excluded(in.ranges, in.partners, in.partnerCount, in.entity, (uint64_t)wall.owner_id)) continue;
        if (!((b.filter[0] & wall.mask) != 0 && (wall.category & b.filter[1]) != 0)) continue;
        const P2 A = p2(wall.a[0], wall.a[1]), B = p2(wall.b[0], wall.b[1]);
        const uint32_t n = b.ranges[1];
        for (uint32_t k = 0; k < n; ++k) {
            const P2 v = p2(in.verts[2 * (b.ranges[0] + k)], in.verts[2 * (b.ranges[0] + k) + 1]);
            const P2 sv = p2(p.x, p.y) + rotate(v, p.a), ev = p2(q.x, q.y) + rotate(v, q.a);
            bool hit = center_crossing(sv, ev, A, B, A, B);
            if (!hit) {
                const uint32_t nk = b.ranges[0] + (k + 1) % n;
                const P2 w = p2(in.verts[2 * nk], in.verts[2 * nk + 1]);
                const P2 ps = p2(p.x, p.y) + rotate(v, p.a), pe = p2(p.x, p.y) + rotate(w, p.a);
                const P2 qs = p2(q.x, q.y) + rotate(v, q.a), qe = p2(q.x, q.y) + rotate(w, q.a);
                hit = center_crossing(A, A, ps, pe, qs, qe) || center_crossing(B, B, ps, pe, qs, qe);
            }
            if (hit) {
                point = closest(ev, A, B);
                normal = hit_normal(A, B, sv);
                owner = wall.owner_id;
                return true;
            }
        }
    }
    return false;
}

bool vertices_ok(const bp_rigid_body& b, uint32_t vertexCount) {
    return b.ranges[1] <= vertexCount && b.ranges[0] <= vertexCount - b.ranges[1];
}

// nativeRigidPredict (NPK:66-115)
void predict(bp_rigid_body* bodies, uint32_t count, const Sweep& base, uint32_t vertexCount, uint32_t bubbleCount,
             float dt, bp_rigid_wall* walls, uint32_t* safety) {
    for (uint32_t index = 0; index < count; ++index) {
        bp_rigid_body b = bodies[index];
        b.previous[0] = b.pose[0]; b.previous[1] = b.pose[1]; b.pose[3] = b.pose[2]; b.flags[2] = 0;
        if (b.flags[0]) {
            b.motion[0] = b.motion[1] = b.motion[2] = 0;
            bodies[index] = b;
            continue;
        }
        b.motion[2] = b.motion[2] * (float)std::exp((double)(-b.motion[3] * dt));
        const P2 v = clamp_speed(p2(b.motion[0], b.motion[1]), b.limits[0]);
        b.motion[0] = v.x; b.motion[1] = v.y;
        b.motion[2] = clamp_spin(b.motion[2], b.limits[1]);
        const Pose start{b.pose[0], b.pose[1], b.pose[2]};
        b.pose[0] = b.pose[0] + b.motion[0] * dt;
        b.pose[1] = b.pose[1] + b.motion[1] * dt;
        b.pose[2] = b.pose[2] + b.motion[2] * dt;
        if (!finite4(b.pose) || !finite4(b.motion)) { *safety |= BP_RIGID_SAFETY_NONFINITE; bodies[index] = b; continue; }
        if (b.filter[2]) { bodies[index] = b; continue; }
        if (!vertices_ok(b, vertexCount)) { *safety |= BP_RIGID_SAFETY_INVALID; bodies[index] = b; continue; }
        const float samples = std::ceil(std::fabs(b.pose[2] - start.a) / 0.05f);
        const uint32_t steps = samples > 128.0f ? 129u : std::max(1u, (uint32_t)samples);
        if (steps > 128) { *safety |= BP_RIGID_SAFETY_ROTATION_BUDGET; bodies[index] = b; continue; }
        Sweep in = base;
        in.entity = bubbleCount + index;
        const Pose end{b.pose[0], b.pose[1], b.pose[2]};
        bool crossed = false;
        P2 point = p2(0, 0), normal = p2(0, 0);
        int64_t owner = 0;
        Pose stop = start;
        for (uint32_t sample = 0; sample < steps && !crossed; ++sample) {
            const Pose p = lerp(start, end, (float)sample / (float)steps);
            const Pose q = lerp(start, end, (float)(sample + 1) / (float)steps);
            crossed = sweep_crossing(b, p, q, in, point, normal, owner);
            if (!crossed) continue;
            Pose last = p, hit = q;
            for (int bisection = 0; bisection < 12; ++bisection) {
                const Pose middle{0.5f * (last.x + hit.x), 0.5f * (last.y + hit.y), 0.5f * (last.a + hit.a)};
                P2 tp, tn;
                int64_t to;
                if (sweep_crossing(b, p, middle, in, tp, tn, to)) hit = middle; else last = middle;
            }
            stop = last;
        }
        if (crossed) {
            const float closing = std::fmax(0.0f, -dot(p2(b.motion[0], b.motion[1]), normal));
            const float stopped = b.physical[0] > 0 ? closing / b.physical[0] * dt : 0.0f;
            b.pose[0] = stop.x; b.pose[1] = stop.y; b.pose[2] = stop.a;
            b.motion[0] = b.motion[1] = b.motion[2] = 0;
            for (uint32_t j = 0; j < count; ++j) {
                if (j != index && bodies[j].flags[0] && bodies[j].id == (uint64_t)owner) {
                    bp_rigid_wall w{};
                    w.participants[0] = (int64_t)b.id; w.participants[1] = owner;
                    w.geometry[0] = normal.x; w.geometry[1] = normal.y; w.geometry[2] = point.x; w.geometry[3] = point.y;
                    w.extra[0] = stopped;
                    walls[index] = w;
                    break;
                }
            }
        }
        bodies[index] = b;
    }
}

// nativeRigidFinish (NPK:172-198)
void finish(bp_rigid_body* bodies, uint32_t count, const float* verts, uint32_t vertexCount, const float* region,
            uint32_t* safety) {
    for (uint32_t index = 0; index < count; ++index) {
        bp_rigid_body b = bodies[index];
        if (!finite4(b.pose) || !finite4(b.previous) || !finite4(b.motion)) { *safety |= BP_RIGID_SAFETY_NONFINITE; continue; }
        if (b.flags[0]) continue;
        const P2 v = clamp_speed(p2(b.motion[0], b.motion[1]), b.limits[0]);
        b.motion[0] = v.x; b.motion[1] = v.y;
        b.motion[2] = clamp_spin(b.motion[2], b.limits[1]);
        if (!vertices_ok(b, vertexCount)) { *safety |= BP_RIGID_SAFETY_INVALID; continue; }
        const float inf = std::numeric_limits<float>::infinity();
        float lowX = inf, lowY = inf, highX = -inf, highY = -inf;
        for (uint32_t i = 0; i < b.ranges[1]; ++i) {
            const uint32_t at = b.ranges[0] + i;
            const P2 w = p2(b.pose[0], b.pose[1]) + rotate(p2(verts[2 * at], verts[2 * at + 1]), b.pose[2]);
            lowX = std::fmin(lowX, w.x); lowY = std::fmin(lowY, w.y);
            highX = std::fmax(highX, w.x); highY = std::fmax(highY, w.y);
        }
        lowX = lowX - b.shape[1]; lowY = lowY - b.shape[1];
        highX = highX + b.shape[1]; highY = highY + b.shape[1];
        const float sizeX = region[2] - region[0], sizeY = region[3] - region[1];
        float shiftX = 0, shiftY = 0;
        if (highX < region[0] || highY < region[1] || lowX > region[2] || lowY > region[3]) {
            if (!b.flags[1]) {
                b.flags[2] = 1;
            } else {
                if (highX < region[0]) shiftX = std::ceil((region[0] - highX) / sizeX) * sizeX;
                if (lowX > region[2]) shiftX = -std::ceil((lowX - region[2]) / sizeX) * sizeX;
                if (highY < region[1]) shiftY = std::ceil((region[1] - highY) / sizeY) * sizeY;
                if (lowY > region[3]) shiftY = -std::ceil((lowY - region[3]) / sizeY) * sizeY;
                b.pose[0] = b.pose[0] + shiftX; b.pose[1] = b.pose[1] + shiftY;
                b.previous[0] = b.previous[0] + shiftX; b.previous[1] = b.previous[1] + shiftY;
                b.flags[2] = 2;
            }
        }
        bodies[index] = b;
    }
}

// nativeJointEnd (NCK:451-464)
struct End { P2 point, arm, velocity; float im, ii, angle, omega; };

bool end_of(uint32_t entity, P2 anchor, const bp_rigid_body* bodies, uint32_t count, uint32_t bubbleCount, End& e) {
    e = End{anchor, p2(0, 0), p2(0, 0), 0, 0, 0, 0};
    if (entity == BP_JOINT_WORLD_END) return true;
    if (entity < bubbleCount || entity - bubbleCount >= count) return false;
    const bp_rigid_body& b = bodies[entity - bubbleCount];
    e.arm = rotate(anchor - p2(b.previous[2], b.previous[3]), b.pose[2]);
    e.point = p2(b.pose[0], b.pose[1]) + e.arm;
    e.velocity = p2(b.motion[0], b.motion[1]);
    e.omega = b.motion[2];
    e.angle = b.pose[2];
    e.im = b.physical[0];
    e.ii = b.physical[1];
    return true;
}

// nativeSolveJoints (NCK:468-543)
void solve(bp_rigid_joint& joint, bp_rigid_correction& out, const bp_rigid_body* bodies, uint32_t count,
           uint32_t bubbleCount, float dt, uint32_t iterationCount, uint32_t* safety) {
    std::memset(&out, 0, sizeof(out));
    End a, b;
    const bool okA = end_of(joint.ends[0], p2(joint.anchors[0], joint.anchors[1]), bodies, count, bubbleCount, a);
    const bool okB = end_of(joint.ends[1], p2(joint.anchors[2], joint.anchors[3]), bodies, count, bubbleCount, b);
    if (!okA || !okB) { *safety |= BP_RIGID_SAFETY_INVALID; return; }
    P2 moveA = p2(0, 0), moveB = p2(0, 0), speedA = p2(0, 0), speedB = p2(0, 0);
    float turnA = 0, turnB = 0, spinA = 0, spinB = 0;
    const P2 perpA = p2(-a.arm.y, a.arm.x), perpB = p2(-b.arm.y, b.arm.x);
    const uint32_t kind = joint.ends[2];
    if (kind == 0) {
        const P2 delta = b.point - a.point;
        const float len = length(delta);
        const P2 n = len > 1e-6f ? delta / len : p2(1, 0);
        const float ca = cross(a.arm, n), cb = cross(b.arm, n);
        const float w = a.im + b.im + a.ii * ca * ca + b.ii * cb * cb;
        if (w > kMin) {
            const float alpha = joint.parameters[1] / (dt * dt);
            const float lambda = (-(len - joint.parameters[0]) - alpha * joint.state[0]) / (w + alpha);
            joint.state[0] = joint.state[0] + lambda;
            moveA = neg(n) * a.im * lambda;
            turnA = -ca * a.ii * lambda;
            moveB = n * b.im * lambda;
            turnB = cb * b.ii * lambda;
            if (joint.parameters[2] > 0) {
                const float relative = dot((b.velocity + perpB * b.omega) - (a.velocity + perpA * a.omega), n);
                const float decay = (float)std::exp((double)(-joint.parameters[2] * dt / (float)std::max(iterationCount, 1u)));
                const float impulse = -relative * (1.0f - decay) / w;
                speedA = speedA - n * a.im * impulse;
                spinA = spinA - ca * a.ii * impulse;
                speedB = speedB + n * b.im * impulse;
                spinB = spinB + cb * b.ii * impulse;
            }
        }
    } else {
        const float weight = a.im + b.im;
        const float k11 = weight + a.ii * perpA.x * perpA.x + b.ii * perpB.x * perpB.x;
        const float k12 = a.ii * perpA.x * perpA.y + b.ii * perpB.x * perpB.y;
        const float k22 = weight + a.ii * perpA.y * perpA.y + b.ii * perpB.y * perpB.y;
        const float det = k11 * k22 - k12 * k12;
        if (det > kMin) {
            const P2 gap = b.point - a.point;
            const P2 impulse = p2(-(k22 * gap.x - k12 * gap.y), -(-k12 * gap.x + k11 * gap.y)) / det;
            moveA = neg(impulse) * a.im;
            turnA = -a.ii * dot(perpA, impulse);
            moveB = impulse * b.im;
            turnB = b.ii * dot(perpB, impulse);
        }
        const float inertia = a.ii + b.ii;
        if (inertia > kMin) {
            const float angle = (b.angle + turnB) - (a.angle + turnA) - joint.parameters[3];
            float violation = 0;
            if (kind == 2) violation = angle;
            else if (joint.ends[3] & 1u)
                violation = angle < joint.limits[0] ? angle - joint.limits[0] : (angle > joint.limits[1] ? angle - joint.limits[1] : 0.0f);
            if (violation != 0) {
                const float lambda = -violation / inertia;
                turnA = turnA - a.ii * lambda;
                turnB = turnB + b.ii * lambda;
            }
            if (kind == 1 && (joint.ends[3] & 2u)) {
                const float relative = (b.omega + turnB / dt) - (a.omega + turnA / dt) - joint.limits[2];
                const float limit = joint.limits[3] * dt;
                const float total = clampf(joint.state[1] - relative / inertia, -limit, limit);
                const float lambda = total - joint.state[1];
                joint.state[1] = total;
                spinA = spinA - a.ii * lambda;
                spinB = spinB + b.ii * lambda;
            }
        }
    }
    out.first[0] = moveA.x; out.first[1] = moveA.y; out.first[2] = turnA;
    out.second[0] = moveB.x; out.second[1] = moveB.y; out.second[2] = turnB;
    out.velocity_first[0] = moveA.x / dt + speedA.x; out.velocity_first[1] = moveA.y / dt + speedA.y;
    out.velocity_first[2] = turnA / dt + spinA;
    out.velocity_second[0] = moveB.x / dt + speedB.x; out.velocity_second[1] = moveB.y / dt + speedB.y;
    out.velocity_second[2] = turnB / dt + spinB;
}

// ---- body contacts, candidates, CCD, wall guard -------------------------------------------------------------

inline bool is_round(const bp_rigid_body& b) { return b.shape[0] > 0.5f; }
inline bool immovable(const bp_rigid_body& b) { return b.flags[0] != 0 || b.filter[2] != 0; }
inline bool accepts(const uint32_t* a, const uint32_t* b) { return (a[0] & b[1]) != 0 && (b[0] & a[1]) != 0; }
inline float distance(P2 a, P2 b) { return length(a - b); }

struct Geo {
    const float* verts;
    uint32_t vertexCount;
    const uint32_t* tris;  // uint4 per triangle (indices into the body's vertex range, pad)
    uint32_t triangleCount;
};

inline P2 local_vertex(const Geo& g, const bp_rigid_body& b, uint32_t i) {
    const uint32_t at = b.ranges[0] + i;
    return p2(g.verts[2 * at], g.verts[2 * at + 1]);
}
// nativeRigidVertex (NGK:139-141)
inline P2 world_vertex(const Geo& g, const bp_rigid_body& b, uint32_t i) {
    return p2(b.pose[0], b.pose[1]) + rotate(local_vertex(g, b, i), b.pose[2]);
}

// A body's vertex and triangle ranges lie inside the arrays and its triangles index its own vertices.
bool geometry_ok(const Geo& g, const bp_rigid_body& b) {
    if (!vertices_ok(b, g.vertexCount)) return false;
    if (b.ranges[3] > g.triangleCount || b.ranges[2] > g.triangleCount - b.ranges[3]) return false;
    for (uint32_t i = 0; i < b.ranges[3]; ++i) {
        const uint32_t* t = g.tris + 4 * (size_t)(b.ranges[2] + i);
        if (t[0] >= b.ranges[1] || t[1] >= b.ranges[1] || t[2] >= b.ranges[1]) return false;
    }
    return is_round(b) ? b.ranges[1] >= 1 : true;
}

// nativeSegmentDistance (NGK:444-462)
float segment_distance(P2 a, P2 b, P2 c, P2 d, P2& pa, P2& pb) {
    const P2 r = b - a, s = d - c;
    const float denominator = cross(r, s);
    if (std::fabs(denominator) > 1e-12f) {
        const P2 qp = c - a;
        const float t = cross(qp, s) / denominator, u = cross(qp, r) / denominator;
        if (t >= 0 && t <= 1 && u >= 0 && u <= 1) { pa = a + r * t; pb = pa; return 0; }
    }
    float best = std::numeric_limits<float>::infinity();
    P2 cp = closest(a, c, d);
    float value = distance(a, cp);
    if (value < best) { best = value; pa = a; pb = cp; }
    cp = closest(b, c, d); value = distance(b, cp);
    if (value < best) { best = value; pa = b; pb = cp; }
    cp = closest(c, a, b); value = distance(c, cp);
    if (value < best) { best = value; pa = cp; pb = c; }
    cp = closest(d, a, b); value = distance(d, cp);
    if (value < best) { best = value; pa = cp; pb = d; }
    return best;
}

struct Core { P2 a, b; float radius; };
// nativeRoundCoreOf (NGK:466-472)
Core core_of(const Geo& g, const bp_rigid_body& b) {
    Core c;
    c.a = world_vertex(g, b, 0);
    c.b = b.ranges[1] > 1 ? world_vertex(g, b, 1) : c.a;
    c.radius = b.shape[1];
    return c;
}

// nativeRigidInside (NGK:477-490)
bool rigid_inside(const Geo& g, P2 p, const bp_rigid_body& b) {
    if (is_round(b)) {
        const Core c = core_of(g, b);
        return distance(p, closest(p, c.a, c.b)) <= c.radius;
    }
    const P2 local = rotate(p - p2(b.pose[0], b.pose[1]), -b.pose[2]);
    for (uint32_t i = 0; i < b.ranges[3]; ++i) {
        const uint32_t* t = g.tris + 4 * (size_t)(b.ranges[2] + i);
        const P2 A = local_vertex(g, b, t[0]), B = local_vertex(g, b, t[1]), C = local_vertex(g, b, t[2]);
        if (cross(B - A, local - A) >= 0 && cross(C - B, local - B) >= 0 && cross(A - C, local - C) >= 0) return true;
    }
    return false;
}

// nativeRoundContact (NGK:546-581)
bool round_contact(const Core& A, const Core& B, P2 fallback, P2& normal, float& depth, P2& point) {
    P2 pa, pb;
    const float separation = segment_distance(A.a, A.b, B.a, B.b, pa, pb);
    if (separation > 1e-4f) {
        normal = (pb - pa) / separation;
        depth = A.radius + B.radius - separation;
        point = ((pa + normal * A.radius) + (pb - normal * B.radius)) * 0.5f;
        return true;
    }
    P2 axes[2];
    uint32_t axisCount = 0;
    const P2 ea = A.b - A.a, eb = B.b - B.a;
    const float la = length(ea), lb = length(eb);
    if (la > 1e-6f) axes[axisCount++] = p2(-ea.y, ea.x) / la;
    if (lb > 1e-6f) axes[axisCount++] = p2(-eb.y, eb.x) / lb;
    P2 axis = fallback;
    float overlap = 0, orientation = 1, best = std::numeric_limits<float>::infinity();
    for (uint32_t i = 0; i < axisCount; ++i) {
        const P2 c = axes[i];
        const float amin = std::fmin(dot(A.a, c), dot(A.b, c)), amax = std::fmax(dot(A.a, c), dot(A.b, c));
        const float bmin = std::fmin(dot(B.a, c), dot(B.b, c)), bmax = std::fmax(dot(B.a, c), dot(B.b, c));
        const float plus = amax - bmin, minus = bmax - amin;
        const float value = std::fmin(plus, minus);
        if (value < best) {
            best = value; axis = c; overlap = value;
            if (std::fabs(plus - minus) < 1e-6f) orientation = dot(c, fallback) >= 0 ? 1.0f : -1.0f;
            else orientation = plus < minus ? 1.0f : -1.0f;
        }
    }
    normal = axis * orientation;
    depth = overlap + A.radius + B.radius;
    point = (pa + pb) * 0.5f;
    return true;
}

// nativeTriangleContact (NCK:248-275)
bool triangle_contact(const P2* a, const P2* b, P2& normal, float& depth, P2& point) {
    depth = std::numeric_limits<float>::infinity();
    for (int shape = 0; shape < 2; ++shape)
        for (int edge = 0; edge < 3; ++edge) {
            const P2 delta = shape == 0 ? a[(edge + 1) % 3] - a[edge] : b[(edge + 1) % 3] - b[edge];
            const float magnitude = length(delta);
            if (magnitude <= kMin) return false;
            const P2 axis = p2(-delta.y, delta.x) / magnitude;
            float amin = std::numeric_limits<float>::infinity(), amax = -amin, bmin = amin, bmax = -amin;
            for (int k = 0; k < 3; ++k) {
                const float pa = dot(a[k], axis), pb = dot(b[k], axis);
                amin = std::fmin(amin, pa); amax = std::fmax(amax, pa);
                bmin = std::fmin(bmin, pb); bmax = std::fmax(bmax, pb);
            }
            if (amax < bmin || bmax < amin) return false;
            const float plus = amax - bmin, minus = bmax - amin;
            const float overlap = std::fmin(plus, minus);
            if (overlap < depth) { depth = overlap; normal = plus < minus ? axis : neg(axis); }
        }
    float maxA = -std::numeric_limits<float>::infinity(), minB = std::numeric_limits<float>::infinity();
    P2 pa = p2(0, 0), pb = p2(0, 0);
    uint32_t na = 0, nb = 0;
    for (int k = 0; k < 3; ++k) { maxA = std::fmax(maxA, dot(a[k], normal)); minB = std::fmin(minB, dot(b[k], normal)); }
    for (int k = 0; k < 3; ++k) {
        if (dot(a[k], normal) >= maxA - 1e-5f) { pa = pa + a[k]; ++na; }
        if (dot(b[k], normal) <= minB + 1e-5f) { pb = pb + b[k]; ++nb; }
    }
    point = (pa / (float)na + pb / (float)nb) * 0.5f;
    return true;
}

inline P2 outward_of(P2 p, P2 q) {
    const P2 edge = q - p;
    const float size = length(edge);
    return size > kMin ? p2(edge.y, -edge.x) / size : p2(0, 1);
}

// nativeRoundPolygonContact (NCK:277-333): normal from the round core R to the polygon P.
bool round_polygon_contact(const Geo& g, const Core& R, const bp_rigid_body& P, P2& normal, float& depth, P2& point) {
    const uint32_t count = P.ranges[1];
    float insideDepth = -1;
    P2 insideOutward = p2(0, 0), insidePoint = p2(0, 0);
    const uint32_t endpoints = (R.b.x != R.a.x || R.b.y != R.a.y) ? 2u : 1u;
    uint32_t insideEndpoints = 0;
    for (uint32_t k = 0; k < endpoints; ++k) {
        const P2 endpoint = k == 0 ? R.a : R.b;
        if (!rigid_inside(g, endpoint, P)) continue;
        ++insideEndpoints;
        float nearest = std::numeric_limits<float>::infinity();
        P2 nearestPoint = p2(0, 0), nearestOutward = p2(0, 0);
        for (uint32_t e = 0; e < count; ++e) {
            const P2 p = world_vertex(g, P, e), q = world_vertex(g, P, (e + 1) % count);
            const P2 c = closest(endpoint, p, q);
            const float d = distance(endpoint, c);
            if (d < nearest) { nearest = d; nearestPoint = c; nearestOutward = outward_of(p, q); }
        }
        if (nearest > insideDepth) { insideDepth = nearest; insidePoint = nearestPoint; insideOutward = nearestOutward; }
    }
    if (insideEndpoints == endpoints) {
        normal = neg(insideOutward); depth = R.radius + insideDepth; point = insidePoint;
        return true;
    }
    float best = std::numeric_limits<float>::infinity();
    P2 pc = p2(0, 0), pe = p2(0, 0);
    for (uint32_t e = 0; e < count; ++e) {
        const P2 p = world_vertex(g, P, e), q = world_vertex(g, P, (e + 1) % count);
        P2 ca, ce;
        const float d = segment_distance(R.a, R.b, p, q, ca, ce);
        if (d < best) { best = d; pc = ca; pe = ce; }
    }
    if (best > 1e-4f) {
        normal = (pe - pc) / best; depth = R.radius - best; point = pe;
        return true;
    }
    float minimum = std::numeric_limits<float>::infinity();
    P2 minimumOutward = p2(0, 1), minimumPoint = pe;
    for (uint32_t e = 0; e < count; ++e) {
        const P2 p = world_vertex(g, P, e), q = world_vertex(g, P, (e + 1) % count);
        const P2 edge = q - p;
        const float size = length(edge);
        if (size <= kMin) continue;
        const P2 outward = p2(edge.y, -edge.x) / size;
        const float da = dot(R.a - p, outward), db = dot(R.b - p, outward);
        const float d = R.radius - std::fmin(da, db);
        if (d < minimum) {
            minimum = d; minimumOutward = outward;
            minimumPoint = (da <= db ? R.a : R.b) - outward * std::fmin(da, db);
        }
    }
    normal = neg(minimumOutward); depth = std::isfinite(minimum) ? minimum : R.radius; point = minimumPoint;
    return true;
}

// nativeRoundCoreCrossesPolygon (NCK:335-344)
bool round_core_crosses_polygon(const Geo& g, const Core& R, const bp_rigid_body& P) {
    if (rigid_inside(g, R.a, P) || rigid_inside(g, R.b, P)) return true;
    for (uint32_t e = 0; e < P.ranges[1]; ++e) {
        const P2 p = world_vertex(g, P, e), q = world_vertex(g, P, (e + 1) % P.ranges[1]);
        P2 ca, ce;
        if (segment_distance(R.a, R.b, p, q, ca, ce) <= 1e-4f) return true;
    }
    return false;
}

// nativeRigidPairContact (NCK:348-373): normal from a to b; false = the shapes do not overlap.
bool pair_contact(const Geo& g, const bp_rigid_body& a, const bp_rigid_body& b, P2& n, float& depth, P2& point) {
    const bool aRound = is_round(a), bRound = is_round(b);
    if (aRound && bRound) return round_contact(core_of(g, a), core_of(g, b), p2(1, 0), n, depth, point);
    if (aRound != bRound) {
        const bp_rigid_body& round = aRound ? a : b;
        const bp_rigid_body& polygon = aRound ? b : a;
        P2 normal;
        if (!round_polygon_contact(g, core_of(g, round), polygon, normal, depth, point)) return false;
        n = aRound ? normal : neg(normal);
        return true;
    }
    bool found = false;
    for (uint32_t i = 0; i < a.ranges[3]; ++i)
        for (uint32_t j = 0; j < b.ranges[3]; ++j) {
            const uint32_t* ta = g.tris + 4 * (size_t)(a.ranges[2] + i);
            const uint32_t* tb = g.tris + 4 * (size_t)(b.ranges[2] + j);
            const P2 av[3] = {world_vertex(g, a, ta[0]), world_vertex(g, a, ta[1]), world_vertex(g, a, ta[2])};
            const P2 bv[3] = {world_vertex(g, b, tb[0]), world_vertex(g, b, tb[1]), world_vertex(g, b, tb[2])};
            P2 normal, p;
            float d;
            if (triangle_contact(av, bv, normal, d, p) && (!found || d > depth)) { found = true; depth = d; n = normal; point = p; }
        }
    return found;
}

// nativeKeyLess / nativeInsertCandidate (NGK:230-251): a row keeps its `limit` smallest keys in order.
bool key_less(const bp_rigid_candidate& a, const bp_rigid_candidate& b) {
    if (a.metadata[0] != b.metadata[0]) return a.metadata[0] < b.metadata[0];
    if (a.participants[0] != b.participants[0]) return a.participants[0] < b.participants[0];
    return a.participants[1] < b.participants[1];
}
void insert_candidate(bp_rigid_candidate* row, uint32_t& count, uint32_t& dropped, uint32_t limit,
                      const bp_rigid_candidate& value) {
    uint32_t location;
    if (count < limit) location = count++;
    else {
        ++dropped;
        if (!key_less(value, row[limit - 1])) return;
        location = limit - 1;
    }
    while (location > 0 && key_less(value, row[location - 1])) { row[location] = row[location - 1]; --location; }
    row[location] = value;
}

// nativeEmitBodyCandidates, body pairs (NGK:394-415, mode `bodies`)
void body_candidates(const bp_rigid_body* bodies, uint32_t count, uint32_t bubbleCount, const uint32_t* ranges,
                     const uint64_t* partners, uint32_t partnerCount, uint32_t limit, bp_rigid_candidate* rows,
                     uint32_t* rowCounts, uint32_t* overflow) {
    for (uint32_t index = 0; index < count; ++index) {
        bp_rigid_candidate* row = rows + (size_t)index * limit;
        uint32_t n = 0, dropped = 0;
        for (uint32_t other = 0; other < count; ++other) {
            if (other == index) continue;
            const uint32_t low = std::min(index, other), high = std::max(index, other);
            const bp_rigid_body& a = bodies[low];
            const bp_rigid_body& c = bodies[high];
            if (immovable(a) && immovable(c)) continue;
            if (!accepts(a.filter, c.filter)) continue;
            if (excluded(ranges, partners, partnerCount, bubbleCount + index, bodies[other].id)) continue;
            const P2 start = p2(a.previous[0], a.previous[1]) - p2(c.previous[0], c.previous[1]);
            const P2 end = p2(a.pose[0], a.pose[1]) - p2(c.pose[0], c.pose[1]);
            const P2 travel = end - start;
            const float travelSquared = dot(travel, travel);
            const float t = travelSquared > kMin ? clampf(-dot(start, travel) / travelSquared, 0.0f, 1.0f) : 0.0f;
            const float radius = 1.25f * (a.physical[2] + c.physical[2]);
            const P2 closestPoint = start + travel * t;
            if (!(dot(closestPoint, closestPoint) <= radius * radius)) continue;
            bp_rigid_candidate value{};
            value.participants[0] = (int64_t)a.id; value.participants[1] = (int64_t)c.id;
            value.metadata[0] = 3; value.metadata[1] = low; value.metadata[2] = high; value.metadata[3] = 0;
            insert_candidate(row, n, dropped, limit, value);
        }
        rowCounts[2 * index] = n;
        rowCounts[2 * index + 1] = 0;  // no bubble candidates in the body-pair rows
        overflow[0] += dropped;
        overflow[1] = std::max(overflow[1], n + dropped);
    }
}

inline float as_float(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
inline uint32_t as_uint(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }

// A candidate row entry points at bodies inside the array.
inline bool candidate_ok(const bp_rigid_candidate& c, uint32_t count) { return c.metadata[1] < count && c.metadata[2] < count; }

// nativeRigidContacts (NCK:375-427), one row slot.
void contact_slot(const Geo& g, const bp_rigid_body* bodies, uint32_t count, bp_rigid_candidate& candidate,
                  bp_rigid_correction& correction, uint32_t* safety) {
    const bp_rigid_correction previous = correction;
    bp_rigid_correction result{};
    result.first[3] = previous.first[3]; result.second[3] = previous.second[3];
    result.velocity_first[3] = previous.velocity_first[3]; result.velocity_second[3] = previous.velocity_second[3];
    correction = result;
    if (candidate.metadata[0] != 3) return;
    if (!candidate_ok(candidate, count)) { *safety |= BP_RIGID_SAFETY_INVALID; return; }
    const uint32_t ai = candidate.metadata[1], bi = candidate.metadata[2];
    const bp_rigid_body& a = bodies[ai];
    const bp_rigid_body& b = bodies[bi];
    if (ai >= bi || (immovable(a) && immovable(b))) return;
    if (!geometry_ok(g, a) || !geometry_ok(g, b)) { *safety |= BP_RIGID_SAFETY_INVALID; return; }
    const P2 end = p2(a.pose[0], a.pose[1]) - p2(b.pose[0], b.pose[1]);
    const float radius = a.physical[2] + b.physical[2], radiusSquared = radius * radius;
    if (dot(end, end) > radiusSquared) return;
    P2 n, point;
    float depth;
    if (!pair_contact(g, a, b, n, depth, point)) return;
    const float wa = a.physical[0], wb = b.physical[0], ia = a.physical[1], ib = b.physical[1];
    const P2 ra = point - p2(a.pose[0], a.pose[1]), rb = point - p2(b.pose[0], b.pose[1]);
    const P2 va = p2(a.motion[0], a.motion[1]), vb = p2(b.motion[0], b.motion[1]);
    const float spinA = a.motion[2], spinB = b.motion[2];
    const float frictionA = a.physical[3], frictionB = b.physical[3];
    const float restitutionA = as_float(a.flags[3]), restitutionB = as_float(b.flags[3]);
    const float ca = cross(ra, n), cb = cross(rb, n), denom = wa + wb + ia * ca * ca + ib * cb * cb;
    if (depth < -0.001f || denom <= kMin) return;
    const float lambda = std::fmax(0.0f, depth) / denom * 0.5f;
    candidate.metadata[3] = as_uint(as_float(candidate.metadata[3]) + lambda);
    const P2 moveA = neg(n) * wa * lambda, moveB = n * wb * lambda;
    correction.first[0] = moveA.x; correction.first[1] = moveA.y; correction.first[2] = -ca * ia * lambda;
    correction.first[3] = n.x;
    correction.second[0] = moveB.x; correction.second[1] = moveB.y; correction.second[2] = cb * ib * lambda;
    correction.second[3] = n.y;
    const float closing = dot(vb - va, n) + spinB * cb - spinA * ca;
    const float friction = std::sqrt(std::fmax(0.0f, frictionA * frictionB));
    const float restitution = std::fmax(restitutionA, restitutionB);
    const float impulse = std::fmax(0.0f, -closing) * (1.0f + restitution) / denom * 0.5f;
    const P2 tangent = p2(-n.y, n.x);
    const float tangentSpeed = dot(vb - va, tangent) + spinB * cross(rb, tangent) - spinA * cross(ra, tangent);
    const float tangentImpulse = -tangentSpeed * friction / denom * 0.5f;
    const P2 vA = neg(n) * wa * impulse - tangent * wa * tangentImpulse;
    const P2 vB = n * wb * impulse + tangent * wb * tangentImpulse;
    correction.velocity_first[0] = vA.x; correction.velocity_first[1] = vA.y;
    correction.velocity_first[2] = -ca * ia * impulse - cross(ra, tangent) * ia * tangentImpulse;
    correction.velocity_first[3] = point.x;
    correction.velocity_second[0] = vB.x; correction.velocity_second[1] = vB.y;
    correction.velocity_second[2] = cb * ib * impulse + cross(rb, tangent) * ib * tangentImpulse;
    correction.velocity_second[3] = point.y;
}

// nativeRigidOverlapAt / nativeRigidTimeOfImpact (NPK:200-233)
bool overlap_at(const Geo& g, bp_rigid_body a, bp_rigid_body b, float t) {
    a.pose[0] = a.previous[0] + (a.pose[0] - a.previous[0]) * t; a.pose[1] = a.previous[1] + (a.pose[1] - a.previous[1]) * t;
    a.pose[2] = a.pose[3] + (a.pose[2] - a.pose[3]) * t;
    b.pose[0] = b.previous[0] + (b.pose[0] - b.previous[0]) * t; b.pose[1] = b.previous[1] + (b.pose[1] - b.previous[1]) * t;
    b.pose[2] = b.pose[3] + (b.pose[2] - b.pose[3]) * t;
    P2 n, point;
    float depth;
    return pair_contact(g, a, b, n, depth, point) && depth > 1e-3f;
}
float time_of_impact(const Geo& g, const bp_rigid_body& a, const bp_rigid_body& b) {
    const P2 da = p2(a.pose[0], a.pose[1]) - p2(a.previous[0], a.previous[1]);
    const P2 db = p2(b.pose[0], b.pose[1]) - p2(b.previous[0], b.previous[1]);
    const float travel = length(da - db) + std::fabs(a.pose[2] - a.pose[3]) * a.physical[2] +
                         std::fabs(b.pose[2] - b.pose[3]) * b.physical[2];
    if (!(travel > 0.5f)) return 2;
    if (overlap_at(g, a, b, 0)) return 2;
    const float samples = std::ceil(travel / 0.5f);
    const uint32_t steps = samples >= 64.0f ? 64u : std::max(2u, (uint32_t)samples);
    float last = 0;
    for (uint32_t step = 1; step <= steps; ++step) {
        const float t = (float)step / (float)steps;
        if (!overlap_at(g, a, b, t)) { last = t; continue; }
        float low = last, high = t;
        for (int bisection = 0; bisection < 12; ++bisection) {
            const float middle = 0.5f * (low + high);
            if (overlap_at(g, a, b, middle)) high = middle; else low = middle;
        }
        return low;
    }
    return 2;
}

// nativeRigidGuardWalls (NPK:118-170), one body.
void guard_body(const Geo& g, bp_rigid_body* bodies, uint32_t count, uint32_t index, uint32_t bubbleCount,
                const uint32_t* ranges, const uint64_t* partners, uint32_t partnerCount, uint32_t* safety) {
    if (bodies[index].flags[0] || bodies[index].filter[2]) return;
    bp_rigid_body b = bodies[index];
    if (!geometry_ok(g, b)) { *safety |= BP_RIGID_SAFETY_INVALID; return; }
    for (uint32_t j = 0; j < count; ++j) {
        const bp_rigid_body& wall = bodies[j];
        if (!wall.flags[0] || is_round(wall) || !accepts(b.filter, wall.filter)) continue;
        if (excluded(ranges, partners, partnerCount, bubbleCount + index, wall.id)) continue;
        if (!geometry_ok(g, wall)) { *safety |= BP_RIGID_SAFETY_INVALID; continue; }
        const uint32_t wn = wall.ranges[1];
        for (uint32_t k = 0; k < b.ranges[1]; ++k) {
            const P2 p = world_vertex(g, b, k);
            const P2 start = p2(b.previous[0], b.previous[1]) + rotate(local_vertex(g, b, k), b.pose[3]);
            const bool inside = rigid_inside(g, p, wall);
            bool startedInside = rigid_inside(g, start, wall);
            if (startedInside)
                for (uint32_t e = 0; e < wn; ++e) {
                    const P2 ea = world_vertex(g, wall, e), eb = world_vertex(g, wall, (e + 1) % wn);
                    if (distance(start, closest(start, ea, eb)) < 1e-5f) { startedInside = false; break; }
                }
            float nearest = std::numeric_limits<float>::infinity(), depth = 0;
            P2 normal = p2(0, 0);
            for (uint32_t e = 0; e < wn; ++e) {
                const P2 ea = world_vertex(g, wall, e), eb = world_vertex(g, wall, (e + 1) % wn);
                const P2 direction = eb - ea;
                const P2 raw = p2(direction.y, -direction.x);
                const P2 out = raw / length(raw);
                const float signedStart = dot(start - ea, out);
                const bool onBoundary = distance(start, closest(start, ea, eb)) < 1e-5f;
                const bool crossing = signedStart >= -1e-5f &&
                                      (center_crossing(start, p, ea, eb, ea, eb) || (onBoundary && dot(p - ea, out) < 0));
                if (!inside && !crossing) continue;
                if (inside && !startedInside && signedStart < -1e-5f) continue;
                const P2 c = closest(p, ea, eb);
                const float d = (crossing || !startedInside) ? distance(start, closest(start, ea, eb)) : distance(p, c);
                if (d < nearest) { nearest = d; normal = out; depth = std::fmax(0.0f, -dot(p - c, out)); }
            }
            if (std::isfinite(nearest) && depth > 0) {
                if (is_round(b)) {
                    bp_rigid_body old = b;
                    old.pose[0] = b.previous[0]; old.pose[1] = b.previous[1]; old.pose[2] = b.pose[3];
                    if (round_core_crosses_polygon(g, core_of(g, old), wall)) break;
                }
                const P2 shift = normal * (depth + 1e-5f);
                b.pose[0] = b.pose[0] + shift.x; b.pose[1] = b.pose[1] + shift.y;
                const P2 r = p - p2(b.pose[0], b.pose[1]);
                const float lever = cross(r, normal);
                const float speed = dot(p2(b.motion[0], b.motion[1]), normal) + b.motion[2] * lever;
                const float denom = b.physical[0] + b.physical[1] * lever * lever;
                const float impulse = std::fmax(0.0f, -speed) / std::fmax(denom, kMin);
                const P2 dv = normal * b.physical[0] * impulse;
                b.motion[0] = b.motion[0] + dv.x; b.motion[1] = b.motion[1] + dv.y;
                b.motion[2] = b.motion[2] + lever * b.physical[1] * impulse;
            }
        }
    }
    bodies[index] = b;
}

}  // namespace rigid

extern "C" {

// (cos, sin) pairs of the library's float sin / cos, for the accuracy test against double precision.
int bpo_sincos(const float* x, float* out, uint32_t count) {
    for (uint32_t i = 0; i < count; ++i) {
        const rigid::P2 cs = rigid::sincos_cw(x[i]);
        out[2 * i] = cs.x;
        out[2 * i + 1] = cs.y;
    }
    return BP_OK;
}

int bpo_rigid_predict(bp_rigid_body* bodies, uint32_t body_count, const float* vertices_xy, uint32_t vertex_count,
                      const bp_segment* segments, uint32_t segment_count, uint32_t bubble_count, float time_step,
                      const uint32_t* joint_ranges, const uint64_t* joint_partners, uint32_t partner_count,
                      bp_rigid_wall* walls, uint32_t* safety) {
    rigid::Sweep in{vertices_xy, segments, segment_count, 0, joint_ranges ? partner_count : 0u, joint_ranges, joint_partners};
    rigid::predict(bodies, body_count, in, vertex_count, bubble_count, time_step, walls, safety);
    return BP_OK;
}

// `iterations` Jacobi rounds of nativeSolveJoints (every joint from the same state) then nativeApplyJointBodies
// (NCK:546-562: each body adds its list's corrections in order, times 1 / count).
int bpo_rigid_solve_joints(bp_rigid_body* bodies, uint32_t body_count, bp_rigid_joint* joints, uint32_t joint_count,
                           bp_rigid_correction* corrections, const uint32_t* references, uint32_t reference_count,
                           const uint32_t* joint_ranges, uint32_t bubble_count, float time_step,
                           uint32_t iteration_count, uint32_t iterations, uint32_t* safety) {
    if (joint_count == 0) return BP_OK;
    const float dt = std::fmax(time_step, 1e-6f);
    for (uint32_t round = 0; round < iterations; ++round) {
        for (uint32_t j = 0; j < joint_count; ++j)
            rigid::solve(joints[j], corrections[j], bodies, body_count, bubble_count, dt, iteration_count, safety);
        for (uint32_t i = 0; i < body_count; ++i) {
            const uint32_t* range = joint_ranges + 4 * (size_t)(bubble_count + i);
            if (range[1] == 0) continue;
            float delta[3] = {0, 0, 0}, velocity[3] = {0, 0, 0};
            bool ok = true;
            for (uint32_t r = 0; r < range[1]; ++r) {
                const uint32_t at = range[0] + r;
                if (at >= reference_count || references[2 * at] >= joint_count) { ok = false; break; }
                const bp_rigid_correction& c = corrections[references[2 * at]];
                const bool second = references[2 * at + 1] != 0;
                for (int q = 0; q < 3; ++q) {
                    delta[q] = delta[q] + (second ? c.second[q] : c.first[q]);
                    velocity[q] = velocity[q] + (second ? c.velocity_second[q] : c.velocity_first[q]);
                }
            }
            if (!ok) { *safety |= BP_RIGID_SAFETY_INVALID; continue; }
            const float relax = 1.0f / (float)range[1];
            for (int q = 0; q < 3; ++q) {
                bodies[i].pose[q] = bodies[i].pose[q] + delta[q] * relax;
                bodies[i].motion[q] = bodies[i].motion[q] + velocity[q] * relax;
            }
        }
    }
    return BP_OK;
}

int bpo_rigid_finish(bp_rigid_body* bodies, uint32_t body_count, const float* vertices_xy, uint32_t vertex_count,
                     const float* region, uint32_t* safety) {
    rigid::finish(bodies, body_count, vertices_xy, vertex_count, region, safety);
    return BP_OK;
}

int bpo_rigid_body_candidates(const bp_rigid_body* bodies, uint32_t body_count, uint32_t bubble_count,
                              const uint32_t* joint_ranges, const uint64_t* joint_partners, uint32_t partner_count,
                              uint32_t row_width, bp_rigid_candidate* rows, uint32_t* row_counts, uint32_t* overflow) {
    rigid::body_candidates(bodies, body_count, bubble_count, joint_ranges, joint_partners,
                           joint_ranges ? partner_count : 0u, row_width, rows, row_counts, overflow);
    return BP_OK;
}

// nativeRigidResolveCCD then nativeRigidApplyCCD (NPK:235-263): every body's earliest impact from the state before
// any body moves back, then the moves.
int bpo_rigid_ccd(bp_rigid_body* bodies, uint32_t body_count, const float* vertices_xy, uint32_t vertex_count,
                  const uint32_t* triangles, uint32_t triangle_count, const bp_rigid_candidate* rows,
                  const uint32_t* row_counts, uint32_t row_width, uint32_t* safety) {
    const rigid::Geo g{vertices_xy, vertex_count, triangles, triangle_count};
    std::vector<float> marker(body_count, 0.0f);
    for (uint32_t index = 0; index < body_count; ++index) {
        float earliest = 2;
        if (!rigid::immovable(bodies[index])) {
            const uint32_t n = std::min(row_counts[2 * index], row_width);
            for (uint32_t slot = row_counts[2 * index + 1]; slot < n; ++slot) {
                const bp_rigid_candidate& c = rows[(size_t)index * row_width + slot];
                if (c.metadata[0] != 3) continue;
                if (!rigid::candidate_ok(c, body_count) || !rigid::geometry_ok(g, bodies[c.metadata[1]]) ||
                    !rigid::geometry_ok(g, bodies[c.metadata[2]])) { *safety |= BP_RIGID_SAFETY_INVALID; continue; }
                earliest = std::fmin(earliest, rigid::time_of_impact(g, bodies[c.metadata[1]], bodies[c.metadata[2]]));
            }
        }
        marker[index] = earliest <= 1 ? 1 + earliest : 0;
    }
    for (uint32_t index = 0; index < body_count; ++index) {
        bp_rigid_body& b = bodies[index];
        b.limits[2] = marker[index];
        if (b.limits[2] >= 1) {
            const float t = b.limits[2] - 1;
            b.pose[0] = b.previous[0] + (b.pose[0] - b.previous[0]) * t;
            b.pose[1] = b.previous[1] + (b.pose[1] - b.previous[1]) * t;
            b.pose[2] = b.pose[3] + (b.pose[2] - b.pose[3]) * t;
        }
        b.limits[2] = 0;
    }
    return BP_OK;
}

// One round of nativeRigidContacts (every slot from the same state) then nativeRigidApplyBodies (NCK:375-444).
int bpo_rigid_solve_contacts(bp_rigid_body* bodies, uint32_t body_count, const float* vertices_xy, uint32_t vertex_count,
                             const uint32_t* triangles, uint32_t triangle_count, bp_rigid_candidate* rows,
                             const uint32_t* row_counts, uint32_t row_width, bp_rigid_correction* corrections,
                             uint32_t* safety) {
    const rigid::Geo g{vertices_xy, vertex_count, triangles, triangle_count};
    for (uint32_t owner = 0; owner < body_count; ++owner) {
        const uint32_t n = std::min(row_counts[2 * owner], row_width);
        for (uint32_t slot = 0; slot < n; ++slot) {
            const size_t at = (size_t)owner * row_width + slot;
            rigid::contact_slot(g, bodies, body_count, rows[at], corrections[at], safety);
        }
    }
    for (uint32_t index = 0; index < body_count; ++index) {
        float delta[3] = {0, 0, 0}, velocity[3] = {0, 0, 0};
        const uint32_t n = std::min(row_counts[2 * index], row_width);
        for (uint32_t slot = 0; slot < n; ++slot) {
            const size_t at = (size_t)index * row_width + slot;
            const bool first = rows[at].metadata[0] == 3 && rows[at].metadata[1] == index;
            const bp_rigid_correction& c = corrections[at];
            for (int q = 0; q < 3; ++q) {
                delta[q] = delta[q] + (first ? c.first[q] : c.second[q]);
                velocity[q] = velocity[q] + (first ? c.velocity_first[q] : c.velocity_second[q]);
            }
        }
        for (int q = 0; q < 3; ++q) {
            bodies[index].pose[q] = bodies[index].pose[q] + delta[q];
            bodies[index].motion[q] = bodies[index].motion[q] + velocity[q];
        }
    }
    return BP_OK;
}

// nativeRigidGuardWalls (NPK:118-170): each dynamic body in turn against the static polygons; a body only writes
// itself and reads static bodies, so the order does not matter.
int bpo_rigid_guard_walls(bp_rigid_body* bodies, uint32_t body_count, const float* vertices_xy, uint32_t vertex_count,
                          const uint32_t* triangles, uint32_t triangle_count, uint32_t bubble_count,
                          const uint32_t* joint_ranges, const uint64_t* joint_partners, uint32_t partner_count,
                          uint32_t* safety) {
    const rigid::Geo g{vertices_xy, vertex_count, triangles, triangle_count};
    for (uint32_t index = 0; index < body_count; ++index)
        rigid::guard_body(g, bodies, body_count, index, bubble_count, joint_ranges, joint_partners,
                          joint_ranges ? partner_count : 0u, safety);
    return BP_OK;
}

}  // extern "C"
