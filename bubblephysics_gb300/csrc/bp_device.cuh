// bp_device.cuh - device data layout and per-pair / per-object arithmetic of the bubble step on sm_103a.
//
// Layout in HBM (all SoA, one slot per bubble of every resident world, worlds back to back):
//   pos, start, vel, acc, a0, ref, rotw : float2     (centre, step-start centre, velocity, acceleration, non-contact
//                                                     acceleration, x0 of the last grid build, rotation / omega)
//   phys                                 : float4     (radius, inverse mass, K_c, gamma)
//   margin                               : float
//   id                                   : int64, flags / result : uint32, filter : uint2 (category, mask)
//   cell                                 : longlong2  (grid cell of the last build)
//   cand rows, adjacency rows            : k x uint32 per bubble (k = candidate limit of the world)
// Segments, bodies, field records are small arrays of records with absolute offsets into shared vertex arrays.
//
// All arithmetic is FP32 and follows the operation order of the reference kernels
// (Sources/BubblePhysicsNativeMetal/Shaders/NativeForceKernels.metal-source = NFK,
//  NativeGeometryKernels.metal-source = NGK); the library is compiled with -fmad=false so no multiply-add is fused.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/bubblephysics.h"

namespace bp {

constexpr uint32_t kFrameLimit = 1024;   // NFK:384 nativeSubstepFrameLimit
constexpr uint32_t kNewtonSteps = 12;    // NFK:39 nativePairNewtonSteps
constexpr uint32_t kRemoved = 0x80000000u;
constexpr uint32_t kKindShift = 30;
constexpr uint32_t kIndexMask = 0x3fffffffu;
constexpr float kFltMin = 1.17549435e-38f;
constexpr float kFltMax = 3.40282347e+38f;

// Per-world table entry (device). Offsets are absolute indices into the shared arrays.
struct DWorld {
    uint32_t boff, n, soff, s;
    uint32_t bodyOff, nb, foff, nf;
    uint32_t bandOff, nbands, motorOff, nmotors;
    uint32_t jrOff, njEnt, k, flags;
    uint32_t injectSubstep, contactCap, threads, treeOff;  // treeOff: first leaf of the world's LBVH arrays
    uint64_t rowOff;       // candidate / adjacency rows: entries rowOff + i * k
    uint64_t bodyRowOff;   // body rows: bodyRowOff + b * k
    uint64_t contactOff;   // contact records
    float dt, sepTol, contactTol, split;
    float2 rmin, rmax, gforce, gravity, injectPos;
    int64_t injectObject;
    uint32_t failed, tree;  // tree: 1 when rigid candidates go through the LBVH
};

struct DSegment {
    float2 a, b, prev;
    float outward, allowed;
    uint32_t flags, cat, mask, pad;
    int64_t id, owner;
};

struct DBody {
    float2 pos, prev;        // end-of-step pose after the kinematic advance, start-of-step pose
    float angle, prevAngle;
    float2 vel;
    float omega, radius, coreRadius, pad;
    float cosPrev, sinPrev, cosEnd, sinEnd;
    uint32_t kind, flags, voff, vcount, toff, tcount, cat, mask;
    int64_t id;
};

struct DField {
    float2 pos;
    float cosr, sinr, falloff, strength, radius, pad;
    float2 dir;
    uint32_t kind, voff, vcount, foff, fcount, hasFilter;
};

// Compact box of a rigid object for the broadphase tests: a segment's [min(a,b), max(a,b)] or a body's swept box
// [min(pos, prev) - R, max(pos, prev) + R]; `flags` holds the segment flags / the body-is-obstacle bit.
struct RigidBox {
    float4 box;  // lo.xy, hi.xy
    uint32_t cat, mask, flags, pad;
};

// Internal node of a world's LBVH over its rigid leaves, child boxes stored inline so a traversal reads one node to
// test both children. A child index with kTreeLeaf set is a sorted leaf position, otherwise an internal node.
struct TreeNode {
    float4 box[2];     // lo.xy, hi.xy of the left and right child (leaf boxes widened by the body hull radius)
    uint32_t child[2];
    uint32_t parent, pad;
};
constexpr uint32_t kTreeLeaf = 0x80000000u;

// End-of-step contact record, index form (ids are looked up on the host).
struct DContact {
    uint32_t a, other, kind, feature;
    float2 normal, point;
    float impulse, penetration, allowed, pad;
};

struct DState {
    const DWorld* worlds;
    bp_step_report* reports;
    float* history;            // kFrameLimit per world
    uint32_t* contactCount;    // per world
    // bubbles
    float2 *pos, *start, *vel, *acc, *a0, *ref, *rotw;
    float4* phys;
    float* margin;
    const int64_t* id;
    uint32_t *flags, *result;
    const uint2* filter;
    longlong2* cell;
    longlong2* acell;          // cells of the assertion grid (current centres; x = INT64_MIN when not gridded)
    uint32_t* candRow;         // k per bubble
    uint2* candCount;          // (pairs kept, segments kept)
    uint32_t* pairTotal;       // pairs found before the k limit
    uint32_t* adj;             // k per bubble
    uint32_t* deg;
    float2 *pPos, *pStart, *pVel, *pRotw;
    uint32_t *pResult, *pFlags;
    // segments, bodies, forces, joints
    const DSegment* seg;
    DBody* body;
    DBody* pBody;
    const float2* bverts;
    const uint32_t* btris;     // triples
    uint32_t* bodyRow;         // k per body
    uint32_t* bodyTotal;
    const DField* fields;
    const float2* fverts;
    const int64_t* fids;
    const bp_band* bands;
    const bp_motor* motors;
    const uint2* jranges;      // per entity (bubbles, then bodies) of a world, from jrOff
    const int64_t* jpartners;
    DContact* contacts;
    uint32_t* failed;          // per world: stopped after a failed step
    uint32_t* scanA;           // per bubble scratch (contact offsets)
    uint32_t* scanB;
    // large-world (grid team) scratch
    float* gpv;                // 2 x grid partial values
    uint32_t* gpo;             // 2 x grid partial owners / counts
    uint32_t* gbuckets;        // hash grid buckets
    uint32_t* gentries;        // hash grid entries
    float4* grecords;          // hash grid entry records (centre, radius, margin) in entry order
    unsigned int* barrier;     // grid barrier counters [arrivals, generation]
    uint32_t* errorFlag;       // bounded-wait failures
    unsigned long long* phaseCycles;  // kPhaseCount per world when built with BP_PHASE_TIMING, else null
    float4* bpose;             // per body: pose at the current step fraction (position.xy, cos, sin)
    RigidBox* segBox;          // per segment
    RigidBox* bodyBox;         // per body (rebuilt every step: kinematic bodies move)
    // LBVH over the rigid leaves of worlds with W.tree set (entries from W.treeOff, s + nb per world)
    unsigned long long* tKeys;     // sorted keys (morton << 32 | leaf)
    unsigned long long* tKeysAlt;  // radix-sort ping-pong
    uint32_t* tCounts;             // 16 digit counters per leaf (radix-sort scratch)
    TreeNode* tNodes;              // s + nb - 1 internal nodes (node 0 is the root)
    uint32_t* tLeafParent;         // per sorted leaf: (parent node << 1) | side
    uint32_t* tVisit;              // per internal node: children finished (bottom-up refit)
    uint32_t* tValid;              // per world: 1 when the last step built its tree
};

constexpr uint32_t kPhaseCount = 26;  // profiling builds: 24 cycle counters, then the start and end times of the world's last step

// Work queues of one persistent step launch (see persistent_step_kernel). The lists and their lengths live in device
// memory so the on-device scheduler can reorder them between steps without a host round trip.
struct QueueArgs {
    const uint32_t* ctaList;   // worlds stepped by a whole block, most expensive first
    const uint32_t* warpList;  // worlds of the group queue (one group of groupWidth threads each), most expensive first
    uint32_t* queue;           // [0] next CTA world, [1] next warp world (zeroed before each launch),
                               // [2] CTA list length, [3] warp list length
    uint32_t nCta, ctaB, ctaMaxN;     // ctaMaxN / warpMaxN size the shared-memory grid of one team (warp*: the group queue)
    uint32_t nWarp, warpB, warpMaxN;
    uint32_t countsOnDevice;          // 1: list lengths are queue[2], queue[3]; 0: nCta, nWarp
    uint32_t ctaWsWords, warpWsWords; // shared-memory workspace of one team (32-bit words) after its grid
    uint32_t tree;                    // 1: some world uses the LBVH (launch the tree-capable kernel)
    uint32_t groupWidth;              // threads of one group-queue team: 32 (a warp), 64, 128 or 256 (<= block width)
};

__host__ __device__ inline uint32_t round4_words(uint32_t v) { return (v + 3u) & ~3u; }
// Words of a team's hash grid in shared memory: B bucket ends and the entries of its largest world (padded to 16
// bytes), then 16-byte records: one per entry (centre, radius, margin of the entry's bubble) that the candidate scan
// reads instead of the bubble's own arrays, and at least one per thread of the team (`width` threads), whose slots the
// row-term passes use between grid builds.
__host__ __device__ inline uint32_t grid_words(uint32_t B, uint32_t maxN, uint32_t width) {
    return round4_words(B + maxN) + 4u * (maxN > width ? maxN : width);
}

// Per-team copies of the world's table entry and state pointers, kept in SHARED memory for the whole step: S is the
// state a team reads and writes (its hot arrays redirected into the shared-memory workspace when the world is staged),
// G the world's arrays in global memory (the served kernel's per-world state; the batched kernels read G from their
// parameter). In shared memory every access is a broadcast load; a per-thread copy would live in local memory, one
// copy per thread.
struct TeamState {
    DState S;
    DState G;
    DWorld W;
};
constexpr uint32_t kTeamStateWords = (uint32_t)((sizeof(TeamState) + 15u) / 16u * 4u);

// Shared-memory slice of one group of the group queue, in 32-bit words: the group's TeamState, its reduction scratch
// (groups wider than a warp; a BlockScratch), then its hash grid (B bucket ends, then the entries of its largest
// world), then its workspace.
constexpr uint32_t kGroupScratchWords = 308;
__host__ __device__ inline uint32_t group_scratch_words(uint32_t width) {
    return kTeamStateWords + (width > 32u ? kGroupScratchWords : 0u);
}
__host__ __device__ inline uint32_t group_slice_words(const QueueArgs& q) {
    return group_scratch_words(q.groupWidth) + grid_words(q.warpB, q.warpMaxN, q.groupWidth > 32u ? q.groupWidth : 32u) +
           q.warpWsWords;
}

constexpr float kPiF = 3.14159265358979323846f;

// Contour samples of a bubble of radius r (nativeAccumulateContactPressure, NativePostSolveKernels:292):
// max(64, ceil((r / maxEdge) * 4 pi)), at most `stride`.
// The whole-GPU team's 8-bit key sort (one block of 16 warps): one 256-digit histogram per warp in dynamic shared
// memory, given to the launches of worlds that build a tree.
constexpr uint32_t kRadixWarps = 16u, kRadixDigits = 256u;
constexpr uint32_t kRadixHistBytes = kRadixWarps * kRadixDigits * 4u;

// Index of the first direction of a bubble with `count` samples in the direction table (the tables of counts 1, 2, ...
// one after another).
__host__ __device__ inline uint32_t contour_dir_offset(uint32_t count) { return count * (count - 1u) / 2u; }

__host__ __device__ inline uint32_t contour_samples(float r, float maxEdge, uint32_t stride) {
    const float q = (r / maxEdge) * (4.0f * kPiF);
    const uint32_t want = (uint32_t)ceilf(q);
    const uint32_t count = want > 64u ? want : 64u;
    return count < stride ? count : stride;
}

// Bytes of a world's shared-memory workspace: per bubble 88 B of hot state, per segment and body a 32 B box, per body
// a 16 B pose; the 15 parts are each padded to 16 bytes.
__host__ __device__ inline uint32_t workspace_bytes(uint32_t n, uint32_t s, uint32_t nb) {
    return n * 88u + s * 32u + nb * 48u + 15u * 16u;
}

// ------------------------------------------------------------------------------------------------------------------
// float2 helpers (Metal semantics restated: length = sqrt(x*x + y*y), min/max = fmin/fmax)
// ------------------------------------------------------------------------------------------------------------------
__device__ __forceinline__ float2 f2(float x, float y) { return make_float2(x, y); }
__device__ __forceinline__ float2 add(float2 a, float2 b) { return f2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 sub(float2 a, float2 b) { return f2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 mul(float2 a, float s) { return f2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 dvd(float2 a, float s) { return f2(a.x / s, a.y / s); }
__device__ __forceinline__ float dot2(float2 a, float2 b) { return a.x * b.x + a.y * b.y; }
__device__ __forceinline__ float len2(float2 a) { return sqrtf(a.x * a.x + a.y * a.y); }
__device__ __forceinline__ float2 vmin2(float2 a, float2 b) { return f2(fminf(a.x, b.x), fminf(a.y, b.y)); }
__device__ __forceinline__ float2 vmax2(float2 a, float2 b) { return f2(fmaxf(a.x, b.x), fmaxf(a.y, b.y)); }
__device__ __forceinline__ float clampf(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }
__device__ __forceinline__ bool finite2(float2 a) { return isfinite(a.x) && isfinite(a.y); }
__device__ __forceinline__ float cross2(float2 a, float2 b) { return a.x * b.y - a.y * b.x; }
__device__ __forceinline__ float2 rot_cs(float2 p, float c, float s) { return f2(p.x * c - p.y * s, p.x * s + p.y * c); }

struct Law {
    float force, epsA, epsB, stiffness;
};

// nativeEpsilonFromForceRatio / nativeRestFromForceRatio, NFK:50-57
__device__ __forceinline__ float eps_from_ratio(float q) {
    if (!(q > 0.0f)) return 0.0f;
    return 2.0f * q / ((2.0f * q + 1.0f) + sqrtf(4.0f * q + 1.0f));
}
__device__ __forceinline__ float rest_from_ratio(float q) { return 2.0f / (1.0f + sqrtf(fmaxf(4.0f * q, 0.0f) + 1.0f)); }

// nativeWallContactLaw, NFK:60-69
__device__ __forceinline__ Law wall_law(float K, float r, float distance) {
    Law law{0.0f, 0.0f, 0.0f, 0.0f};
    float d = fmaxf(distance, r * 1e-6f);
    if (!(K > 0.0f) || !(r > 0.0f) || !(d < r)) return law;
    float rest = d / r;
    law.epsA = (r - d) / r;
    law.force = K * (r - d) * r / (d * d);
    law.stiffness = K * (1.0f + law.epsA) / (r * rest * rest * rest);
    return law;
}

// nativePairContactLaw, NFK:75-102. Same material: closed form; different: 12 Newton steps from the K_min bound.
__device__ __forceinline__ Law pair_law(float Ka, float ra, float Kb, float rb, float distance) {
    Law law{0.0f, 0.0f, 0.0f, 0.0f};
    float R = ra + rb;
    float d = fmaxf(distance, R * 1e-6f);
    float overlap = R - d;
    if (!(Ka > 0.0f) || !(Kb > 0.0f) || !(overlap > 0.0f)) return law;
    float lowest = fminf(Ka, Kb) * overlap * R / (d * d);
    float force = lowest;
    if (Ka != Kb) {
        for (uint32_t step = 0; step < kNewtonSteps; ++step) {
            float qa = force / Ka, qb = force / Kb;
            float ea = eps_from_ratio(qa), eb = eps_from_ratio(qb);
            float sa = rest_from_ratio(qa), sb = rest_from_ratio(qb);
            float residual = ra * ea + rb * eb - overlap;
            float slope = ra * sa * sa * sa / ((1.0f + ea) * Ka) + rb * sb * sb * sb / ((1.0f + eb) * Kb);
            if (!(slope > kFltMin)) break;
            force = fmaxf(force - residual / slope, lowest);
        }
    }
    float qa = force / Ka, qb = force / Kb;
    float ea = eps_from_ratio(qa), eb = eps_from_ratio(qb);
    float sa = rest_from_ratio(qa), sb = rest_from_ratio(qb);
    float compliance = ra * sa * sa * sa / ((1.0f + ea) * Ka) + rb * sb * sb * sb / ((1.0f + eb) * Kb);
    law.force = force;
    law.epsA = ea;
    law.epsB = eb;
    law.stiffness = compliance > kFltMin ? 1.0f / compliance : 0.0f;
    return law;
}

// nativeFilterAccepts, NGK:124-126
__device__ __forceinline__ bool filter_accepts(uint2 a, uint2 b) { return (a.x & b.y) != 0u && (b.x & a.y) != 0u; }

// nativeClosestPoint, NGK:437-441
__device__ __forceinline__ float2 closest_point(float2 p, float2 a, float2 b) {
    float2 edge = sub(b, a);
    float square = dot2(edge, edge);
    float t = square > kFltMin ? clampf(dot2(sub(p, a), edge) / square, 0.0f, 1.0f) : 0.0f;
    return add(a, mul(edge, t));
}
// nativePastSegmentEnd, NGK:665-668 (explicit fma, exact complement at a shared vertex)
__device__ __forceinline__ bool past_segment_end(float2 center, float2 from, float2 to) {
    float2 edge = sub(to, from), rel = sub(center, from);
    return fmaf(rel.x, edge.x, rel.y * edge.y) >= fmaf(edge.x, edge.x, edge.y * edge.y);
}

// nativeWallRegion, NFK:112-136
__device__ __forceinline__ bool wall_region(const DSegment& sg, float2 center, float2& normal, float& distance) {
    float2 start = sg.a, end = sg.b, edge = sub(end, start);
    float edgeLength = len2(edge);
    float2 base = edgeLength > 0.0f ? dvd(f2(-edge.y, edge.x), edgeLength) : f2(0.0f, 1.0f);
    if (sg.flags & BP_SEGMENT_POLYGON_EDGE) {
        float2 outward = mul(base, sg.outward);
        float along = dot2(sub(center, start), edge);
        bool convexStart = (sg.flags & BP_SEGMENT_CONVEX_START) != 0u;
        if (convexStart && along <= 0.0f && past_segment_end(center, sg.prev, start)) {
            float2 delta = sub(center, start);
            distance = len2(delta);
            normal = distance > 0.0f ? dvd(delta, distance) : outward;
        } else if (along > 0.0f && !past_segment_end(center, start, end) && dot2(sub(center, start), outward) >= 0.0f) {
            normal = outward;
            distance = dot2(sub(center, start), outward);
        } else {
            return false;
        }
    } else {
        float2 delta = sub(center, closest_point(center, start, end));
        distance = len2(delta);
        normal = distance > 0.0f ? dvd(delta, distance) : base;
    }
    return true;
}

struct Pose {
    float2 pos;
    float c, s;
};
// nativeBodyAtFraction, NFK:155-159; rotations of the two step poses are precomputed, other angles use cosf/sinf.
__device__ __forceinline__ Pose body_at(const DBody& b, float fraction) {
    Pose p;
    p.pos = add(b.prev, mul(sub(b.pos, b.prev), fraction));
    float angle = b.prevAngle + (b.angle - b.prevAngle) * fraction;
    if (angle == b.prevAngle) { p.c = b.cosPrev; p.s = b.sinPrev; }
    else if (angle == b.angle) { p.c = b.cosEnd; p.s = b.sinEnd; }
    else { p.c = cosf(angle); p.s = sinf(angle); }
    return p;
}
__device__ __forceinline__ float2 body_vertex(const float2* verts, const DBody& b, const Pose& p, uint32_t i) {
    return add(p.pos, rot_cs(verts[b.voff + i], p.c, p.s));
}
// nativeRigidInside, NGK:477-490
__device__ __forceinline__ bool rigid_inside(const float2* verts, const uint32_t* tris, float2 pt, const DBody& b, const Pose& p) {
    if (b.kind != BP_BODY_POLYGON) {
        float2 ca = body_vertex(verts, b, p, 0), cb = b.vcount > 1 ? body_vertex(verts, b, p, 1) : ca;
        return len2(sub(pt, closest_point(pt, ca, cb))) <= b.coreRadius;
    }
    float2 local = rot_cs(sub(pt, p.pos), p.c, -p.s);
    for (uint32_t i = 0; i < b.tcount; ++i) {
        const uint32_t* t = tris + 3 * (b.toff + i);
        float2 a = verts[b.voff + t[0]], bb = verts[b.voff + t[1]], c = verts[b.voff + t[2]];
        if (cross2(sub(bb, a), sub(local, a)) >= 0.0f && cross2(sub(c, bb), sub(local, bb)) >= 0.0f &&
            cross2(sub(a, c), sub(local, c)) >= 0.0f)
            return true;
    }
    return false;
}

struct Obstacle {
    float2 normal;
    float distance;
    float speedBound;
};
// nativeBodyObstacle, NFK:170-210 (the point velocity is not used by the step)
__device__ __forceinline__ Obstacle body_obstacle(const float2* verts, const uint32_t* tris, const DBody& b, const Pose& p,
                                                  float2 center) {
    Obstacle o;
    float2 point, normal;
    float distance;
    if (b.kind != BP_BODY_POLYGON) {
        float2 ca = body_vertex(verts, b, p, 0), cb = b.vcount > 1 ? body_vertex(verts, b, p, 1) : ca;
        point = closest_point(center, ca, cb);
        float2 delta = sub(center, point);
        float away = len2(delta);
        float2 axis = sub(cb, ca);
        float axisLength = len2(axis);
        float2 fallback = axisLength > 1e-6f ? dvd(f2(-axis.y, axis.x), axisLength) : f2(0.0f, 1.0f);
        normal = away > 1e-7f ? dvd(delta, away) : fallback;
        distance = away - b.coreRadius;
        point = add(point, mul(normal, b.coreRadius));
    } else {
        float best = __int_as_float(0x7f800000);
        float2 nearest = f2(0.0f, 0.0f), outward = f2(0.0f, 1.0f);
        for (uint32_t e = 0; e < b.vcount; ++e) {
            float2 pp = body_vertex(verts, b, p, e), q = body_vertex(verts, b, p, (e + 1) % b.vcount);
            float2 cand = closest_point(center, pp, q);
            float d = len2(sub(center, cand));
            if (d < best) {
                best = d;
                nearest = cand;
                float2 edge = sub(q, pp);
                float size = len2(edge);
                outward = size > kFltMin ? dvd(f2(edge.y, -edge.x), size) : f2(0.0f, 1.0f);
            }
        }
        bool inside = rigid_inside(verts, tris, center, b, p);
        normal = inside ? outward : (best > 1e-7f ? dvd(sub(center, nearest), best) : outward);
        distance = inside ? -best : best;
        point = nearest;
    }
    float2 arm = sub(point, p.pos);
    o.normal = normal;
    o.distance = distance;
    o.speedBound = len2(b.vel) + fabsf(b.omega) * len2(arm);
    return o;
}

// nativeHalfImpulseFactor, NFK:754-758
__device__ __forceinline__ float half_impulse(float gamma, float halfStep) {
    float x = gamma * halfStep;
    if (x < 0.05f)
        return halfStep * (1.0f - x * 0.5f + x * x * (1.0f / 6) - x * x * x * (1.0f / 24) + x * x * x * x * (1.0f / 120));
    return (1.0f - expf(-x)) / gamma;
}

}  // namespace bp
