// bp_rigid.cu - the rigid body solver on the caller's device arrays: predict, body-pair rows, CCD, contact rounds,
// joint rounds, the wall guard and the finish, one entry per reference kernel (or kernel pair).
//
// The reference steps rigid bodies once per step, before the bubble substeps (NativeMetalSolver.swift:767-799):
// nativeRigidPredict (NativePostSolveKernels.metal-source = NPK:66-115), body-pair candidates and CCD, then 8 rounds
// of {nativeRigidContacts, nativeRigidApplyBodies, nativeSolveJoints, nativeApplyJointBodies, nativeRigidGuardWalls},
// and nativeRigidFinish (NPK:172-198) after the bubble step. Here:
//  - predict, finish, the contact apply and the CCD moves: one thread per body; the contacts: one thread per row slot;
//  - body-pair rows, CCD and the wall guard: one warp per body (see each kernel for how the lanes split the work
//    without changing the reference's order of insertion or correction);
//  - the joint rounds: a round is a Jacobi pass: every joint computes both ends' corrections from the same body state
//    (a thread per joint), then every body adds its joints' corrections in list order (a thread per body). A small
//    world (<= 512 joints, <= 1,024 bodies) runs all rounds in ONE launch of one 512-thread block, the halves
//    separated by __syncthreads(); a larger one runs two grid launches per round, so all SMs share the work.
// Records keep the reference's layouts (bp_rigid_body = NativeRigidBody, 160 B, ...), read as float4 / uint4 words.
// Arithmetic is FP32 in the reference's operation order (built with -fmad=false). sin and cos are this library's own
// float functions (sincos_cw), exp the float of the double-precision exp, so the CPU oracle gets the same bits.
#include <cmath>

#include "bp_device.cuh"

namespace bp {

struct __align__(16) RBody {
    unsigned long long id, reserved;
    float4 pose, previous, motion, physical;
    uint4 ranges, flags, filter;
    float4 shape, limits;
};
struct __align__(16) RJoint {
    unsigned long long id, reserved;
    uint4 ends;
    float4 anchors, parameters, limits, state;
};
struct __align__(16) RCorrection {
    float4 first, second, velocityFirst, velocitySecond;
};
struct __align__(16) RWall {
    long long body, owner;
    float4 geometry, extra;
};
static_assert(sizeof(RBody) == sizeof(bp_rigid_body), "bp_rigid_body layout");
static_assert(sizeof(RJoint) == sizeof(bp_rigid_joint), "bp_rigid_joint layout");
static_assert(sizeof(RCorrection) == sizeof(bp_rigid_correction), "bp_rigid_correction layout");
static_assert(sizeof(RWall) == sizeof(bp_rigid_wall), "bp_rigid_wall layout");

constexpr uint32_t kRigidThreads = 128;
constexpr uint32_t kJointThreads = 512;     // the one block of a small world's joint rounds
constexpr uint32_t kRoundThreads = 128;     // the grid launches of a larger world's rounds
// A world with at most this many joints and bodies runs all rounds in one block (its rotation and damping cache is
// at most 10 KB of shared memory); a larger one runs two grid launches per round.
constexpr uint32_t kSingleBlockJoints = 512, kSingleBlockBodies = 1024;
constexpr float kFltEpsilon = 1.1920929e-7f;

__device__ __forceinline__ bool finite4(float4 v) { return isfinite(v.x) && isfinite(v.y) && isfinite(v.z) && isfinite(v.w); }

// sin and cos of a float angle, this library's own: Cody-Waite reduction by pi/2 (pi/2 split into three floats of
// 8, 11 and 24 bits, so k * C1 and k * C2 are exact for |k| < 8192, |x| < 12867) and the Taylor series of sin and
// cos on |r| <= pi/4 up to r^11 and r^12 (truncation below 1e-11), by Horner. Plain float operations in a fixed
// order, so the CPU oracle computes the same bits; within 2 ulp of the exact values on |x| < 12867.
__device__ __forceinline__ float2 sincos_cw(float x) {
    if (!isfinite(x)) return f2(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
    const float k = rintf(x * 0x1.45f306p-1f);
    const float r = ((x - k * 0x1.92p+0f) - k * 0x1.fb6p-12f) - k * -0x1.777a5cp-25f;
    const float r2 = r * r;
    const float sr = r + r * r2 * (-0x1.555556p-3f + r2 * (0x1.111112p-7f + r2 * (-0x1.a01a02p-13f +
                                   r2 * (0x1.71de3ap-19f + r2 * -0x1.ae6456p-26f))));
    const float cr = 1.0f + r2 * (-0x1.0p-1f + r2 * (0x1.555556p-5f + r2 * (-0x1.6c16c2p-10f +
                                   r2 * (0x1.a01a02p-16f + r2 * (-0x1.27e4fcp-22f + r2 * 0x1.1eed8ep-29f)))));
    const int q = (int)k & 3;
    const float sn = q == 0 ? sr : q == 1 ? cr : q == 2 ? -sr : -cr;
    const float cs = q == 0 ? cr : q == 1 ? -sr : q == 2 ? -cr : sr;
    return f2(cs, sn);  // (cos, sin)
}

// nativeRotate (NativeGeometryKernels.metal-source = NGK:136-138)
__device__ __forceinline__ float2 rotate_by(float2 p, float angle) {
    const float2 cs = sincos_cw(angle);
    return rot_cs(p, cs.x, cs.y);
}

__device__ __forceinline__ float2 normalized(float2 v) { return dvd(v, len2(v)); }

// nativeClampLinearSpeed / nativeClampAngularSpeed (NGK:151-158)
__device__ __forceinline__ float2 clamp_linear(float2 v, float limit) {
    const float speed = len2(v);
    return limit > 0.0f && speed > limit ? mul(v, limit / speed) : v;
}
__device__ __forceinline__ float clamp_angular(float w, float limit) { return limit > 0.0f ? clampf(w, -limit, limit) : w; }

// Metal mix(x, y, t) = x + (y - x) * t, per component of (x, y, angle).
__device__ __forceinline__ float3 mix3(float3 x, float3 y, float t) {
    return make_float3(x.x + (y.x - x.x) * t, x.y + (y.y - x.y) * t, x.z + (y.z - x.z) * t);
}

// nativeCenterCrossing (NGK:583-622): does the point moving from `start` to `end` cross the segment that moves
// linearly from (pa, pb) to (ca, cb) within the step? The signed area is quadratic in t: both roots are checked,
// with the along-edge test at each; a collinear motion is checked by the minimum of r(t).(r(t) - edge(t)).
__device__ bool center_crossing(float2 start, float2 end, float2 pa, float2 pb, float2 ca, float2 cb) {
    const float2 e0 = sub(pb, pa);
    const float2 de = sub(sub(cb, ca), e0);
    const float2 r0 = sub(start, pa);
    const float2 dr = sub(sub(end, start), sub(ca, pa));
    const float a = cross2(de, dr), b = cross2(e0, dr) + cross2(de, r0);
    const float c = cross2(e0, r0);
    if (a == 0.0f && b == 0.0f && c == 0.0f) {
        const float q0 = dot2(r0, sub(r0, e0));
        if (q0 <= 0.0f) return false;
        const float qa = dot2(dr, sub(dr, de));
        const float qb = dot2(dr, sub(r0, e0)) + dot2(r0, sub(dr, de));
        float minimum = fminf(q0, qa + qb + q0);
        if (qa > 0.0f) {
            const float t = clampf(-qb / (2.0f * qa), 0.0f, 1.0f);
            minimum = fminf(minimum, (qa * t + qb) * t + q0);
        }
        return minimum <= 0.0f;
    }
    float roots[2] = {-1.0f, -1.0f};
    if (fabsf(a) <= kFltEpsilon * fmaxf(fabsf(b), fabsf(c))) {
        if (fabsf(b) > kFltMin) roots[0] = -c / b;
    } else {
        const float d = b * b - 4.0f * a * c;
        if (d > 0.0f) {
            const float q = -0.5f * (b + copysignf(sqrtf(d), b));
            roots[0] = q / a;
            roots[1] = fabsf(q) > kFltMin ? c / q : -1.0f;
        }
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const float t = roots[k];
        if (!(t > 0.0f && t < 1.0f)) continue;
        const float2 edge = add(e0, mul(de, t)), relative = add(r0, mul(dr, t));
        const float square = dot2(edge, edge), along = dot2(relative, edge);
        if (square > kFltMin && along >= 0.0f && along <= square) return true;
    }
    return false;
}

// nativeJointExcluded (NGK:254-258), with the partner list bounded by its array.
__device__ __forceinline__ bool joint_excluded(const uint4* ranges, const unsigned long long* partners,
                                               uint32_t partnerCount, uint32_t entity, unsigned long long partner) {
    if (!ranges) return false;
    const uint4 r = ranges[entity];
    for (uint32_t i = 0; i < r.w; ++i) {
        const uint32_t at = r.z + i;
        if (at >= partnerCount) break;
        if (partners[at] == partner) return true;
    }
    return false;
}

struct SweepInputs {
    const float2* verts;
    const bp_segment* segs;
    uint32_t segmentCount, entity, partnerCount;
    const uint4* jointRanges;
    const unsigned long long* partners;
};

// The wall normal of a sweep hit: the segment's right normal, turned towards the vertex's start side.
__device__ __forceinline__ float2 sweep_normal(float2 a, float2 b, float2 startVertex) {
    const float2 edge = sub(b, a);
    float2 normal = normalized(f2(edge.y, -edge.x));
    if (dot2(sub(startVertex, a), normal) < 0.0f) normal = f2(-normal.x, -normal.y);
    return normal;
}

// nativeRigidSweepCrossing (NPK:30-63): does the body moved from pose p to pose q cross a segment with a vertex, or
// does a segment end cross one of its edges? The first hit gives the contact point, normal and the wall's owner.
__device__ bool sweep_crossing(const RBody& b, float3 p, float3 q, const SweepInputs& in, float2& point,
                               float2& normal, long long& owner) {
    const uint32_t first = b.ranges.x, count = b.ranges.y;
    for (uint32_t j = 0; j < in.segmentCount; ++j) {
        const bp_segment& wall = in.segs[j];
        const bool hasOwner = (wall.flags & BP_SEGMENT_HAS_OWNER) != 0u;
        if ((unsigned long long)wall.owner_id == b.id && hasOwner) continue;
        if (hasOwner && joint_excluded(in.jointRanges, in.partners, in.partnerCount, in.entity,
                                       (unsigned long long)wall.owner_id))
            continue;
        if (!filter_accepts(make_uint2(b.filter.x, b.filter.y), make_uint2(wall.category, wall.mask))) continue;
        const float2 wa = f2(wall.a[0], wall.a[1]), wb = f2(wall.b[0], wall.b[1]);
        for (uint32_t k = 0; k < count; ++k) {
            const float2 v = in.verts[first + k];
            const float2 startVertex = add(f2(p.x, p.y), rotate_by(v, p.z));
            const float2 endVertex = add(f2(q.x, q.y), rotate_by(v, q.z));
            if (center_crossing(startVertex, endVertex, wa, wb, wa, wb)) {
                point = closest_point(endVertex, wa, wb);
                normal = sweep_normal(wa, wb, startVertex);
                owner = wall.owner_id;
                return true;
            }
            // a segment end must not pass through an edge of the body either
            const float2 next = in.verts[first + (k + 1u) % count];
            const float2 ps = add(f2(p.x, p.y), rotate_by(v, p.z)), pe = add(f2(p.x, p.y), rotate_by(next, p.z));
            const float2 qs = add(f2(q.x, q.y), rotate_by(v, q.z)), qe = add(f2(q.x, q.y), rotate_by(next, q.z));
            if (center_crossing(wa, wa, ps, pe, qs, qe) || center_crossing(wb, wb, ps, pe, qs, qe)) {
                point = closest_point(endVertex, wa, wb);
                normal = sweep_normal(wa, wb, startVertex);
                owner = wall.owner_id;
                return true;
            }
        }
    }
    return false;
}

__device__ __forceinline__ bool vertex_range_ok(const RBody& b, uint32_t vertexCount) {
    return b.ranges.y <= vertexCount && b.ranges.x <= vertexCount - b.ranges.y;
}

// nativeRigidPredict (NPK:66-115)
__global__ void __launch_bounds__(kRigidThreads) rigid_predict_kernel(RBody* bodies, uint32_t bodyCount, SweepInputs in,
                                                                    uint32_t vertexCount, uint32_t bubbleCount,
                                                                    float dt, RWall* walls, uint32_t* safety) {
    const uint32_t index = blockIdx.x * blockDim.x + threadIdx.x;
    if (index >= bodyCount) return;
    RBody b = bodies[index];
    b.previous.x = b.pose.x; b.previous.y = b.pose.y; b.pose.w = b.pose.z; b.flags.z = 0u;
    if (b.flags.x) {
        b.motion.x = 0.0f; b.motion.y = 0.0f; b.motion.z = 0.0f;
        bodies[index] = b;
        return;
    }
    b.motion.z *= (float)exp((double)(-b.motion.w * dt));
    const float2 velocity = clamp_linear(f2(b.motion.x, b.motion.y), b.limits.x);
    b.motion.x = velocity.x; b.motion.y = velocity.y;
    b.motion.z = clamp_angular(b.motion.z, b.limits.y);
    const float3 start = make_float3(b.pose.x, b.pose.y, b.pose.z);
    b.pose.x += b.motion.x * dt; b.pose.y += b.motion.y * dt; b.pose.z += b.motion.z * dt;
    if (!finite4(b.pose) || !finite4(b.motion)) {
        atomicOr(safety, BP_RIGID_SAFETY_NONFINITE);
        bodies[index] = b;
        return;
    }
    if (b.filter.z) {  // a kinematic body follows its path: no damping stop, no wall, no neighbour
        bodies[index] = b;
        return;
    }
    if (!vertex_range_ok(b, vertexCount)) {
        atomicOr(safety, BP_RIGID_SAFETY_INVALID);
        bodies[index] = b;
        return;
    }
    // conservative vertex sweep: the rotation is sampled every 0.05 rad, at most 128 samples
    const float samples = ceilf(fabsf(b.pose.z - start.z) / 0.05f);
    const uint32_t steps = samples > 128.0f ? 129u : max(1u, (uint32_t)samples);
    if (steps > 128u) {
        atomicOr(safety, BP_RIGID_SAFETY_ROTATION_BUDGET);
        bodies[index] = b;
        return;
    }
    SweepInputs sweep = in;
    sweep.entity = bubbleCount + index;
    const float3 end = make_float3(b.pose.x, b.pose.y, b.pose.z);
    bool crossed = false;
    float2 contactPoint = f2(0.0f, 0.0f), contactNormal = f2(0.0f, 0.0f);
    long long contactOwner = 0;
    float3 stopPose = start;
    for (uint32_t sample = 0; sample < steps && !crossed; ++sample) {
        const float3 p = mix3(start, end, (float)sample / (float)steps);
        const float3 q = mix3(start, end, (float)(sample + 1u) / (float)steps);
        crossed = sweep_crossing(b, p, q, sweep, contactPoint, contactNormal, contactOwner);
        if (!crossed) continue;
        // stop at the last pose without a crossing (12 bisections between p and q)
        float3 last = p, hit = q;
        for (uint32_t bisection = 0; bisection < 12u; ++bisection) {
            const float3 middle = make_float3(0.5f * (last.x + hit.x), 0.5f * (last.y + hit.y), 0.5f * (last.z + hit.z));
            float2 pointTmp, normalTmp;
            long long ownerTmp;
            if (sweep_crossing(b, p, middle, sweep, pointTmp, normalTmp, ownerTmp)) hit = middle;
            else last = middle;
        }
        stopPose = last;
    }
    if (crossed) {
        const float closing = fmaxf(0.0f, -dot2(f2(b.motion.x, b.motion.y), contactNormal));
        const float stopped = b.physical.x > 0.0f ? closing / b.physical.x * dt : 0.0f;
        b.pose.x = stopPose.x; b.pose.y = stopPose.y; b.pose.z = stopPose.z;
        b.motion.x = 0.0f; b.motion.y = 0.0f; b.motion.z = 0.0f;
        for (uint32_t j = 0; j < bodyCount; ++j) {
            if (j != index && bodies[j].flags.x && bodies[j].id == (unsigned long long)contactOwner) {
                RWall w;
                w.body = (long long)b.id; w.owner = contactOwner;
                w.geometry = make_float4(contactNormal.x, contactNormal.y, contactPoint.x, contactPoint.y);
                w.extra = make_float4(stopped, 0.0f, 0.0f, 0.0f);
                walls[index] = w;
                break;
            }
        }
    }
    bodies[index] = b;
}

// nativeRigidFinish (NPK:172-198)
__global__ void __launch_bounds__(kRigidThreads) rigid_finish_kernel(RBody* bodies, uint32_t bodyCount,
                                                                   const float2* verts, uint32_t vertexCount,
                                                                   float4 region, uint32_t* safety) {
    const uint32_t index = blockIdx.x * blockDim.x + threadIdx.x;
    if (index >= bodyCount) return;
    RBody b = bodies[index];
    if (!finite4(b.pose) || !finite4(b.previous) || !finite4(b.motion)) {
        atomicOr(safety, BP_RIGID_SAFETY_NONFINITE);
        return;
    }
    if (b.flags.x) return;
    const float2 velocity = clamp_linear(f2(b.motion.x, b.motion.y), b.limits.x);
    b.motion.x = velocity.x; b.motion.y = velocity.y;
    b.motion.z = clamp_angular(b.motion.z, b.limits.y);
    if (!vertex_range_ok(b, vertexCount)) {
        atomicOr(safety, BP_RIGID_SAFETY_INVALID);
        return;
    }
    float2 low = f2(INFINITY, INFINITY), high = f2(-INFINITY, -INFINITY);
    for (uint32_t i = 0; i < b.ranges.y; ++i) {
        const float2 v = add(f2(b.pose.x, b.pose.y), rotate_by(verts[b.ranges.x + i], b.pose.z));
        low = vmin2(low, v);
        high = vmax2(high, v);
    }
    // the core of a circle or capsule grows by its radius (0 for a polygon)
    low = f2(low.x - b.shape.y, low.y - b.shape.y);
    high = f2(high.x + b.shape.y, high.y + b.shape.y);
    float2 shift = f2(0.0f, 0.0f);
    const float2 size = f2(region.z - region.x, region.w - region.y);
    const bool outside = high.x < region.x || high.y < region.y || low.x > region.z || low.y > region.w;
    if (outside) {
        if (!b.flags.y) {
            b.flags.z = 1u;
        } else {
            if (high.x < region.x) shift.x = ceilf((region.x - high.x) / size.x) * size.x;
            if (low.x > region.z) shift.x = -ceilf((low.x - region.z) / size.x) * size.x;
            if (high.y < region.y) shift.y = ceilf((region.y - high.y) / size.y) * size.y;
            if (low.y > region.w) shift.y = -ceilf((low.y - region.w) / size.y) * size.y;
            b.pose.x += shift.x; b.pose.y += shift.y;
            b.previous.x += shift.x; b.previous.y += shift.y;
            b.flags.z = 2u;
        }
    }
    bodies[index] = b;
}

// nativeJointEnd (NativeContactKernels.metal-source = NCK:451-464): an end is a world point or a body's anchor,
// measured from the centre of mass (the anchor frame starts at the geometry origin, previous.zw the centroid).
struct JointEnd {
    float2 point, arm, velocity;
    float inverseMass, inverseInertia, angle, omega;
};

__device__ __forceinline__ bool joint_end(uint32_t entity, float2 anchor, const RBody* bodies, uint32_t bodyCount,
                                          uint32_t bubbleCount, const float2* trig, JointEnd& e) {
    e.point = anchor; e.arm = f2(0.0f, 0.0f); e.velocity = f2(0.0f, 0.0f);
    e.inverseMass = 0.0f; e.inverseInertia = 0.0f; e.angle = 0.0f; e.omega = 0.0f;
    if (entity == BP_JOINT_WORLD_END) return true;
    if (entity < bubbleCount || entity - bubbleCount >= bodyCount) return false;
    const uint32_t at = entity - bubbleCount;
    const RBody& b = bodies[at];
    const float4 pose = b.pose, previous = b.previous, motion = b.motion, physical = b.physical;
    const float2 cs = trig ? trig[at] : sincos_cw(pose.z);  // (cos, sin) of pose.z, cached per round when it fits
    e.arm = rot_cs(sub(anchor, f2(previous.z, previous.w)), cs.x, cs.y);
    e.point = add(f2(pose.x, pose.y), e.arm);
    e.velocity = f2(motion.x, motion.y);
    e.omega = motion.z;
    e.angle = pose.z;
    e.inverseMass = physical.x;
    e.inverseInertia = physical.y;
    return true;
}

__device__ __forceinline__ float2 perpendicular(float2 v) { return f2(-v.y, v.x); }

// nativeSolveJoints (NCK:468-543): both ends' corrections of one joint from the current state.
__device__ __forceinline__ float damping_decay(const RJoint& joint, float dt, uint32_t iterationCount) {
    return (float)exp((double)(-joint.parameters.z * dt / (float)max(iterationCount, 1u)));
}

__device__ void solve_joint(RJoint& joint, RCorrection& out, const RBody* bodies, uint32_t bodyCount,
                            uint32_t bubbleCount, float dt, uint32_t iterationCount, const float2* trig,
                            const float* decays, uint32_t j, uint32_t* safety) {
    JointEnd a, b;
    const bool okA =
        joint_end(joint.ends.x, f2(joint.anchors.x, joint.anchors.y), bodies, bodyCount, bubbleCount, trig, a);
    const bool okB =
        joint_end(joint.ends.y, f2(joint.anchors.z, joint.anchors.w), bodies, bodyCount, bubbleCount, trig, b);
    float2 moveA = f2(0.0f, 0.0f), moveB = f2(0.0f, 0.0f), speedA = f2(0.0f, 0.0f), speedB = f2(0.0f, 0.0f);
    float turnA = 0.0f, turnB = 0.0f, spinA = 0.0f, spinB = 0.0f;
    if (!okA || !okB) {
        atomicOr(safety, BP_RIGID_SAFETY_INVALID);
        out.first = out.second = out.velocityFirst = out.velocitySecond = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return;
    }
    const float2 pointA = perpendicular(a.arm), pointB = perpendicular(b.arm);
    const uint32_t kind = joint.ends.z;
    if (kind == 0u) {
        const float2 delta = sub(b.point, a.point);
        const float length = len2(delta);
        const float2 n = length > 1e-6f ? dvd(delta, length) : f2(1.0f, 0.0f);
        const float ca = cross2(a.arm, n), cb = cross2(b.arm, n);
        const float w = a.inverseMass + b.inverseMass + a.inverseInertia * ca * ca + b.inverseInertia * cb * cb;
        if (w > kFltMin) {
            // XPBD: compliance / dt^2, lambda accumulated over the step (compliance 0 = rigid distance)
            const float alpha = joint.parameters.y / (dt * dt);
            const float lambda = (-(length - joint.parameters.x) - alpha * joint.state.x) / (w + alpha);
            joint.state.x += lambda;
            moveA = mul(mul(f2(-n.x, -n.y), a.inverseMass), lambda);
            turnA = -ca * a.inverseInertia * lambda;
            moveB = mul(mul(n, b.inverseMass), lambda);
            turnB = cb * b.inverseInertia * lambda;
            if (joint.parameters.z > 0.0f) {
                // damping of the relative velocity along the joint, spread over the iterations (exp(-d dt) a step)
                const float2 va = add(a.velocity, mul(pointA, a.omega)), vb = add(b.velocity, mul(pointB, b.omega));
                const float relative = dot2(sub(vb, va), n);
                const float decay = decays ? decays[j] : damping_decay(joint, dt, iterationCount);
                const float impulse = -relative * (1.0f - decay) / w;
                speedA = sub(speedA, mul(mul(n, a.inverseMass), impulse));
                spinA -= ca * a.inverseInertia * impulse;
                speedB = add(speedB, mul(mul(n, b.inverseMass), impulse));
                spinB += cb * b.inverseInertia * impulse;
            }
        }
    } else {
        // hinge and weld: the two ends meet in a point (2x2 effective mass block)
        const float weight = a.inverseMass + b.inverseMass;
        const float k11 = weight + a.inverseInertia * pointA.x * pointA.x + b.inverseInertia * pointB.x * pointB.x;
        const float k12 = a.inverseInertia * pointA.x * pointA.y + b.inverseInertia * pointB.x * pointB.y;
        const float k22 = weight + a.inverseInertia * pointA.y * pointA.y + b.inverseInertia * pointB.y * pointB.y;
        const float determinant = k11 * k22 - k12 * k12;
        if (determinant > kFltMin) {
            const float2 gap = sub(b.point, a.point);
            const float2 impulse = dvd(f2(-(k22 * gap.x - k12 * gap.y), -(-k12 * gap.x + k11 * gap.y)), determinant);
            moveA = mul(f2(-impulse.x, -impulse.y), a.inverseMass);
            turnA = -a.inverseInertia * dot2(pointA, impulse);
            moveB = mul(impulse, b.inverseMass);
            turnB = b.inverseInertia * dot2(pointB, impulse);
        }
        const float inertia = a.inverseInertia + b.inverseInertia;
        if (inertia > kFltMin) {
            // relative angle after the point correction: turn of B - turn of A - reference angle
            const float angle = (b.angle + turnB) - (a.angle + turnA) - joint.parameters.w;
            float violation = 0.0f;
            if (kind == 2u) violation = angle;
            else if (joint.ends.w & 1u)
                violation = angle < joint.limits.x ? angle - joint.limits.x
                                                   : (angle > joint.limits.y ? angle - joint.limits.y : 0.0f);
            if (violation != 0.0f) {
                const float lambda = -violation / inertia;
                turnA -= a.inverseInertia * lambda;
                turnB += b.inverseInertia * lambda;
            }
            if (kind == 1u && (joint.ends.w & 2u)) {
                // motor: towards the target relative angular velocity, total impulse of the step within torque x dt
                const float relative = (b.omega + turnB / dt) - (a.omega + turnA / dt) - joint.limits.z;
                const float limit = joint.limits.w * dt;
                const float total = clampf(joint.state.y - relative / inertia, -limit, limit);
                const float lambda = total - joint.state.y;
                joint.state.y = total;
                spinA -= a.inverseInertia * lambda;
                spinB += b.inverseInertia * lambda;
            }
        }
    }
    out.first = make_float4(moveA.x, moveA.y, turnA, 0.0f);
    out.second = make_float4(moveB.x, moveB.y, turnB, 0.0f);
    out.velocityFirst = make_float4(moveA.x / dt + speedA.x, moveA.y / dt + speedA.y, turnA / dt + spinA, 0.0f);
    out.velocitySecond = make_float4(moveB.x / dt + speedB.x, moveB.y / dt + speedB.y, turnB / dt + spinB, 0.0f);
}

// nativeApplyJointBodies (NCK:546-562) for body i: the body adds its joints' corrections in list order and averages
// them (Jacobi without overshoot); `trig`, when given, gets the (cos, sin) of the body's new angle.
__device__ __forceinline__ void apply_joint_corrections(uint32_t i, RBody* bodies, const RCorrection* corrections,
                                                        const uint2* references, uint32_t referenceCount,
                                                        uint32_t jointCount, const uint4* jointRanges,
                                                        uint32_t bubbleCount, float2* trig, uint32_t* safety) {
    const uint4 range = jointRanges[bubbleCount + i];
    if (range.y == 0u) return;
    float3 delta = make_float3(0.0f, 0.0f, 0.0f), velocity = make_float3(0.0f, 0.0f, 0.0f);
    for (uint32_t r = 0; r < range.y; ++r) {
        const uint32_t at = range.x + r;
        if (at >= referenceCount || references[at].x >= jointCount) {
            atomicOr(safety, BP_RIGID_SAFETY_INVALID);
            return;
        }
        const uint2 ref = references[at];
        const RCorrection& c = corrections[ref.x];
        const float4 d = ref.y ? c.second : c.first, v = ref.y ? c.velocitySecond : c.velocityFirst;
        delta.x += d.x; delta.y += d.y; delta.z += d.z;
        velocity.x += v.x; velocity.y += v.y; velocity.z += v.z;
    }
    const float relax = 1.0f / (float)range.y;
    float4 pose = bodies[i].pose, motion = bodies[i].motion;
    pose.x += delta.x * relax; pose.y += delta.y * relax; pose.z += delta.z * relax;
    motion.x += velocity.x * relax; motion.y += velocity.y * relax; motion.z += velocity.z * relax;
    bodies[i].pose = pose;
    bodies[i].motion = motion;
    if (trig) trig[i] = sincos_cw(pose.z);
}

// Small worlds: all `iterations` rounds of nativeSolveJoints + nativeApplyJointBodies (NCK:468-562) in one block,
// the two halves of a round separated by __syncthreads(). The dynamic shared memory holds (cos, sin) of every body's
// angle (refreshed by the body's own thread after its apply) and every joint's damping factor (constant over the
// launch): one rotation per body and round instead of two per joint, one exp per joint and launch.
__global__ void __launch_bounds__(kJointThreads) rigid_joints_kernel(RBody* bodies, uint32_t bodyCount, RJoint* joints,
                                                                   uint32_t jointCount, RCorrection* corrections,
                                                                   const uint2* references, uint32_t referenceCount,
                                                                   const uint4* jointRanges, uint32_t bubbleCount,
                                                                   float dt, uint32_t iterationCount,
                                                                   uint32_t iterations, uint32_t* safety) {
    extern __shared__ float2 g_rigid_cache[];
    float2* trig = g_rigid_cache;
    float* decays = reinterpret_cast<float*>(g_rigid_cache + bodyCount);
    for (uint32_t i = threadIdx.x; i < bodyCount; i += blockDim.x) trig[i] = sincos_cw(bodies[i].pose.z);
    for (uint32_t j = threadIdx.x; j < jointCount; j += blockDim.x) decays[j] = damping_decay(joints[j], dt, iterationCount);
    __syncthreads();
    for (uint32_t round = 0; round < iterations; ++round) {
        for (uint32_t j = threadIdx.x; j < jointCount; j += blockDim.x) {
            RJoint joint = joints[j];
            RCorrection c;
            solve_joint(joint, c, bodies, bodyCount, bubbleCount, dt, iterationCount, trig, decays, j, safety);
            corrections[j] = c;
            joints[j] = joint;
        }
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < bodyCount; i += blockDim.x)
            apply_joint_corrections(i, bodies, corrections, references, referenceCount, jointCount, jointRanges,
                                    bubbleCount, trig, safety);
        __syncthreads();
    }
}

// Larger worlds: one round is two grid launches, a thread per joint, then a thread per body (the launch boundary is
// the round's barrier), so every SM works on it; rotations and damping factors are computed in place (same bits).
__global__ void __launch_bounds__(kRoundThreads) rigid_joint_round_kernel(RBody* bodies, uint32_t bodyCount,
                                                                        RJoint* joints, uint32_t jointCount,
                                                                        RCorrection* corrections, uint32_t bubbleCount,
                                                                        float dt, uint32_t iterationCount,
                                                                        uint32_t* safety) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= jointCount) return;
    RJoint joint = joints[j];
    RCorrection c;
    solve_joint(joint, c, bodies, bodyCount, bubbleCount, dt, iterationCount, nullptr, nullptr, j, safety);
    corrections[j] = c;
    joints[j] = joint;
}

__global__ void __launch_bounds__(kRoundThreads) rigid_apply_round_kernel(RBody* bodies, uint32_t bodyCount,
                                                                        const RCorrection* corrections,
                                                                        const uint2* references,
                                                                        uint32_t referenceCount, uint32_t jointCount,
                                                                        const uint4* jointRanges, uint32_t bubbleCount,
                                                                        uint32_t* safety) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= bodyCount) return;
    apply_joint_corrections(i, bodies, corrections, references, referenceCount, jointCount, jointRanges, bubbleCount,
                            nullptr, safety);
}

// ---- body contacts, body-pair rows, CCD, wall guard ----------------------------------------------------------

struct __align__(16) RCandidate {
    long long first, second;  // participants
    uint4 meta;               // kind, lower index, higher index, float bits of the summed normal lambda
};
static_assert(sizeof(RCandidate) == sizeof(bp_rigid_candidate), "bp_rigid_candidate layout");

struct Geo {
    const float2* verts;
    uint32_t vertexCount;
    const uint4* tris;
    uint32_t triangleCount;
};

__device__ __forceinline__ bool is_round(const RBody& b) { return b.shape.x > 0.5f; }
__device__ __forceinline__ bool immovable(const RBody& b) { return b.flags.x != 0u || b.filter.z != 0u; }
__device__ __forceinline__ bool accepts(const RBody& a, const RBody& b) {
    return filter_accepts(make_uint2(a.filter.x, a.filter.y), make_uint2(b.filter.x, b.filter.y));
}
__device__ __forceinline__ float dist2(float2 a, float2 b) { return len2(sub(a, b)); }
__device__ __forceinline__ float2 neg2(float2 a) { return f2(-a.x, -a.y); }
__device__ __forceinline__ float2 pose_xy(const RBody& b) { return f2(b.pose.x, b.pose.y); }

// nativeRigidVertex (NGK:139-141)
__device__ __forceinline__ float2 world_vertex(const Geo& g, const RBody& b, uint32_t i) {
    return add(pose_xy(b), rotate_by(g.verts[b.ranges.x + i], b.pose.z));
}

// A body's vertex and triangle ranges lie inside the arrays and its triangles index its own vertices.
__device__ bool geometry_ok(const Geo& g, const RBody& b) {
    if (!vertex_range_ok(b, g.vertexCount)) return false;
    if (b.ranges.w > g.triangleCount || b.ranges.z > g.triangleCount - b.ranges.w) return false;
    for (uint32_t i = 0; i < b.ranges.w; ++i) {
        const uint4 t = g.tris[b.ranges.z + i];
        if (t.x >= b.ranges.y || t.y >= b.ranges.y || t.z >= b.ranges.y) return false;
    }
    return is_round(b) ? b.ranges.y >= 1u : true;
}

// nativeSegmentDistance (NGK:444-462)
__device__ float segment_distance(float2 a, float2 b, float2 c, float2 d, float2& pa, float2& pb) {
    const float2 r = sub(b, a), s = sub(d, c);
    const float denominator = cross2(r, s);
    if (fabsf(denominator) > 1e-12f) {
        const float2 qp = sub(c, a);
        const float t = cross2(qp, s) / denominator, u = cross2(qp, r) / denominator;
        if (t >= 0.0f && t <= 1.0f && u >= 0.0f && u <= 1.0f) { pa = add(a, mul(r, t)); pb = pa; return 0.0f; }
    }
    float best = INFINITY;
    float2 cp = closest_point(a, c, d);
    float value = dist2(a, cp);
    if (value < best) { best = value; pa = a; pb = cp; }
    cp = closest_point(b, c, d); value = dist2(b, cp);
    if (value < best) { best = value; pa = b; pb = cp; }
    cp = closest_point(c, a, b); value = dist2(c, cp);
    if (value < best) { best = value; pa = cp; pb = c; }
    cp = closest_point(d, a, b); value = dist2(d, cp);
    if (value < best) { best = value; pa = cp; pb = d; }
    return best;
}

struct Core { float2 a, b; float radius; };
// nativeRoundCoreOf (NGK:466-472)
__device__ __forceinline__ Core core_of(const Geo& g, const RBody& b) {
    Core c;
    c.a = world_vertex(g, b, 0);
    c.b = b.ranges.y > 1u ? world_vertex(g, b, 1) : c.a;
    c.radius = b.shape.y;
    return c;
}

// nativeRigidInside (NGK:477-490)
__device__ bool rigid_inside_body(const Geo& g, float2 p, const RBody& b) {
    if (is_round(b)) {
        const Core c = core_of(g, b);
        return dist2(p, closest_point(p, c.a, c.b)) <= c.radius;
    }
    const float2 local = rotate_by(sub(p, pose_xy(b)), -b.pose.z);
    for (uint32_t i = 0; i < b.ranges.w; ++i) {
        const uint4 t = g.tris[b.ranges.z + i];
        const float2 A = g.verts[b.ranges.x + t.x], B = g.verts[b.ranges.x + t.y], C = g.verts[b.ranges.x + t.z];
        if (cross2(sub(B, A), sub(local, A)) >= 0.0f && cross2(sub(C, B), sub(local, B)) >= 0.0f &&
            cross2(sub(A, C), sub(local, C)) >= 0.0f)
            return true;
    }
    return false;
}

// nativeRoundContact (NGK:546-581)
__device__ bool round_contact(const Core& A, const Core& B, float2 fallback, float2& normal, float& depth,
                              float2& point) {
    float2 pa, pb;
    const float separation = segment_distance(A.a, A.b, B.a, B.b, pa, pb);
    if (separation > 1e-4f) {
        normal = dvd(sub(pb, pa), separation);
        depth = A.radius + B.radius - separation;
        point = mul(add(add(pa, mul(normal, A.radius)), sub(pb, mul(normal, B.radius))), 0.5f);
        return true;
    }
    float2 axes[2];
    uint32_t axisCount = 0;
    const float2 ea = sub(A.b, A.a), eb = sub(B.b, B.a);
    const float la = len2(ea), lb = len2(eb);
    if (la > 1e-6f) axes[axisCount++] = dvd(f2(-ea.y, ea.x), la);
    if (lb > 1e-6f) axes[axisCount++] = dvd(f2(-eb.y, eb.x), lb);
    float2 axis = fallback;
    float overlap = 0.0f, orientation = 1.0f, best = INFINITY;
    for (uint32_t i = 0; i < axisCount; ++i) {
        const float2 c = axes[i];
        const float amin = fminf(dot2(A.a, c), dot2(A.b, c)), amax = fmaxf(dot2(A.a, c), dot2(A.b, c));
        const float bmin = fminf(dot2(B.a, c), dot2(B.b, c)), bmax = fmaxf(dot2(B.a, c), dot2(B.b, c));
        const float plus = amax - bmin, minus = bmax - amin;
        const float value = fminf(plus, minus);
        if (value < best) {
            best = value; axis = c; overlap = value;
            if (fabsf(plus - minus) < 1e-6f) orientation = dot2(c, fallback) >= 0.0f ? 1.0f : -1.0f;
            else orientation = plus < minus ? 1.0f : -1.0f;
        }
    }
    normal = mul(axis, orientation);
    depth = overlap + A.radius + B.radius;
    point = mul(add(pa, pb), 0.5f);
    return true;
}

// nativeTriangleContact (NCK:248-275)
__device__ bool triangle_contact(const float2* a, const float2* b, float2& normal, float& depth, float2& point) {
    depth = INFINITY;
    for (int shape = 0; shape < 2; ++shape)
        for (int edge = 0; edge < 3; ++edge) {
            const float2 delta = shape == 0 ? sub(a[(edge + 1) % 3], a[edge]) : sub(b[(edge + 1) % 3], b[edge]);
            const float magnitude = len2(delta);
            if (magnitude <= kFltMin) return false;
            const float2 axis = dvd(f2(-delta.y, delta.x), magnitude);
            float amin = INFINITY, amax = -INFINITY, bmin = INFINITY, bmax = -INFINITY;
            for (int k = 0; k < 3; ++k) {
                const float pa = dot2(a[k], axis), pb = dot2(b[k], axis);
                amin = fminf(amin, pa); amax = fmaxf(amax, pa);
                bmin = fminf(bmin, pb); bmax = fmaxf(bmax, pb);
            }
            if (amax < bmin || bmax < amin) return false;
            const float plus = amax - bmin, minus = bmax - amin;
            const float overlap = fminf(plus, minus);
            if (overlap < depth) { depth = overlap; normal = plus < minus ? axis : neg2(axis); }
        }
    float maxA = -INFINITY, minB = INFINITY;
    float2 pa = f2(0.0f, 0.0f), pb = f2(0.0f, 0.0f);
    uint32_t na = 0, nb = 0;
    for (int k = 0; k < 3; ++k) { maxA = fmaxf(maxA, dot2(a[k], normal)); minB = fminf(minB, dot2(b[k], normal)); }
    for (int k = 0; k < 3; ++k) {
        if (dot2(a[k], normal) >= maxA - 1e-5f) { pa = add(pa, a[k]); ++na; }
        if (dot2(b[k], normal) <= minB + 1e-5f) { pb = add(pb, b[k]); ++nb; }
    }
    point = mul(add(dvd(pa, (float)na), dvd(pb, (float)nb)), 0.5f);
    return true;
}

__device__ __forceinline__ float2 outward_of(float2 p, float2 q) {
    const float2 edge = sub(q, p);
    const float size = len2(edge);
    return size > kFltMin ? dvd(f2(edge.y, -edge.x), size) : f2(0.0f, 1.0f);
}

// nativeRoundPolygonContact (NCK:277-333): normal from the round core R to the polygon P.
__device__ bool round_polygon_contact(const Geo& g, const Core& R, const RBody& P, float2& normal, float& depth,
                                      float2& point) {
    const uint32_t count = P.ranges.y;
    float insideDepth = -1.0f;
    float2 insideOutward = f2(0.0f, 0.0f), insidePoint = f2(0.0f, 0.0f);
    const uint32_t endpoints = (R.b.x != R.a.x || R.b.y != R.a.y) ? 2u : 1u;
    uint32_t insideEndpoints = 0;
    for (uint32_t k = 0; k < endpoints; ++k) {
        const float2 endpoint = k == 0 ? R.a : R.b;
        if (!rigid_inside_body(g, endpoint, P)) continue;
        ++insideEndpoints;
        float nearest = INFINITY;
        float2 nearestPoint = f2(0.0f, 0.0f), nearestOutward = f2(0.0f, 0.0f);
        for (uint32_t e = 0; e < count; ++e) {
            const float2 p = world_vertex(g, P, e), q = world_vertex(g, P, (e + 1u) % count);
            const float2 c = closest_point(endpoint, p, q);
            const float d = dist2(endpoint, c);
            if (d < nearest) { nearest = d; nearestPoint = c; nearestOutward = outward_of(p, q); }
        }
        if (nearest > insideDepth) { insideDepth = nearest; insidePoint = nearestPoint; insideOutward = nearestOutward; }
    }
    if (insideEndpoints == endpoints) {
        normal = neg2(insideOutward); depth = R.radius + insideDepth; point = insidePoint;
        return true;
    }
    float best = INFINITY;
    float2 pc = f2(0.0f, 0.0f), pe = f2(0.0f, 0.0f);
    for (uint32_t e = 0; e < count; ++e) {
        const float2 p = world_vertex(g, P, e), q = world_vertex(g, P, (e + 1u) % count);
        float2 ca, ce;
        const float d = segment_distance(R.a, R.b, p, q, ca, ce);
        if (d < best) { best = d; pc = ca; pe = ce; }
    }
    if (best > 1e-4f) {
        normal = dvd(sub(pe, pc), best); depth = R.radius - best; point = pe;
        return true;
    }
    float minimum = INFINITY;
    float2 minimumOutward = f2(0.0f, 1.0f), minimumPoint = pe;
    for (uint32_t e = 0; e < count; ++e) {
        const float2 p = world_vertex(g, P, e), q = world_vertex(g, P, (e + 1u) % count);
        const float2 edge = sub(q, p);
        const float size = len2(edge);
        if (size <= kFltMin) continue;
        const float2 outward = dvd(f2(edge.y, -edge.x), size);
        const float da = dot2(sub(R.a, p), outward), db = dot2(sub(R.b, p), outward);
        const float d = R.radius - fminf(da, db);
        if (d < minimum) {
            minimum = d; minimumOutward = outward;
            minimumPoint = sub(da <= db ? R.a : R.b, mul(outward, fminf(da, db)));
        }
    }
    normal = neg2(minimumOutward); depth = isfinite(minimum) ? minimum : R.radius; point = minimumPoint;
    return true;
}

// nativeRoundCoreCrossesPolygon (NCK:335-344)
__device__ bool round_core_crosses_polygon(const Geo& g, const Core& R, const RBody& P) {
    if (rigid_inside_body(g, R.a, P) || rigid_inside_body(g, R.b, P)) return true;
    for (uint32_t e = 0; e < P.ranges.y; ++e) {
        const float2 p = world_vertex(g, P, e), q = world_vertex(g, P, (e + 1u) % P.ranges.y);
        float2 ca, ce;
        if (segment_distance(R.a, R.b, p, q, ca, ce) <= 1e-4f) return true;
    }
    return false;
}

// nativeRigidPairContact (NCK:348-373): normal from a to b; false = the shapes do not overlap.
__device__ bool pair_contact(const Geo& g, const RBody& a, const RBody& b, float2& n, float& depth, float2& point) {
    const bool aRound = is_round(a), bRound = is_round(b);
    if (aRound && bRound) return round_contact(core_of(g, a), core_of(g, b), f2(1.0f, 0.0f), n, depth, point);
    if (aRound != bRound) {
        const RBody& round = aRound ? a : b;
        const RBody& polygon = aRound ? b : a;
        float2 normal;
        if (!round_polygon_contact(g, core_of(g, round), polygon, normal, depth, point)) return false;
        n = aRound ? normal : neg2(normal);
        return true;
    }
    bool found = false;
    for (uint32_t i = 0; i < a.ranges.w; ++i)
        for (uint32_t j = 0; j < b.ranges.w; ++j) {
            const uint4 ta = g.tris[a.ranges.z + i], tb = g.tris[b.ranges.z + j];
            const float2 av[3] = {world_vertex(g, a, ta.x), world_vertex(g, a, ta.y), world_vertex(g, a, ta.z)};
            const float2 bv[3] = {world_vertex(g, b, tb.x), world_vertex(g, b, tb.y), world_vertex(g, b, tb.z)};
            float2 normal, p;
            float d;
            if (triangle_contact(av, bv, normal, d, p) && (!found || d > depth)) {
                found = true; depth = d; n = normal; point = p;
            }
        }
    return found;
}

// nativeKeyLess / nativeInsertCandidate (NGK:230-251)
__device__ __forceinline__ bool key_less(const RCandidate& a, const RCandidate& b) {
    if (a.meta.x != b.meta.x) return a.meta.x < b.meta.x;
    if (a.first != b.first) return a.first < b.first;
    return a.second < b.second;
}
__device__ void insert_candidate(RCandidate* row, uint32_t& count, uint32_t& dropped, uint32_t limit,
                                 const RCandidate& value) {
    uint32_t location;
    if (count < limit) location = count++;
    else {
        ++dropped;
        if (!key_less(value, row[limit - 1u])) return;
        location = limit - 1u;
    }
    while (location > 0u && key_less(value, row[location - 1u])) { row[location] = row[location - 1u]; --location; }
    row[location] = value;
}

// nativeEmitBodyCandidates, body pairs (NGK:394-415): one warp per body and row. The lanes test 32 other bodies at
// a time and lane 0 inserts the hits in increasing index order, the order of the reference's one-thread loop.
__global__ void __launch_bounds__(kRoundThreads) rigid_candidates_kernel(const RBody* bodies, uint32_t bodyCount,
                                                                       uint32_t bubbleCount, const uint4* jointRanges,
                                                                       const unsigned long long* partners,
                                                                       uint32_t partnerCount, uint32_t limit,
                                                                       RCandidate* rows, uint2* rowCounts,
                                                                       uint32_t* overflow) {
    const uint32_t index = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if (index >= bodyCount) return;  // whole warps
    RCandidate* row = rows + (size_t)index * limit;
    uint32_t count = 0, dropped = 0;
    for (uint32_t base = 0; base < bodyCount; base += 32u) {
        const uint32_t other = base + lane;
        bool hit = false;
        if (other < bodyCount && other != index) {
            const uint32_t low = min(index, other), high = max(index, other);
            const RBody& a = bodies[low];
            const RBody& c = bodies[high];
            hit = !(immovable(a) && immovable(c)) && accepts(a, c) &&
                  !joint_excluded(jointRanges, partners, partnerCount, bubbleCount + index, bodies[other].id);
            if (hit) {
                const float2 start = sub(f2(a.previous.x, a.previous.y), f2(c.previous.x, c.previous.y));
                const float2 end = sub(pose_xy(a), pose_xy(c));
                const float2 travel = sub(end, start);
                const float travelSquared = dot2(travel, travel);
                const float t =
                    travelSquared > kFltMin ? clampf(-dot2(start, travel) / travelSquared, 0.0f, 1.0f) : 0.0f;
                const float radius = 1.25f * (a.physical.z + c.physical.z);
                const float2 closest = add(start, mul(travel, t));
                hit = dot2(closest, closest) <= radius * radius;
            }
        }
        unsigned int hits = __ballot_sync(0xffffffffu, hit);
        if (lane == 0u) {
            while (hits) {
                const uint32_t o = base + (uint32_t)(__ffs(hits) - 1);
                hits &= hits - 1u;
                const uint32_t low = min(index, o), high = max(index, o);
                RCandidate value;
                value.first = (long long)bodies[low].id; value.second = (long long)bodies[high].id;
                value.meta = make_uint4(3u, low, high, 0u);
                insert_candidate(row, count, dropped, limit, value);
            }
        }
    }
    if (lane == 0u) {
        rowCounts[index] = make_uint2(count, 0u);
        if (dropped) atomicAdd(overflow, dropped);
        atomicMax(overflow + 1, count + dropped);
    }
}

__device__ __forceinline__ bool candidate_ok(const RCandidate& c, uint32_t count) {
    return c.meta.y < count && c.meta.z < count;
}

// nativeRigidOverlapAt / nativeRigidTimeOfImpact (NPK:200-233)
__device__ bool overlap_at(const Geo& g, RBody a, RBody b, float t) {
    a.pose.x = a.previous.x + (a.pose.x - a.previous.x) * t; a.pose.y = a.previous.y + (a.pose.y - a.previous.y) * t;
    a.pose.z = a.pose.w + (a.pose.z - a.pose.w) * t;
    b.pose.x = b.previous.x + (b.pose.x - b.previous.x) * t; b.pose.y = b.previous.y + (b.pose.y - b.previous.y) * t;
    b.pose.z = b.pose.w + (b.pose.z - b.pose.w) * t;
    float2 n, point;
    float depth;
    return pair_contact(g, a, b, n, depth, point) && depth > 1e-3f;
}
__device__ float time_of_impact(const Geo& g, const RBody& a, const RBody& b) {
    const float2 da = sub(pose_xy(a), f2(a.previous.x, a.previous.y));
    const float2 db = sub(pose_xy(b), f2(b.previous.x, b.previous.y));
    const float travel = len2(sub(da, db)) + fabsf(a.pose.z - a.pose.w) * a.physical.z +
                         fabsf(b.pose.z - b.pose.w) * b.physical.z;
    if (!(travel > 0.5f)) return 2.0f;
    if (overlap_at(g, a, b, 0.0f)) return 2.0f;
    const float samples = ceilf(travel / 0.5f);
    const uint32_t steps = samples >= 64.0f ? 64u : max(2u, (uint32_t)samples);
    float last = 0.0f;
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
    return 2.0f;
}

// nativeRigidResolveCCD (NPK:235-250): the earliest impact of the body's row, kept in its own limits.z (1 + t). One
// warp per body, a lane per row slot; the minimum does not depend on the order of the slots.
__global__ void __launch_bounds__(kRoundThreads) rigid_ccd_resolve_kernel(RBody* bodies, uint32_t bodyCount, Geo g,
                                                                        const RCandidate* rows,
                                                                        const uint2* rowCounts, uint32_t width,
                                                                        uint32_t* safety) {
    const uint32_t index = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if (index >= bodyCount) return;  // whole warps
    float earliest = 2.0f;
    if (!immovable(bodies[index])) {
        const uint2 rc = rowCounts[index];
        const uint32_t n = min(rc.x, width);
        for (uint32_t slot = rc.y + lane; slot < n; slot += 32u) {
            const RCandidate c = rows[(size_t)index * width + slot];
            if (c.meta.x != 3u) continue;
            if (!candidate_ok(c, bodyCount)) { atomicOr(safety, BP_RIGID_SAFETY_INVALID); continue; }
            const RBody a = bodies[c.meta.y], b = bodies[c.meta.z];
            if (!geometry_ok(g, a) || !geometry_ok(g, b)) { atomicOr(safety, BP_RIGID_SAFETY_INVALID); continue; }
            earliest = fminf(earliest, time_of_impact(g, a, b));
        }
    }
#pragma unroll
    for (int offset = 16; offset > 0; offset >>= 1) earliest = fminf(earliest, __shfl_xor_sync(0xffffffffu, earliest, offset));
    __syncwarp();
    if (lane == 0u) bodies[index].limits.z = earliest <= 1.0f ? 1.0f + earliest : 0.0f;
}

// nativeRigidApplyCCD (NPK:253-263)
__global__ void __launch_bounds__(kRoundThreads) rigid_ccd_apply_kernel(RBody* bodies, uint32_t bodyCount) {
    const uint32_t index = blockIdx.x * blockDim.x + threadIdx.x;
    if (index >= bodyCount) return;
    float4 pose = bodies[index].pose, limits = bodies[index].limits;
    const float4 previous = bodies[index].previous;
    if (limits.z >= 1.0f) {
        const float t = limits.z - 1.0f;
        pose.x = previous.x + (pose.x - previous.x) * t;
        pose.y = previous.y + (pose.y - previous.y) * t;
        pose.z = pose.w + (pose.z - pose.w) * t;
    }
    limits.z = 0.0f;
    bodies[index].pose = pose;
    bodies[index].limits = limits;
}

// nativeRigidContacts (NCK:375-427): one thread per row slot.
__global__ void __launch_bounds__(kRoundThreads) rigid_contacts_kernel(const RBody* bodies, uint32_t bodyCount, Geo g,
                                                                     RCandidate* rows, const uint2* rowCounts,
                                                                     uint32_t width, RCorrection* corrections,
                                                                     uint32_t* safety) {
    const size_t index = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t owner = (uint32_t)(index / width), slot = (uint32_t)(index % width);
    if (owner >= bodyCount || slot >= min(rowCounts[owner].x, width)) return;
    RCandidate& candidate = rows[index];
    const RCorrection previous = corrections[index];
    RCorrection result;
    result.first = make_float4(0.0f, 0.0f, 0.0f, previous.first.w);
    result.second = make_float4(0.0f, 0.0f, 0.0f, previous.second.w);
    result.velocityFirst = make_float4(0.0f, 0.0f, 0.0f, previous.velocityFirst.w);
    result.velocitySecond = make_float4(0.0f, 0.0f, 0.0f, previous.velocitySecond.w);
    const uint4 meta = candidate.meta;
    if (meta.x != 3u) { corrections[index] = result; return; }
    if (meta.y >= bodyCount || meta.z >= bodyCount) {
        atomicOr(safety, BP_RIGID_SAFETY_INVALID);
        corrections[index] = result;
        return;
    }
    const uint32_t ai = meta.y, bi = meta.z;
    const RBody a = bodies[ai], b = bodies[bi];
    if (ai >= bi || (immovable(a) && immovable(b))) { corrections[index] = result; return; }
    if (!geometry_ok(g, a) || !geometry_ok(g, b)) {
        atomicOr(safety, BP_RIGID_SAFETY_INVALID);
        corrections[index] = result;
        return;
    }
    const float2 end = sub(pose_xy(a), pose_xy(b));
    const float radius = a.physical.z + b.physical.z, radiusSquared = radius * radius;
    if (dot2(end, end) > radiusSquared) { corrections[index] = result; return; }
    float2 n, point;
    float depth;
    if (!pair_contact(g, a, b, n, depth, point)) { corrections[index] = result; return; }
    const float wa = a.physical.x, wb = b.physical.x, ia = a.physical.y, ib = b.physical.y;
    const float2 ra = sub(point, pose_xy(a)), rb = sub(point, pose_xy(b));
    const float2 va = f2(a.motion.x, a.motion.y), vb = f2(b.motion.x, b.motion.y);
    const float spinA = a.motion.z, spinB = b.motion.z;
    const float frictionA = a.physical.w, frictionB = b.physical.w;
    const float restitutionA = __uint_as_float(a.flags.w), restitutionB = __uint_as_float(b.flags.w);
    const float ca = cross2(ra, n), cb = cross2(rb, n), denom = wa + wb + ia * ca * ca + ib * cb * cb;
    if (depth < -0.001f || denom <= kFltMin) { corrections[index] = result; return; }
    const float lambda = fmaxf(0.0f, depth) / denom * 0.5f;
    candidate.meta.w = __float_as_uint(__uint_as_float(meta.w) + lambda);
    const float2 moveA = mul(mul(neg2(n), wa), lambda), moveB = mul(mul(n, wb), lambda);
    result.first = make_float4(moveA.x, moveA.y, -ca * ia * lambda, n.x);
    result.second = make_float4(moveB.x, moveB.y, cb * ib * lambda, n.y);
    const float closing = dot2(sub(vb, va), n) + spinB * cb - spinA * ca;
    const float friction = sqrtf(fmaxf(0.0f, frictionA * frictionB));
    const float restitution = fmaxf(restitutionA, restitutionB);
    const float impulse = fmaxf(0.0f, -closing) * (1.0f + restitution) / denom * 0.5f;
    const float2 tangent = f2(-n.y, n.x);
    const float tangentSpeed = dot2(sub(vb, va), tangent) + spinB * cross2(rb, tangent) - spinA * cross2(ra, tangent);
    const float tangentImpulse = -tangentSpeed * friction / denom * 0.5f;
    const float2 vA = sub(mul(mul(neg2(n), wa), impulse), mul(mul(tangent, wa), tangentImpulse));
    const float2 vB = add(mul(mul(n, wb), impulse), mul(mul(tangent, wb), tangentImpulse));
    result.velocityFirst = make_float4(vA.x, vA.y, -ca * ia * impulse - cross2(ra, tangent) * ia * tangentImpulse,
                                       point.x);
    result.velocitySecond = make_float4(vB.x, vB.y, cb * ib * impulse + cross2(rb, tangent) * ib * tangentImpulse,
                                        point.y);
    corrections[index] = result;
}

// nativeRigidApplyBodies (NCK:429-444)
__global__ void __launch_bounds__(kRoundThreads) rigid_apply_bodies_kernel(RBody* bodies, uint32_t bodyCount,
                                                                         const RCandidate* rows,
                                                                         const uint2* rowCounts, uint32_t width,
                                                                         const RCorrection* corrections) {
    const uint32_t index = blockIdx.x * blockDim.x + threadIdx.x;
    if (index >= bodyCount) return;
    float3 delta = make_float3(0.0f, 0.0f, 0.0f), velocity = make_float3(0.0f, 0.0f, 0.0f);
    const uint32_t n = min(rowCounts[index].x, width);
    for (uint32_t slot = 0; slot < n; ++slot) {
        const size_t at = (size_t)index * width + slot;
        const uint4 meta = rows[at].meta;
        const bool first = meta.x == 3u && meta.y == index;
        const RCorrection& c = corrections[at];
        const float4 d = first ? c.first : c.second, v = first ? c.velocityFirst : c.velocitySecond;
        delta.x += d.x; delta.y += d.y; delta.z += d.z;
        velocity.x += v.x; velocity.y += v.y; velocity.z += v.z;
    }
    float4 pose = bodies[index].pose, motion = bodies[index].motion;
    pose.x += delta.x; pose.y += delta.y; pose.z += delta.z;
    motion.x += velocity.x; motion.y += velocity.y; motion.z += velocity.z;
    bodies[index].pose = pose;
    bodies[index].motion = motion;
}

// nativeRigidGuardWalls (NPK:118-170): one warp per dynamic body; static bodies are never written. The walls, the
// vertices of the body and their corrections stay in the reference's order (a correction moves the body before its
// next vertex); within one vertex the lanes split the wall's triangles and edges: "inside" is an OR over triangles,
// the start-on-the-boundary test an OR over edges, and the nearest edge the smallest (distance, edge index) pair,
// which is the edge the reference's strict "<" loop keeps. Every lane keeps the same copy of the body.
__global__ void __launch_bounds__(kRoundThreads) rigid_guard_kernel(RBody* bodies, uint32_t bodyCount, Geo g,
                                                                  uint32_t bubbleCount, const uint4* jointRanges,
                                                                  const unsigned long long* partners,
                                                                  uint32_t partnerCount, uint32_t* safety) {
    const uint32_t index = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if (index >= bodyCount) return;  // whole warps
    if (bodies[index].flags.x || bodies[index].filter.z) return;
    RBody b = bodies[index];
    if (!geometry_ok(g, b)) {
        if (lane == 0u) atomicOr(safety, BP_RIGID_SAFETY_INVALID);
        return;
    }
    // the guard moves a body without turning it: one (cos, sin) of its end angle and one of its start angle serve
    // every vertex; each wall's pose is fixed, so one pair per wall serves all its vertices (the same bits as
    // rotating each vertex by its angle)
    const float2 bodyCS = sincos_cw(b.pose.z), startCS = sincos_cw(b.pose.w);
    for (uint32_t base = 0; base < bodyCount; base += 32u) {
        // the lanes find this chunk's walls; they are then visited in index order
        const uint32_t candidate = base + lane;
        bool isWall = false;
        if (candidate < bodyCount && bodies[candidate].flags.x) {
            const RBody& w = bodies[candidate];
            isWall = !is_round(w) && accepts(b, w) &&
                     !joint_excluded(jointRanges, partners, partnerCount, bubbleCount + index, w.id);
        }
        unsigned int walls = __ballot_sync(0xffffffffu, isWall);
        while (walls) {
            const uint32_t j = base + (uint32_t)(__ffs(walls) - 1);
            walls &= walls - 1u;
            const RBody wall = bodies[j];
            if (!geometry_ok(g, wall)) {
                if (lane == 0u) atomicOr(safety, BP_RIGID_SAFETY_INVALID);
                continue;
            }
            const uint32_t wn = wall.ranges.y, wt = wall.ranges.w;
            const float2 wallCS = sincos_cw(wall.pose.z), wallInverse = sincos_cw(-wall.pose.z);
            const float2 wallAt = pose_xy(wall);
            auto wall_vertex = [&](uint32_t e) {
                return add(wallAt, rot_cs(g.verts[wall.ranges.x + e], wallCS.x, wallCS.y));
            };
            // nativeRigidInside for the polygon wall (NGK:485-490), the triangles split over the lanes
            auto inside_wall = [&](float2 q) {
                const float2 local = rot_cs(sub(q, wallAt), wallInverse.x, wallInverse.y);
                bool in = false;
                for (uint32_t i = lane; i < wt; i += 32u) {
                    const uint4 t = g.tris[wall.ranges.z + i];
                    const float2 A = g.verts[wall.ranges.x + t.x], B = g.verts[wall.ranges.x + t.y];
                    const float2 C = g.verts[wall.ranges.x + t.z];
                    in = in || (cross2(sub(B, A), sub(local, A)) >= 0.0f && cross2(sub(C, B), sub(local, B)) >= 0.0f &&
                                cross2(sub(A, C), sub(local, C)) >= 0.0f);
                }
                return __any_sync(0xffffffffu, in) != 0;
            };
            for (uint32_t k = 0; k < b.ranges.y; ++k) {
                const float2 p = add(pose_xy(b), rot_cs(g.verts[b.ranges.x + k], bodyCS.x, bodyCS.y));
                const float2 start =
                    add(f2(b.previous.x, b.previous.y), rot_cs(g.verts[b.ranges.x + k], startCS.x, startCS.y));
                const bool inside = inside_wall(p);
                bool startedInside = inside_wall(start);
                if (startedInside) {
                    bool onEdge = false;
                    for (uint32_t e = lane; e < wn; e += 32u) {
                        const float2 ea = wall_vertex(e), eb = wall_vertex((e + 1u) % wn);
                        onEdge = onEdge || dist2(start, closest_point(start, ea, eb)) < 1e-5f;
                    }
                    if (__any_sync(0xffffffffu, onEdge)) startedInside = false;
                }
                // each lane's nearest edge among its own (increasing e, strict <), then the warp's smallest pair
                float nearest = INFINITY, depth = 0.0f;
                float2 normal = f2(0.0f, 0.0f);
                uint32_t nearestEdge = 0xffffffffu;
                for (uint32_t e = lane; e < wn; e += 32u) {
                    const float2 ea = wall_vertex(e), eb = wall_vertex((e + 1u) % wn);
                    const float2 direction = sub(eb, ea);
                    const float2 out = normalized(f2(direction.y, -direction.x));
                    const float signedStart = dot2(sub(start, ea), out);
                    const bool onBoundary = dist2(start, closest_point(start, ea, eb)) < 1e-5f;
                    const bool crossing = signedStart >= -1e-5f && (center_crossing(start, p, ea, eb, ea, eb) ||
                                                                     (onBoundary && dot2(sub(p, ea), out) < 0.0f));
                    if (!inside && !crossing) continue;
                    if (inside && !startedInside && signedStart < -1e-5f) continue;
                    const float2 c = closest_point(p, ea, eb);
                    const float d =
                        (crossing || !startedInside) ? dist2(start, closest_point(start, ea, eb)) : dist2(p, c);
                    if (d < nearest) {
                        nearest = d; normal = out; depth = fmaxf(0.0f, -dot2(sub(p, c), out)); nearestEdge = e;
                    }
                }
#pragma unroll
                for (int offset = 16; offset > 0; offset >>= 1) {
                    const float od = __shfl_xor_sync(0xffffffffu, nearest, offset);
                    const uint32_t oe = __shfl_xor_sync(0xffffffffu, nearestEdge, offset);
                    const float onx = __shfl_xor_sync(0xffffffffu, normal.x, offset);
                    const float ony = __shfl_xor_sync(0xffffffffu, normal.y, offset);
                    const float odepth = __shfl_xor_sync(0xffffffffu, depth, offset);
                    if (oe != 0xffffffffu && (nearestEdge == 0xffffffffu || od < nearest || (od == nearest && oe < nearestEdge))) {
                        nearest = od; nearestEdge = oe; normal = f2(onx, ony); depth = odepth;
                    }
                }
                if (nearestEdge == 0xffffffffu) { nearest = INFINITY; depth = 0.0f; }
                if (isfinite(nearest) && depth > 0.0f) {
                    if (is_round(b)) {
                        RBody old = b;
                        old.pose.x = b.previous.x; old.pose.y = b.previous.y; old.pose.z = b.pose.w;
                        if (round_core_crosses_polygon(g, core_of(g, old), wall)) break;
                    }
                    const float2 shift = mul(normal, depth + 1e-5f);
                    b.pose.x += shift.x; b.pose.y += shift.y;
                    const float2 r = sub(p, pose_xy(b));
                    const float lever = cross2(r, normal);
                    const float speed = dot2(f2(b.motion.x, b.motion.y), normal) + b.motion.z * lever;
                    const float denom = b.physical.x + b.physical.y * lever * lever;
                    const float impulse = fmaxf(0.0f, -speed) / fmaxf(denom, kFltMin);
                    const float2 dv = mul(mul(normal, b.physical.x), impulse);
                    b.motion.x += dv.x; b.motion.y += dv.y;
                    b.motion.z += lever * b.physical.y * impulse;
                }
            }
        }
    }
    if (lane == 0u) bodies[index] = b;
}

static bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0u; }
static bool aligned8(const void* p) { return ((uintptr_t)p & 7u) == 0u; }

static int launch_status() { return cudaGetLastError() == cudaSuccess ? BP_OK : BP_E_CUDA; }

}  // namespace bp

extern "C" int bp_rigid_predict(bp_rigid_body* bodies, uint32_t body_count, const float* vertices_xy,
                                uint32_t vertex_count, const bp_segment* segments, uint32_t segment_count,
                                uint32_t bubble_count, float time_step, const uint32_t* joint_ranges,
                                const uint64_t* joint_partners, uint32_t partner_count, bp_rigid_wall* walls,
                                uint32_t* safety, void* stream) {
    using namespace bp;
    if (body_count == 0) return BP_OK;
    if (!bodies || !walls || !safety || (!vertices_xy && vertex_count) || (!segments && segment_count) ||
        (!joint_partners && partner_count))
        return BP_E_INVALID;
    if (!aligned16(bodies) || !aligned16(walls) || !aligned16(joint_ranges) || !aligned16(segments) ||
        !aligned8(vertices_xy) || !aligned8(joint_partners))
        return BP_E_INVALID;
    if (!isfinite(time_step)) return BP_E_INVALID;
    SweepInputs in;
    in.verts = reinterpret_cast<const float2*>(vertices_xy);
    in.segs = segments;
    in.segmentCount = segment_count;
    in.entity = 0;
    in.partnerCount = joint_ranges ? partner_count : 0u;
    in.jointRanges = reinterpret_cast<const uint4*>(joint_ranges);
    in.partners = reinterpret_cast<const unsigned long long*>(joint_partners);
    const uint32_t blocks = (body_count + kRigidThreads - 1u) / kRigidThreads;
    rigid_predict_kernel<<<blocks, kRigidThreads, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<RBody*>(bodies), body_count, in, vertex_count, bubble_count, time_step,
        reinterpret_cast<RWall*>(walls), safety);
    return launch_status();
}

extern "C" int bp_rigid_solve_joints(bp_rigid_body* bodies, uint32_t body_count, bp_rigid_joint* joints,
                                     uint32_t joint_count, bp_rigid_correction* corrections,
                                     const uint32_t* references, uint32_t reference_count,
                                     const uint32_t* joint_ranges, uint32_t bubble_count, float time_step,
                                     uint32_t iteration_count, uint32_t iterations, uint32_t* safety, void* stream) {
    using namespace bp;
    if (joint_count == 0 || iterations == 0) return BP_OK;
    if (!bodies || !joints || !corrections || !joint_ranges || !safety || (!references && reference_count))
        return BP_E_INVALID;
    if (!aligned16(bodies) || !aligned16(joints) || !aligned16(corrections) || !aligned16(joint_ranges) ||
        !aligned8(references))
        return BP_E_INVALID;
    if (!isfinite(time_step)) return BP_E_INVALID;
    const float dt = fmaxf(time_step, 1e-6f);
    RBody* b = reinterpret_cast<RBody*>(bodies);
    RJoint* jn = reinterpret_cast<RJoint*>(joints);
    RCorrection* c = reinterpret_cast<RCorrection*>(corrections);
    const uint2* refs = reinterpret_cast<const uint2*>(references);
    const uint4* ranges = reinterpret_cast<const uint4*>(joint_ranges);
    cudaStream_t s = (cudaStream_t)stream;
    if (joint_count <= kSingleBlockJoints && body_count <= kSingleBlockBodies) {
        const size_t cacheBytes = (size_t)body_count * sizeof(float2) + (size_t)joint_count * sizeof(float);
        rigid_joints_kernel<<<1, kJointThreads, cacheBytes, s>>>(b, body_count, jn, joint_count, c, refs,
                                                                reference_count, ranges, bubble_count, dt,
                                                                iteration_count, iterations, safety);
        return launch_status();
    }
    const uint32_t jointBlocks = (joint_count + kRoundThreads - 1u) / kRoundThreads;
    const uint32_t bodyBlocks = (body_count + kRoundThreads - 1u) / kRoundThreads;
    for (uint32_t round = 0; round < iterations; ++round) {
        rigid_joint_round_kernel<<<jointBlocks, kRoundThreads, 0, s>>>(b, body_count, jn, joint_count, c, bubble_count,
                                                                      dt, iteration_count, safety);
        if (body_count)
            rigid_apply_round_kernel<<<bodyBlocks, kRoundThreads, 0, s>>>(b, body_count, c, refs, reference_count,
                                                                         joint_count, ranges, bubble_count, safety);
        if (cudaPeekAtLastError() != cudaSuccess) break;
    }
    return launch_status();
}

extern "C" int bp_rigid_finish(bp_rigid_body* bodies, uint32_t body_count, const float* vertices_xy,
                               uint32_t vertex_count, const float* region, uint32_t* safety, void* stream) {
    using namespace bp;
    if (body_count == 0) return BP_OK;
    if (!bodies || !region || !safety || (!vertices_xy && vertex_count)) return BP_E_INVALID;
    if (!aligned16(bodies) || !aligned8(vertices_xy)) return BP_E_INVALID;
    const float4 r = make_float4(region[0], region[1], region[2], region[3]);
    const uint32_t blocks = (body_count + kRigidThreads - 1u) / kRigidThreads;
    rigid_finish_kernel<<<blocks, kRigidThreads, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<RBody*>(bodies), body_count, reinterpret_cast<const float2*>(vertices_xy), vertex_count, r,
        safety);
    return launch_status();
}

extern "C" int bp_rigid_body_candidates(const bp_rigid_body* bodies, uint32_t body_count, uint32_t bubble_count,
                                        const uint32_t* joint_ranges, const uint64_t* joint_partners,
                                        uint32_t partner_count, uint32_t row_width, bp_rigid_candidate* rows,
                                        uint32_t* row_counts, uint32_t* overflow, void* stream) {
    using namespace bp;
    if (body_count == 0) return BP_OK;
    if (!bodies || !rows || !row_counts || !overflow || row_width == 0 || (!joint_partners && partner_count))
        return BP_E_INVALID;
    if (!aligned16(bodies) || !aligned16(rows) || !aligned8(row_counts) || !aligned16(joint_ranges) ||
        !aligned8(joint_partners))
        return BP_E_INVALID;
    const uint32_t blocks = (uint32_t)(((size_t)body_count * 32u + kRoundThreads - 1u) / kRoundThreads);
    rigid_candidates_kernel<<<blocks, kRoundThreads, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const RBody*>(bodies), body_count, bubble_count, reinterpret_cast<const uint4*>(joint_ranges),
        reinterpret_cast<const unsigned long long*>(joint_partners), joint_ranges ? partner_count : 0u, row_width,
        reinterpret_cast<RCandidate*>(rows), reinterpret_cast<uint2*>(row_counts), overflow);
    return launch_status();
}

namespace bp {
static bool geometry_args(const float* vertices_xy, uint32_t vertex_count, const uint32_t* triangles,
                          uint32_t triangle_count, Geo& g) {
    if ((!vertices_xy && vertex_count) || (!triangles && triangle_count)) return false;
    if (!aligned8(vertices_xy) || !aligned16(triangles)) return false;
    g.verts = reinterpret_cast<const float2*>(vertices_xy);
    g.vertexCount = vertex_count;
    g.tris = reinterpret_cast<const uint4*>(triangles);
    g.triangleCount = triangle_count;
    return true;
}
}  // namespace bp

extern "C" int bp_rigid_ccd(bp_rigid_body* bodies, uint32_t body_count, const float* vertices_xy, uint32_t vertex_count,
                            const uint32_t* triangles, uint32_t triangle_count, const bp_rigid_candidate* rows,
                            const uint32_t* row_counts, uint32_t row_width, uint32_t* safety, void* stream) {
    using namespace bp;
    if (body_count == 0) return BP_OK;
    Geo g;
    if (!bodies || !rows || !row_counts || !safety || row_width == 0 || !aligned16(bodies) || !aligned16(rows) ||
        !aligned8(row_counts) || !geometry_args(vertices_xy, vertex_count, triangles, triangle_count, g))
        return BP_E_INVALID;
    const uint32_t blocks = (body_count + kRoundThreads - 1u) / kRoundThreads;
    const uint32_t warpBlocks = (uint32_t)(((size_t)body_count * 32u + kRoundThreads - 1u) / kRoundThreads);
    cudaStream_t s = (cudaStream_t)stream;
    RBody* b = reinterpret_cast<RBody*>(bodies);
    rigid_ccd_resolve_kernel<<<warpBlocks, kRoundThreads, 0, s>>>(b, body_count, g,
                                                                  reinterpret_cast<const RCandidate*>(rows),
                                                                  reinterpret_cast<const uint2*>(row_counts),
                                                                  row_width, safety);
    rigid_ccd_apply_kernel<<<blocks, kRoundThreads, 0, s>>>(b, body_count);
    return launch_status();
}

extern "C" int bp_rigid_solve_contacts(bp_rigid_body* bodies, uint32_t body_count, const float* vertices_xy,
                                       uint32_t vertex_count, const uint32_t* triangles, uint32_t triangle_count,
                                       bp_rigid_candidate* rows, const uint32_t* row_counts, uint32_t row_width,
                                       bp_rigid_correction* corrections, uint32_t* safety, void* stream) {
    using namespace bp;
    if (body_count == 0) return BP_OK;
    Geo g;
    if (!bodies || !rows || !row_counts || !corrections || !safety || row_width == 0 || !aligned16(bodies) ||
        !aligned16(rows) || !aligned8(row_counts) || !aligned16(corrections) ||
        !geometry_args(vertices_xy, vertex_count, triangles, triangle_count, g))
        return BP_E_INVALID;
    const size_t slots = (size_t)body_count * row_width;
    if (slots > 0x7fffffffull) return BP_E_CAPACITY;
    cudaStream_t s = (cudaStream_t)stream;
    RBody* b = reinterpret_cast<RBody*>(bodies);
    RCandidate* r = reinterpret_cast<RCandidate*>(rows);
    const uint2* rc = reinterpret_cast<const uint2*>(row_counts);
    RCorrection* c = reinterpret_cast<RCorrection*>(corrections);
    rigid_contacts_kernel<<<(uint32_t)((slots + kRoundThreads - 1u) / kRoundThreads), kRoundThreads, 0, s>>>(
        b, body_count, g, r, rc, row_width, c, safety);
    rigid_apply_bodies_kernel<<<(body_count + kRoundThreads - 1u) / kRoundThreads, kRoundThreads, 0, s>>>(
        b, body_count, r, rc, row_width, c);
    return launch_status();
}

extern "C" int bp_rigid_guard_walls(bp_rigid_body* bodies, uint32_t body_count, const float* vertices_xy,
                                    uint32_t vertex_count, const uint32_t* triangles, uint32_t triangle_count,
                                    uint32_t bubble_count, const uint32_t* joint_ranges,
                                    const uint64_t* joint_partners, uint32_t partner_count, uint32_t* safety,
                                    void* stream) {
    using namespace bp;
    if (body_count == 0) return BP_OK;
    Geo g;
    if (!bodies || !safety || (!joint_partners && partner_count) || !aligned16(bodies) || !aligned16(joint_ranges) ||
        !aligned8(joint_partners) || !geometry_args(vertices_xy, vertex_count, triangles, triangle_count, g))
        return BP_E_INVALID;
    const uint32_t warpBlocks = (uint32_t)(((size_t)body_count * 32u + kRoundThreads - 1u) / kRoundThreads);
    rigid_guard_kernel<<<warpBlocks, kRoundThreads, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<RBody*>(bodies), body_count, g, bubble_count, reinterpret_cast<const uint4*>(joint_ranges),
        reinterpret_cast<const unsigned long long*>(joint_partners), joint_ranges ? partner_count : 0u, safety);
    return launch_status();
}
