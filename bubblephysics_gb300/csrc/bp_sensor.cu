// bp_sensor.cu - sensor enter / exit events of a world's bubbles and bodies after each step.
//
// The reference compares every (sensor, object) pair on the GPU after the step, bubbles in nativeCompactSensorEvents
// (NativePostSolveKernels:601-648) and rigid bodies in nativeCompactPolygonSensorEvents (:740-775, overlap rule
// nativeRigidOverlapsSensor :697-738): a pair the sensor's object filter does not allow, or whose object was removed,
// overlaps nothing; an enter or exit event goes out when the pair's state flips and the sensor asked for that kind.
// The reference appends events with an atomic counter; here one kernel writes each pair's event kind and a second,
// single-block kernel compacts them in pair order (sensor, then the world's bubbles, then its bodies), so the list is
// deterministic. The sensor's rotation is taken once on the host (cosf / sinf), so the oracle evaluates the same
// floats.
#include "bp_device.cuh"

namespace bp {

struct DSensor {
    float2 pos;
    float c, s, radius;
    uint32_t voff, vcount, flags;
    int64_t id;
};

__device__ __forceinline__ float2 sensor_vertex(const DSensor& sn, const float2* verts, uint32_t j) {
    return add(sn.pos, rot_cs(verts[sn.voff + j], sn.c, sn.s));
}

// nativePointInPolygon (NativePostSolveKernels:650-659) over the sensor's world-frame ring.
__device__ bool inside_sensor(float2 p, const DSensor& sn, const float2* verts) {
    bool inside = false;
    for (uint32_t j = 0; j < sn.vcount; ++j) {
        const float2 a = sensor_vertex(sn, verts, j), b = sensor_vertex(sn, verts, (j + 1u) % sn.vcount);
        if ((a.y > p.y) != (b.y > p.y) && p.x < (b.x - a.x) * (p.y - a.y) / (b.y - a.y) + a.x) inside = !inside;
    }
    return inside;
}
// The same rule over a body polygon at its end-of-step pose.
__device__ bool inside_body(float2 p, const DBody& b, const Pose& pose, const float2* verts) {
    bool inside = false;
    for (uint32_t j = 0; j < b.vcount; ++j) {
        const float2 a = body_vertex(verts, b, pose, j), c = body_vertex(verts, b, pose, (j + 1u) % b.vcount);
        if ((a.y > p.y) != (c.y > p.y) && p.x < (c.x - a.x) * (p.y - a.y) / (c.y - a.y) + a.x) inside = !inside;
    }
    return inside;
}
// nativePointSegmentDistanceSquared (:660-665)
__device__ __forceinline__ float point_segment_d2(float2 p, float2 a, float2 b) {
    const float2 ab = sub(b, a);
    const float t = clampf(dot2(sub(p, a), ab) / fmaxf(dot2(ab, ab), 1e-20f), 0.0f, 1.0f);
    const float2 d = sub(p, add(a, mul(ab, t)));
    return dot2(d, d);
}
// nativeSegmentsCross (:667-676): boxes first, then the four orientation signs (touching counts).
__device__ bool segments_cross(float2 a, float2 b, float2 c, float2 d) {
    if (fmaxf(fminf(a.x, b.x), fminf(c.x, d.x)) > fminf(fmaxf(a.x, b.x), fmaxf(c.x, d.x)) ||
        fmaxf(fminf(a.y, b.y), fminf(c.y, d.y)) > fminf(fmaxf(a.y, b.y), fmaxf(c.y, d.y)))
        return false;
    const float2 ab = sub(b, a), cd = sub(d, c);
    const float p = cross2(ab, sub(c, a)), q = cross2(ab, sub(d, a));
    const float r = cross2(cd, sub(a, c)), s = cross2(cd, sub(b, c));
    return ((p <= 0.0f && q >= 0.0f) || (p >= 0.0f && q <= 0.0f)) && ((r <= 0.0f && s >= 0.0f) || (r >= 0.0f && s <= 0.0f));
}
// nativeSegmentDistance (NativeGeometryKernels:444-462): 0 when the segments cross, else the smallest of the four
// endpoint-to-segment distances.
__device__ float segment_distance(float2 a, float2 b, float2 c, float2 d) {
    const float2 r = sub(b, a), s = sub(d, c);
    const float denominator = cross2(r, s);
    if (fabsf(denominator) > 1e-12f) {
        const float2 qp = sub(c, a);
        const float t = cross2(qp, s) / denominator, u = cross2(qp, r) / denominator;
        if (t >= 0.0f && t <= 1.0f && u >= 0.0f && u <= 1.0f) return 0.0f;
    }
    float best = INFINITY;
    best = fminf(best, len2(sub(a, closest_point(a, c, d))));
    best = fminf(best, len2(sub(b, closest_point(b, c, d))));
    best = fminf(best, len2(sub(c, closest_point(c, a, b))));
    best = fminf(best, len2(sub(d, closest_point(d, a, b))));
    return best;
}

// A bubble against a sensor: its centre in the sensor's frame, within the summed radii of a circle sensor, or inside a
// polygon sensor or within its radius of an edge (:610-632).
__device__ bool bubble_overlaps(const DSensor& sn, const float2* verts, float2 center, float radius) {
    const float2 d = sub(center, sn.pos);
    const float2 local = f2(sn.c * d.x + sn.s * d.y, -sn.s * d.x + sn.c * d.y);
    if (sn.vcount == 0u) {
        const float reach = sn.radius + radius;
        return dot2(local, local) <= reach * reach;
    }
    bool inside = false, near = false;
    for (uint32_t j = 0; j < sn.vcount; ++j) {
        const float2 a = verts[sn.voff + j], b = verts[sn.voff + (j + 1u) % sn.vcount];
        if ((a.y > local.y) != (b.y > local.y) && local.x < (b.x - a.x) * (local.y - a.y) / (b.y - a.y) + a.x)
            inside = !inside;
        const float2 ab = sub(b, a);
        const float t = clampf(dot2(sub(local, a), ab) / fmaxf(dot2(ab, ab), 1e-20f), 0.0f, 1.0f);
        const float2 delta = sub(local, add(a, mul(ab, t)));
        if (dot2(delta, delta) <= radius * radius) near = true;
    }
    return near || inside;
}

// A body at its end-of-step pose against a sensor (nativeRoundOverlapsSensor / nativeRigidOverlapsSensor): a circle or
// capsule as its core with the shape radius; a polygon by its edges, plus containment either way.
__device__ bool body_overlaps(const DSensor& sn, const float2* sverts, const DBody& b, const float2* bverts) {
    if (b.vcount == 0u) return false;
    const Pose pose{b.pos, b.cosEnd, b.sinEnd};
    if (b.kind != BP_BODY_POLYGON) {
        const float2 a = body_vertex(bverts, b, pose, 0), e = b.vcount > 1u ? body_vertex(bverts, b, pose, 1) : a;
        if (sn.vcount == 0u) {
            const float reach = b.coreRadius + sn.radius;
            return point_segment_d2(sn.pos, a, e) <= reach * reach;
        }
        if (inside_sensor(a, sn, sverts)) return true;
        for (uint32_t j = 0; j < sn.vcount; ++j)
            if (segment_distance(a, e, sensor_vertex(sn, sverts, j), sensor_vertex(sn, sverts, (j + 1u) % sn.vcount)) <=
                b.coreRadius)
                return true;
        return false;
    }
    if (sn.vcount == 0u && inside_body(sn.pos, b, pose, bverts)) return true;
    for (uint32_t i = 0; i < b.vcount; ++i) {
        const float2 a = body_vertex(bverts, b, pose, i), e = body_vertex(bverts, b, pose, (i + 1u) % b.vcount);
        if (sn.vcount == 0u) {
            if (point_segment_d2(sn.pos, a, e) <= sn.radius * sn.radius) return true;
        } else {
            if (inside_sensor(a, sn, sverts)) return true;
            for (uint32_t j = 0; j < sn.vcount; ++j)
                if (segments_cross(a, e, sensor_vertex(sn, sverts, j), sensor_vertex(sn, sverts, (j + 1u) % sn.vcount)))
                    return true;
        }
    }
    if (sn.vcount) return inside_body(sensor_vertex(sn, sverts, 0), b, pose, bverts);
    return false;
}

// One thread per (sensor, object) pair; objects are the world's bubbles, then its bodies.
__global__ void sensor_overlap_kernel(DState S, DWorld W, const DSensor* sensors, uint32_t sensorCount,
                                      const float2* verts, const uint8_t* allowed, uint8_t* state, uint8_t* kinds) {
    const uint32_t objects = W.n + W.nb;
    const uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (uint64_t)sensorCount * objects) return;
    const uint32_t si = (uint32_t)(idx / objects), j = (uint32_t)(idx % objects);
    const DSensor sensor = sensors[si];
    bool overlapping = false;
    if (!allowed || allowed[idx]) {
        if (j < W.n) {
            const uint32_t g = W.boff + j;
            if (!(S.flags[g] & kRemoved)) overlapping = bubble_overlaps(sensor, verts, S.pPos[g], S.phys[g].x);
        } else {
            overlapping = body_overlaps(sensor, verts, S.body[W.bodyOff + (j - W.n)], S.bverts);
        }
    }
    const bool was = state[idx] != 0;
    state[idx] = overlapping ? 1 : 0;
    uint8_t kind = 0;
    if (overlapping && !was && (sensor.flags & BP_SENSOR_ENTER_EVENTS)) kind = 1;
    else if (!overlapping && was && (sensor.flags & BP_SENSOR_EXIT_EVENTS)) kind = 2;
    kinds[idx] = kind;
}

// One block: the pairs with an event, in pair order, into `events` (at most `capacity`); *count = all of them.
__global__ void __launch_bounds__(1024) sensor_compact_kernel(DState S, DWorld W, const DSensor* sensors,
                                                              uint32_t sensorCount, const uint8_t* kinds,
                                                              bp_sensor_event* events, uint32_t capacity,
                                                              uint32_t* count) {
    __shared__ uint32_t warpTotals[32];
    __shared__ uint32_t running;
    const uint32_t t = threadIdx.x, lane = t & 31u, warp = t >> 5, warps = blockDim.x >> 5;
    const uint32_t objects = W.n + W.nb;
    const uint64_t total = (uint64_t)sensorCount * objects;
    if (t == 0) running = 0;
    __syncthreads();
    for (uint64_t base = 0; base < total; base += blockDim.x) {
        const uint64_t idx = base + t;
        const uint8_t kind = idx < total ? kinds[idx] : 0;
        const uint32_t flag = kind ? 1u : 0u;
        const uint32_t ballot = __ballot_sync(0xffffffffu, flag);
        const uint32_t before = __popc(ballot & ((1u << lane) - 1u));
        if (lane == 0) warpTotals[warp] = __popc(ballot);
        __syncthreads();
        uint32_t offset = running;
        for (uint32_t w = 0; w < warp; ++w) offset += warpTotals[w];
        if (flag) {
            const uint32_t slot = offset + before;
            if (slot < capacity) {
                const uint32_t si = (uint32_t)(idx / objects), j = (uint32_t)(idx % objects);
                bp_sensor_event e;
                e.sensor = sensors[si].id;
                e.kind = kind;
                if (j < W.n) {
                    const uint32_t g = W.boff + j;
                    e.object = S.id[g];
                    e.point[0] = S.pPos[g].x;
                    e.point[1] = S.pPos[g].y;
                    e.object_kind = 0;
                } else {
                    const DBody& b = S.body[W.bodyOff + (j - W.n)];
                    e.object = b.id;
                    e.point[0] = b.pos.x;
                    e.point[1] = b.pos.y;
                    e.object_kind = 1;
                }
                events[slot] = e;
            }
        }
        __syncthreads();
        if (t == 0) {
            uint32_t sum = 0;
            for (uint32_t w = 0; w < warps; ++w) sum += warpTotals[w];
            running += sum;
        }
        __syncthreads();
    }
    if (t == 0) *count = running;
}

cudaError_t launch_sensors(const DState& S, const DWorld& W, const void* sensors, uint32_t sensorCount,
                           const float2* verts, const uint8_t* allowed, uint8_t* state, uint8_t* kinds,
                           bp_sensor_event* events, uint32_t capacity, uint32_t* count, cudaStream_t stream) {
    const uint64_t total = (uint64_t)sensorCount * (W.n + W.nb);
    if (total == 0u) return cudaMemsetAsync(count, 0, sizeof(uint32_t), stream);
    const DSensor* ds = (const DSensor*)sensors;
    sensor_overlap_kernel<<<(unsigned)((total + 255u) / 256u), 256, 0, stream>>>(S, W, ds, sensorCount, verts, allowed,
                                                                                 state, kinds);
    sensor_compact_kernel<<<1, 1024, 0, stream>>>(S, W, ds, sensorCount, kinds, events, capacity, count);
    return cudaGetLastError();
}

size_t sensor_record_bytes() { return sizeof(DSensor); }

// Host records -> device records: the rotation as cosf / sinf of the angle (the oracle takes the same two floats).
void sensor_to_device(const bp_sensor& in, void* out) {
    DSensor d{};
    d.pos = make_float2(in.position[0], in.position[1]);
    d.c = std::cos(in.angle);
    d.s = std::sin(in.angle);
    d.radius = in.radius;
    d.voff = in.vertex_offset;
    d.vcount = in.vertex_count;
    d.flags = in.flags;
    d.id = in.id;
    *(DSensor*)out = d;
}

}  // namespace bp
