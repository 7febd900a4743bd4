// bp_sensor.cu - sensor enter / exit events of a world's bubbles after each step.
//
// The reference compares every (sensor, bubble) pair on the GPU after the step (nativeCompactSensorEvents,
// NativePostSolveKernels:601-648): the bubble's centre is taken into the sensor's frame; a circle sensor overlaps a
// bubble within the sum of the radii, a polygon sensor when the centre is inside (even-odd rule) or an edge is within
// the bubble's radius; a removed bubble overlaps nothing; an enter or exit event goes out when the state flips and the
// sensor asked for that kind. The reference appends events with an atomic counter; here one kernel writes each pair's
// event kind and a second, single-block kernel compacts them in (sensor, bubble) order, so the list is deterministic.
#include "bp_device.cuh"

namespace bp {

struct DSensor {
    float2 pos;
    float angle, radius;
    uint32_t voff, vcount, flags, cat, mask, pad;
    int64_t id;
};

__global__ void sensor_overlap_kernel(DState S, DWorld W, const DSensor* sensors, uint32_t sensorCount,
                                      const float2* verts, uint8_t* state, uint8_t* kinds) {
    const uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t total = (uint64_t)sensorCount * W.n;
    if (idx >= total) return;
    const uint32_t si = (uint32_t)(idx / W.n), i = (uint32_t)(idx % W.n), g = W.boff + i;
    const DSensor sensor = sensors[si];
    bool overlapping = false;
    if (!(S.flags[g] & kRemoved) && filter_accepts(S.filter[g], make_uint2(sensor.cat, sensor.mask))) {
        const float2 d = sub(S.pPos[g], sensor.pos);
        const float c = cosf(sensor.angle), s = sinf(sensor.angle);
        const float2 local = f2(c * d.x + s * d.y, -s * d.x + c * d.y);
        const float radius = S.phys[g].x;
        if (sensor.vcount == 0u) {
            const float reach = sensor.radius + radius;
            overlapping = dot2(local, local) <= reach * reach;
        } else {
            bool inside = false;
            for (uint32_t j = 0; j < sensor.vcount; ++j) {
                const float2 a = verts[sensor.voff + j], b = verts[sensor.voff + (j + 1u) % sensor.vcount];
                if ((a.y > local.y) != (b.y > local.y) && local.x < (b.x - a.x) * (local.y - a.y) / (b.y - a.y) + a.x)
                    inside = !inside;
                const float2 ab = sub(b, a);
                const float t = clampf(dot2(sub(local, a), ab) / fmaxf(dot2(ab, ab), 1e-20f), 0.0f, 1.0f);
                const float2 delta = sub(local, add(a, mul(ab, t)));
                if (dot2(delta, delta) <= radius * radius) overlapping = true;
            }
            overlapping = overlapping || inside;
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
    const uint64_t total = (uint64_t)sensorCount * W.n;
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
                const uint32_t si = (uint32_t)(idx / W.n), i = (uint32_t)(idx % W.n), g = W.boff + i;
                bp_sensor_event e;
                e.sensor = sensors[si].id;
                e.object = S.id[g];
                e.kind = kind;
                e.point[0] = S.pPos[g].x;
                e.point[1] = S.pPos[g].y;
                e.reserved = 0;
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
                           const float2* verts, uint8_t* state, uint8_t* kinds, bp_sensor_event* events,
                           uint32_t capacity, uint32_t* count, cudaStream_t stream) {
    if (sensorCount == 0u || W.n == 0u) return cudaMemsetAsync(count, 0, sizeof(uint32_t), stream);
    const uint64_t total = (uint64_t)sensorCount * W.n;
    const DSensor* ds = (const DSensor*)sensors;
    sensor_overlap_kernel<<<(unsigned)((total + 255u) / 256u), 256, 0, stream>>>(S, W, ds, sensorCount, verts, state, kinds);
    sensor_compact_kernel<<<1, 1024, 0, stream>>>(S, W, ds, sensorCount, kinds, events, capacity, count);
    return cudaGetLastError();
}

size_t sensor_record_bytes() { return sizeof(DSensor); }

// Host records -> device records (same fields, the device layout).
void sensor_to_device(const bp_sensor& in, void* out) {
    DSensor d{};
    d.pos = make_float2(in.position[0], in.position[1]);
    d.angle = in.angle;
    d.radius = in.radius;
    d.voff = in.vertex_offset;
    d.vcount = in.vertex_count;
    d.flags = in.flags;
    d.cat = in.category;
    d.mask = in.mask;
    d.id = in.id;
    *(DSensor*)out = d;
}

}  // namespace bp
