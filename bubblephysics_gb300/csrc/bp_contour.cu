// bp_contour.cu - bubble contours of a world's published state as a headless device buffer (draw-only data: contours
// never feed back into the physics).
//
// The reference builds them after the step in three passes (NativePostSolveKernels.metal-source):
// nativeAccumulateContactPressure (:280-334) casts one ray per sample from the centre and shortens it to the nearest
// one-sided segment and to the flat chord of every overlapping pair, which lies at r (1 - eps) from the centre with
// eps the pair law's deflection of this end; nativeGenerateContoursFused (:353-381) smooths the radial deficits with
// 13 Jacobi passes that never go below the hard limit; nativePrepareRenderDataGrouped (:437-527) closes the field with
// the smallest majorant of bounded slope (two serial passes from the global maximum), then writes the points, the
// bounds, the effective radius and the largest deficit. Here one block steps one bubble through all three, one thread
// per sample, with the deficits in shared memory; the serial majorant runs on one thread like the reference's (a chain
// of float subtractions whose order fixes the bits).
#include <cmath>
#include <vector>

#include "bp_device.cuh"

namespace bp {

constexpr uint32_t kContourPasses = 13;

struct ContourArgs {
    float maxEdge, tension, clearance;
    uint32_t stride;
};

// nativeContourRayLimit (NativePostSolveKernels:268-277)
__device__ __forceinline__ float contour_ray_limit(float2 center, float2 direction, float2 a, float2 b, float radius,
                                                   float clearance) {
    const float2 edge = sub(b, a), offset = sub(a, center);
    const float denominator = cross2(direction, edge);
    if (fabsf(denominator) < 1e-6f) return radius;
    const float distance = cross2(offset, edge) / denominator;
    const float fraction = cross2(offset, direction) / denominator;
    return distance >= 0.0f && fraction >= 0.0f && fraction <= 1.0f ? fminf(radius, fmaxf(0.0f, distance - clearance))
                                                                      : radius;
}

__global__ void __launch_bounds__(1024) contour_kernel(DState S, DWorld W, ContourArgs a, const float2* dirs,
                                                       float2* points, uint32_t* counts, float* level, float* shape) {
    __shared__ float lvl[1024];
    __shared__ float part[32][6];
    __shared__ float seedMaximum;
    const uint32_t i = blockIdx.x, s = threadIdx.x, g = W.boff + i;
    const float r = S.phys[g].x;
    const bool gone = (S.flags[g] & kRemoved) != 0u || !(r > 0.0f);
    const uint32_t count = gone ? 0u : contour_samples(r, a.maxEdge, a.stride);
    if (s == 0) counts[i] = count;
    if (count == 0u) return;  // uniform over the block
    const bool active = s < count;
    const float2 c = S.pPos[g];
    float2 direction = f2(1.0f, 0.0f);
    float deficit = 0.0f;
    if (active) {
        direction = dirs[contour_dir_offset(count) + s];
        float limit = r;
        const uint2 fi = S.filter[g];
        for (uint32_t j = 0; j < W.s; ++j) {
            const DSegment& sg = S.seg[W.soff + j];
            if (!filter_accepts(fi, make_uint2(sg.cat, sg.mask))) continue;
            limit = contour_ray_limit(c, direction, sg.a, sg.b, limit, a.clearance);
        }
        const uint32_t* row = S.adj + W.rowOff + (uint64_t)i * W.k;
        const uint32_t deg = S.deg[g];
        for (uint32_t e = 0; e < deg; ++e) {
            const uint32_t key = row[e];
            if (key >> kKindShift) continue;  // walls and segments cut the contour through the loop above
            const uint32_t j = key & kIndexMask, gj = W.boff + j;
            const float2 delta = sub(S.pPos[gj], c);
            const float distance = len2(delta);
            const float rj = S.phys[gj].x;
            if (distance <= 1.1920929e-7f || distance >= r + rj) continue;
            const float2 normal = dvd(delta, distance);
            const bool lowIsSelf = i < j;
            const float4 first = lowIsSelf ? S.phys[g] : S.phys[gj], second = lowIsSelf ? S.phys[gj] : S.phys[g];
            const Law law = pair_law(first.z, first.x, second.z, second.x, distance);
            const float eps = lowIsSelf ? law.epsA : law.epsB;
            const float plane = clampf(r * (1.0f - eps), 0.0f, r);
            const float half = sqrtf(fmaxf(0.0f, r * r - plane * plane));
            const float2 tangent = f2(-normal.y, normal.x);
            const float2 point = add(c, mul(normal, plane));
            limit = contour_ray_limit(c, direction, sub(point, mul(tangent, half)), add(point, mul(tangent, half)), limit,
                                      a.clearance);
        }
        deficit = clampf(1.0f - limit / r, 0.0f, 1.0f);
    }
    // smoothing: a convex combination with the neighbours' mean, never below the hard deficit
    float x = deficit;
    const float floorValue = deficit;
    lvl[s] = active ? x : 0.0f;
    __syncthreads();
    const float tension = fminf(0.8f, a.tension / (a.tension + 10.0f));
    for (uint32_t pass = 0; pass < kContourPasses; ++pass) {
        if (active) {
            const float neighbour = (lvl[(s + count - 1u) % count] + lvl[(s + 1u) % count]) * 0.5f;
            x = clampf(fmaxf(floorValue, x + (neighbour - x) * tension), 0.0f, 1.0f);
        }
        __syncthreads();
        lvl[s] = x;
        __syncthreads();
    }
    // bounded-slope majorant from the global maximum, both ways round
    if (s == 0) {
        float maximum = 0.0f;
        uint32_t anchor = 0;
        for (uint32_t k = 0; k < count; ++k)
            if (lvl[k] > maximum) { maximum = lvl[k]; anchor = k; }
        const float slope = a.maxEdge / (2.0f * r);
        float previous = maximum;
        for (uint32_t step = 1; step < count; ++step) {
            const uint32_t k = (anchor + step) % count;
            const float v = fmaxf(lvl[k], previous - slope);
            lvl[k] = v;
            previous = v;
        }
        previous = maximum;
        for (uint32_t step = 1; step < count; ++step) {
            const uint32_t k = (anchor + count - step) % count;
            const float v = fmaxf(lvl[k], previous - slope);
            lvl[k] = v;
            previous = v;
        }
        seedMaximum = maximum;
    }
    __syncthreads();
    const float inf = __int_as_float(0x7f800000);
    float v[6] = {inf, -inf, inf, inf, -inf, -inf};  // min |p - c|, max level, bounds min x, min y, max x, max y
    if (active) {
        const float l = lvl[s];
        const float2 p = add(c, mul(direction, r * (1.0f - l)));
        const uint64_t at = (uint64_t)i * a.stride + s;
        points[at] = p;
        if (level) level[at] = l;
        v[0] = len2(sub(p, c));
        v[1] = l;
        v[2] = p.x; v[3] = p.y; v[4] = p.x; v[5] = p.y;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        v[0] = fminf(v[0], __shfl_xor_sync(0xffffffffu, v[0], off));
        v[1] = fmaxf(v[1], __shfl_xor_sync(0xffffffffu, v[1], off));
        v[2] = fminf(v[2], __shfl_xor_sync(0xffffffffu, v[2], off));
        v[3] = fminf(v[3], __shfl_xor_sync(0xffffffffu, v[3], off));
        v[4] = fmaxf(v[4], __shfl_xor_sync(0xffffffffu, v[4], off));
        v[5] = fmaxf(v[5], __shfl_xor_sync(0xffffffffu, v[5], off));
    }
    const uint32_t lane = s & 31u, warp = s >> 5, warps = (blockDim.x + 31u) >> 5;
    if (lane == 0)
        for (int q = 0; q < 6; ++q) part[warp][q] = v[q];
    __syncthreads();
    if (s == 0) {
        for (uint32_t w = 1; w < warps; ++w) {
            v[0] = fminf(v[0], part[w][0]);
            v[1] = fmaxf(v[1], part[w][1]);
            v[2] = fminf(v[2], part[w][2]);
            v[3] = fminf(v[3], part[w][3]);
            v[4] = fmaxf(v[4], part[w][4]);
            v[5] = fmaxf(v[5], part[w][5]);
        }
        float* out = shape + (uint64_t)i * 6u;
        out[0] = fmaxf(seedMaximum, v[1]);       // largest deficit
        out[1] = fminf(r, v[0]);                 // effective radius
        out[2] = fminf(c.x, v[2]);
        out[3] = fminf(c.y, v[3]);
        out[4] = fmaxf(c.x, v[4]);
        out[5] = fmaxf(c.y, v[5]);
    }
}

// Hit test of query points (nativeHitTest, NativeGeometryKernels:501-541): among the bubbles whose contour contains the
// point (bounds first, then the even-odd rule over the contour, the reference's crossing formula), the bodies that
// contain it, and the static polygons that contain it (their one-sided edges, consecutive per owner), the highest
// (layer as a signed 32-bit value, then id as an unsigned 64-bit value) wins.
__global__ void hit_test_kernel(DState S, DWorld W, const float2* queries, uint32_t queryCount, const float2* cpoints,
                                const uint32_t* ccounts, const float* shape, uint32_t stride,
                                const uint32_t* bubbleLayers, const uint32_t* segLayers, const uint32_t* bodyLayers,
                                long long* ids, uint32_t* layers, uint32_t* found) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= queryCount) return;
    const float2 query = queries[q];
    bool any = false;
    uint32_t bestLayer = 0;
    unsigned long long bestId = 0;
    auto offer = [&](uint32_t bits, long long id) {  // layers order like Int32 (NativeMetalHitTestTests.swift:123-132)
        const int32_t layer = (int32_t)bits, best = (int32_t)bestLayer;
        const unsigned long long u = (unsigned long long)id;
        if (!any || layer > best || (layer == best && u > bestId)) { any = true; bestLayer = bits; bestId = u; }
    };
    for (uint32_t i = 0; i < W.n; ++i) {
        const uint32_t g = W.boff + i;
        if (S.flags[g] & kRemoved) continue;
        const float* box = shape + (uint64_t)i * 6u;
        if (query.x < box[2] || query.y < box[3] || query.x > box[4] || query.y > box[5]) continue;
        const uint32_t count = min(ccounts[i], stride);
        if (count < 3u) continue;
        bool inside = false;
        const float2* ring = cpoints + (uint64_t)i * stride;
        for (uint32_t k = 0, j = count - 1u; k < count; j = k++) {
            const float2 a = ring[k], b = ring[j];
            const bool crosses = ((a.y > query.y) != (b.y > query.y)) &&
                                 (query.x <= (b.x - a.x) * (query.y - a.y) / (b.y - a.y) + a.x);
            inside = crosses ? !inside : inside;
        }
        if (inside) offer(bubbleLayers[i], S.id[g]);
    }
    for (uint32_t bi = 0; bi < W.nb; ++bi) {
        const DBody& b = S.body[W.bodyOff + bi];
        if (rigid_inside(S.bverts, S.btris, query, b, body_at(b, 1.0f))) offer(bodyLayers[bi], b.id);
    }
    // static polygons: even-odd over each owner's run of polygon edges
    bool inside = false;
    for (uint32_t j = 0; j < W.s; ++j) {
        const DSegment& sg = S.seg[W.soff + j];
        if ((sg.flags & (BP_SEGMENT_POLYGON_EDGE | BP_SEGMENT_HAS_OWNER)) != (BP_SEGMENT_POLYGON_EDGE | BP_SEGMENT_HAS_OWNER))
            continue;
        const float2 a = sg.b, b = sg.a;
        if (((a.y > query.y) != (b.y > query.y)) && (query.x <= (b.x - a.x) * (query.y - a.y) / (b.y - a.y) + a.x))
            inside = !inside;
        const bool last = j + 1u == W.s || S.seg[W.soff + j + 1u].owner != sg.owner;
        if (last) {
            if (inside) offer(segLayers[j], sg.owner);
            inside = false;
        }
    }
    ids[q] = (long long)bestId;
    layers[q] = bestLayer;
    found[q] = any ? 1u : 0u;
}

cudaError_t launch_hit_test(const DState& S, const DWorld& W, const float2* queries, uint32_t queryCount,
                            const float2* cpoints, const uint32_t* ccounts, const float* shape, uint32_t stride,
                            const uint32_t* bubbleLayers, const uint32_t* segLayers, const uint32_t* bodyLayers,
                            long long* ids, uint32_t* layers, uint32_t* found, cudaStream_t stream) {
    if (queryCount == 0u) return cudaSuccess;
    hit_test_kernel<<<(queryCount + 127u) / 128u, 128, 0, stream>>>(S, W, queries, queryCount, cpoints, ccounts, shape,
                                                                    stride, bubbleLayers, segLayers, bodyLayers, ids,
                                                                    layers, found);
    return cudaGetLastError();
}

// Sample directions of every sample count from 1 to `stride` (contour_dir_offset): sample s of a count lies at the float
// angle 2 pi s / count (the reference's expression), and its direction is the cosine and sine of that angle evaluated in
// double precision and rounded to float. They are computed on the host once, so every build of the contours uses the
// same directions.
std::vector<float2> contour_directions(uint32_t stride) {
    std::vector<float2> out(contour_dir_offset(stride + 1u));
    for (uint32_t count = 1; count <= stride; ++count) {
        float2* d = out.data() + contour_dir_offset(count);
        for (uint32_t s = 0; s < count; ++s) {
            const float angle = 2.0f * kPiF * (float)s / (float)count;
            d[s] = make_float2((float)std::cos((double)angle), (float)std::sin((double)angle));
        }
    }
    return out;
}

cudaError_t launch_contours(const DState& S, const DWorld& W, float maxEdge, float tension, float clearance,
                            uint32_t stride, const float2* dirs, float2* points, uint32_t* counts, float* level,
                            float* shape, cudaStream_t stream) {
    if (W.n == 0u) return cudaSuccess;
    if (stride == 0u || stride > 1024u || !dirs) return cudaErrorInvalidValue;
    ContourArgs a{maxEdge, tension, clearance, stride};
    const uint32_t threads = (stride + 31u) & ~31u;
    contour_kernel<<<W.n, threads, 0, stream>>>(S, W, a, dirs, points, counts, level, shape);
    return cudaGetLastError();
}

}  // namespace bp
