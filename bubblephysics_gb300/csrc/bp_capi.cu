// bp_capi.cu - host side of the C ABI (include/bubblephysics.h).
//
// A single world (bp_world) and a batch (bp_batch) share one implementation, WorldSet: every resident world's bubbles,
// segments and bodies live back to back in SoA device arrays, with a per-world table (DWorld) of offsets. Worlds of up
// to kCtaMaxBubbles bubbles are stepped one thread block per world, grouped into power-of-two size classes (one launch
// per class and step, all classes of a step captured into one CUDA graph); larger worlds use a cooperative launch over
// the whole GPU. The plain per-world path launches each world on its own, one after another (what the reference does:
// one command-buffer pair per world and frame, NativeMetalSubstepLoop.swift:216-273).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "bp_host.h"


using namespace bp;
using namespace bp_host;

static_assert(sizeof(bp_bubble) == 80, "bp_bubble layout");
static_assert(sizeof(bp_segment) == 64, "bp_segment layout");
static_assert(sizeof(bp_body) == 80, "bp_body layout");
static_assert(sizeof(bp_force_field) == 64, "bp_force_field layout");
static_assert(sizeof(bp_band) == 24 && sizeof(bp_motor) == 24, "band / motor layout");
static_assert(sizeof(bp_world_desc) == 64, "bp_world_desc layout");
static_assert(sizeof(bp_step_report) == 96, "bp_step_report layout");
static_assert(sizeof(bp_contact) == 64, "bp_contact layout");
static_assert(sizeof(bp_candidate_key) == 24, "bp_candidate_key layout");
static_assert(sizeof(bp_sensor) == 48 && sizeof(bp_sensor_event) == 32, "sensor record layouts");
static_assert(sizeof(bp_contour_config) == 16, "bp_contour_config layout");
static_assert(sizeof(bp_contact_event) == 48, "bp_contact_event layout");
static_assert(offsetof(bp_bubble, center) == 8 && offsetof(bp_bubble, flags) == 60, "bp_bubble offsets");
static_assert(offsetof(bp_step_report, limiter_object) == 40, "bp_step_report offsets");




struct bp_world {
    WorldSet set;
};
struct bp_batch {
    WorldSet set;
};

namespace bp_host {

int validate(const bp_world_desc& d, const bp_world_input& in) {
    if (!(d.time_step > 0.0f) || !std::isfinite(d.time_step)) return BP_E_INVALID;
    if (d.candidate_limit > 128u) return BP_E_CAPACITY;
    if (in.bubble_count && !in.bubbles) return BP_E_INVALID;
    if (in.segment_count && !in.segments) return BP_E_INVALID;
    if (in.body_count && !in.bodies) return BP_E_INVALID;
    for (uint32_t i = 0; i < in.bubble_count; ++i) {
        const bp_bubble& b = in.bubbles[i];
        if (i > 0 && !(in.bubbles[i - 1].id < b.id)) return BP_E_INVALID;  // sorted by id (NativePublicWorld.swift:248)
        if (!std::isfinite(b.center[0]) || !std::isfinite(b.center[1]) || !std::isfinite(b.velocity[0]) ||
            !std::isfinite(b.velocity[1]) || !(b.radius > 0.0f) || !std::isfinite(b.radius) || !std::isfinite(b.mass))
            return BP_E_INVALID;
    }
    for (uint32_t j = 1; j < in.segment_count; ++j)
        if (!(in.segments[j - 1].id < in.segments[j].id)) return BP_E_INVALID;
    for (uint32_t b = 0; b < in.body_count; ++b) {
        const bp_body& r = in.bodies[b];
        if (!(r.flags & (BP_BODY_STATIC | BP_BODY_KINEMATIC))) return BP_E_INVALID;  // dynamic bodies: not with bubbles
        if ((uint64_t)r.vertex_offset + r.vertex_count > in.body_vertex_count) return BP_E_INVALID;
        if ((uint64_t)r.triangle_offset + r.triangle_count > in.body_triangle_count) return BP_E_INVALID;
        if (r.vertex_count == 0) return BP_E_INVALID;
    }
    for (uint32_t b = 0; b < in.body_count; ++b) {
        const bp_body& r = in.bodies[b];
        for (uint64_t t = 0; t < 3ull * r.triangle_count; ++t)
            if (in.body_triangles[3ull * r.triangle_offset + t] >= r.vertex_count) return BP_E_INVALID;
    }
    for (uint32_t f = 0; f < in.field_count; ++f) {
        const bp_force_field& r = in.fields[f];
        if ((uint64_t)r.vertex_offset + r.vertex_count > in.field_vertex_count) return BP_E_INVALID;
        if (r.has_filter && (uint64_t)r.filter_offset + r.filter_count > in.field_object_id_count) return BP_E_INVALID;
    }
    if (in.joint_entity_count && in.joint_entity_count > in.bubble_count + in.body_count) return BP_E_INVALID;
    return BP_OK;
}

bool group_layout(uint32_t threads, uint32_t groupWidth, uint32_t maxN, uint32_t* wsCap) {
    const uint32_t groups = std::max(threads / std::max(groupWidth, 32u), 1u);
    const uint32_t gridBytes = team_grid_bytes(maxN, std::max(groupWidth, 32u));
    const uint32_t fixed = 4u * group_scratch_words(groupWidth) + gridBytes;
    const uint32_t perGroup = kMaxDynamicSmem / groups;
    if (fixed + 16u > perGroup) return false;
    *wsCap = std::min(kWarpWorkspaceCap * std::max(groupWidth / 32u, 1u), perGroup - fixed - 16u);
    return true;
}

// Initial split of the non-large worlds into the CTA and group queues (largest first) for a block width, group-queue
// threshold and group width; after every batched step the on-device scheduler reorders both queues by predicted
// cost. Shared memory is sized so any world can be a CTA world and any world up to the threshold a group world.
cudaError_t schedule(WorldSet& ws, uint32_t threads, uint32_t warpMax, uint32_t groupWidth) {
    groupWidth = std::min(std::max(groupWidth, 32u), threads);
    if (threads % groupWidth) groupWidth = 32u;  // groups tile the block exactly
    ws.threads = threads;
    ws.warpMax = warpMax;
    ws.groupWidth = groupWidth;
    ws.ctaWorlds.clear();
    ws.warpWorlds.clear();
    std::vector<uint32_t> candidates;
    uint32_t maxN = 1, maxWarpN = 0, ctaWs = 0, warpWs = 0;
    for (uint32_t w = 0; w < ws.nWorlds; ++w) {
        const DWorld& W = ws.hWorlds[w];
        if (W.n > kCtaMaxBubbles || (W.flags & BP_WORLD_FORCE_MULTI_CTA)) continue;
        candidates.push_back(w);
        maxN = std::max(maxN, W.n);
        if (W.n <= warpMax) maxWarpN = std::max(maxWarpN, W.n);
        (W.n <= warpMax ? ws.warpWorlds : ws.ctaWorlds).push_back(w);
    }
    // workspace caps that keep one block within the dynamic shared memory limit
    const uint32_t ctaGridBytes = team_grid_bytes(maxN, threads);
    const uint32_t ctaCap = std::min(kCtaWorkspaceCap, kMaxDynamicSmem - std::min(kMaxDynamicSmem, ctaGridBytes));
    uint32_t warpCap = 0;
    if (maxWarpN && !group_layout(threads, groupWidth, maxWarpN, &warpCap)) return cudaErrorInvalidValue;
    for (uint32_t w : candidates) {
        const DWorld& W = ws.hWorlds[w];
        uint32_t bytes = workspace_bytes(W.n, W.s, W.nb);
        if (bytes <= ctaCap) ctaWs = std::max(ctaWs, bytes);
        if (W.n <= warpMax && bytes <= warpCap) warpWs = std::max(warpWs, bytes);
    }
    auto bySize = [&](uint32_t a, uint32_t b) { return ws.hWorlds[a].n > ws.hWorlds[b].n; };
    std::stable_sort(ws.ctaWorlds.begin(), ws.ctaWorlds.end(), bySize);
    std::stable_sort(ws.warpWorlds.begin(), ws.warpWorlds.end(), bySize);
    QueueArgs& q = ws.queue;
    q.ctaList = ws.dCtaList;
    q.warpList = ws.dWarpList;
    q.queue = ws.dQueue;
    q.nCta = (uint32_t)ws.ctaWorlds.size();
    q.nWarp = (uint32_t)ws.warpWorlds.size();
    q.ctaMaxN = candidates.empty() ? 0u : maxN;
    q.ctaB = candidates.empty() ? 0u : grid_buckets(maxN);
    q.warpMaxN = maxWarpN;
    q.warpB = maxWarpN ? grid_buckets(maxWarpN) : 0u;
    q.countsOnDevice = 1u;
    q.tree = 0u;
    for (uint32_t w : candidates) q.tree |= ws.hWorlds[w].tree;
    q.ctaWsWords = ws.staging ? (ctaWs + 3u) / 4u : 0u;
    q.warpWsWords = ws.staging ? (warpWs + 3u) / 4u : 0u;
    q.ctaWsWords = (q.ctaWsWords + 3u) & ~3u;
    q.warpWsWords = (q.warpWsWords + 3u) & ~3u;
    q.groupWidth = groupWidth;
    ws.nCandidates = (uint32_t)candidates.size();
    uint32_t counts[2] = {q.nCta, q.nWarp};
    cudaError_t err = upload(ws.dCtaList, ws.ctaWorlds.data(), ws.ctaWorlds.size(), ws.ctx->stream);
    if (!err) err = upload(ws.dWarpList, ws.warpWorlds.data(), ws.warpWorlds.size(), ws.ctx->stream);
    if (!err) err = upload(ws.dCandidates, candidates.data(), candidates.size(), ws.ctx->stream);
    if (!err) err = upload(ws.dQueue + 2, counts, 2, ws.ctx->stream);
    if (!err) err = cudaStreamSynchronize(ws.ctx->stream);
    ws.blocks = persistent_blocks(q, threads);
    if (ws.graph) { cudaGraphExecDestroy(ws.graph); ws.graph = nullptr; }
    return err;
}

int build_set(WorldSet& ws, bp_context* ctx, uint32_t count, const bp_world_desc* descs, const bp_world_input* inputs,
              bool single) {
    ws.ctx = ctx;
    ws.nWorlds = count;
    DeviceGuard guard(ctx->device);
    // totals and validation
    uint64_t nb = 0, rows = 0, brows = 0, contacts = 0;
    uint64_t ns = 0, nbo = 0, nbv = 0, nbt = 0, nf = 0, nfv = 0, nfi = 0, nband = 0, nmotor = 0, njr = 0, njp = 0;
    for (uint32_t w = 0; w < count; ++w) {
        int st = validate(descs[w], inputs[w]);
        if (st != BP_OK) return st;
        const bp_world_input& in = inputs[w];
        uint32_t k = descs[w].candidate_limit == 0 ? 128u : descs[w].candidate_limit;
        nb += in.bubble_count;
        rows += (uint64_t)in.bubble_count * k;
        brows += (uint64_t)in.body_count * k;
        contacts += single ? (uint64_t)in.bubble_count * k + 64 : (uint64_t)in.bubble_count * 16 + 64;
        ns += in.segment_count; nbo += in.body_count; nbv += in.body_vertex_count; nbt += in.body_triangle_count;
        nf += in.field_count; nfv += in.field_vertex_count; nfi += in.field_object_id_count;
        nband += in.band_count; nmotor += in.motor_count;
        njr += in.joint_ranges ? in.joint_entity_count : 0; njp += in.joint_partners ? in.joint_partner_count : 0;
    }
    if (nb > 0x3fffffffull || ns > 0x3fffffffull) return BP_E_CAPACITY;
    ws.totalBubbles = nb;
    ws.totalRows = rows;
    ws.totalBodyRows = brows;
    ws.totalContacts = contacts;
    ws.totalSegments = (uint32_t)ns;
    ws.totalBodies = (uint32_t)nbo;

    // host staging in device layout
    std::vector<float2> pos(nb), start(nb), vel(nb), rotw(nb);
    std::vector<float4> phys(nb);
    std::vector<int64_t> ids(nb);
    std::vector<uint32_t> flags(nb);
    std::vector<uint2> filter(nb);
    std::vector<DSegment> segs(ns);
    std::vector<DBody> bodies(nbo);
    std::vector<float2> bverts(nbv);
    std::vector<uint32_t> btris(3 * nbt);
    std::vector<DField> fields(nf);
    std::vector<float2> fverts(nfv);
    std::vector<int64_t> fids(nfi);
    std::vector<bp_band> bands(nband);
    std::vector<bp_motor> motors(nmotor);
    std::vector<uint2> jranges(njr);
    std::vector<int64_t> jpartners(njp);
    ws.hWorlds.resize(count);
    ws.hBubbles.resize(nb);
    ws.hSegIds.resize(ns);
    ws.hBodyIds.resize(nbo);
    ws.hBodyLayers.resize(nbo);
    ws.hSegLayers.resize(ns);
    uint64_t otree = 0;
    uint64_t ob = 0, orow = 0, obrow = 0, ocon = 0, os = 0, obo = 0, obv = 0, obt = 0, of = 0, ofv = 0, ofi = 0, oband = 0,
             omotor = 0, ojr = 0, ojp = 0;
    for (uint32_t w = 0; w < count; ++w) {
        const bp_world_desc& d = descs[w];
        const bp_world_input& in = inputs[w];
        DWorld& W = ws.hWorlds[w];
        std::memset(&W, 0, sizeof(W));
        W.boff = (uint32_t)ob; W.n = in.bubble_count;
        W.soff = (uint32_t)os; W.s = in.segment_count;
        W.bodyOff = (uint32_t)obo; W.nb = in.body_count;
        W.foff = (uint32_t)of; W.nf = in.field_count;
        W.bandOff = (uint32_t)oband; W.nbands = in.band_count;
        W.motorOff = (uint32_t)omotor; W.nmotors = in.motor_count;
        W.jrOff = (uint32_t)ojr; W.njEnt = in.joint_ranges ? in.joint_entity_count : 0;
        W.k = d.candidate_limit == 0 ? 128u : d.candidate_limit;
        W.flags = d.flags;
        const uint32_t leaves = in.segment_count + in.body_count;
        const bool tree = leaves > 0u && !(d.flags & BP_WORLD_NO_RIGID_TREE) &&
                          ((d.flags & BP_WORLD_RIGID_TREE) || leaves >= kTreeMinLeaves);
        W.tree = tree ? 1u : 0u;
        W.treeOff = tree ? (uint32_t)otree : 0u;
        if (tree) otree += leaves;
        W.injectSubstep = 0;
        W.contactCap = single ? in.bubble_count * W.k + 64 : in.bubble_count * 16 + 64;
        W.rowOff = orow; W.bodyRowOff = obrow; W.contactOff = ocon;
        W.dt = d.time_step; W.sepTol = d.separation_tolerance; W.contactTol = d.contact_tolerance;
        W.split = d.substep_split_multiplier;
        W.rmin = make_float2(d.region[0], d.region[1]); W.rmax = make_float2(d.region[2], d.region[3]);
        W.gforce = make_float2(d.global_force[0], d.global_force[1]);
        W.gravity = make_float2(d.gravity[0], d.gravity[1]);
        W.injectPos = make_float2(0.0f, 0.0f);
        W.injectObject = d.inject_object;
        for (uint32_t i = 0; i < in.bubble_count; ++i) {
            const bp_bubble& b = in.bubbles[i];
            uint64_t g = ob + i;
            pos[g] = make_float2(b.center[0], b.center[1]);
            start[g] = make_float2(b.previous_center[0], b.previous_center[1]);
            vel[g] = make_float2(b.velocity[0], b.velocity[1]);
            rotw[g] = make_float2(b.rotation, b.angular_velocity);
            phys[g] = make_float4(b.radius, b.inverse_mass, b.contact_stiffness, b.damping);
            ids[g] = b.id;
            flags[g] = b.flags & 0xffu;
            filter[g] = make_uint2(b.category, b.mask);
            ws.hBubbles[g] = b;
        }
        for (uint32_t j = 0; j < in.segment_count; ++j) {
            const bp_segment& r = in.segments[j];
            DSegment& sg = segs[os + j];
            std::memset(&sg, 0, sizeof(sg));
            sg.a = make_float2(r.a[0], r.a[1]); sg.b = make_float2(r.b[0], r.b[1]);
            sg.prev = make_float2(r.previous_start[0], r.previous_start[1]);
            sg.outward = r.outward_sign; sg.allowed = r.allowed_side;
            sg.flags = r.flags; sg.cat = r.category; sg.mask = r.mask;
            sg.id = r.id; sg.owner = r.owner_id;
            ws.hSegIds[os + j] = r.id;
            ws.hSegLayers[os + j] = r.layer;
        }
        for (uint32_t v = 0; v < in.body_vertex_count; ++v)
            bverts[obv + v] = make_float2(in.body_vertices[2 * v], in.body_vertices[2 * v + 1]);
        for (uint64_t t = 0; t < 3ull * in.body_triangle_count; ++t) btris[3 * obt + t] = in.body_triangles[t];
        for (uint32_t b = 0; b < in.body_count; ++b) {
            const bp_body& r = in.bodies[b];
            DBody& B = bodies[obo + b];
            std::memset(&B, 0, sizeof(B));
            B.pos = make_float2(r.position[0], r.position[1]);
            B.prev = B.pos;
            B.angle = r.angle; B.prevAngle = r.angle;
            B.vel = make_float2(r.velocity[0], r.velocity[1]);
            B.omega = r.angular_velocity; B.radius = r.bounding_radius; B.coreRadius = r.core_radius;
            // rotation of the pose, computed on the host (the CPU oracle does the same)
            B.cosEnd = std::cos(r.angle); B.sinEnd = std::sin(r.angle);
            B.cosPrev = B.cosEnd; B.sinPrev = B.sinEnd;
            B.kind = r.kind; B.flags = r.flags;
            B.voff = (uint32_t)(obv + r.vertex_offset); B.vcount = r.vertex_count;
            B.toff = (uint32_t)(obt + r.triangle_offset); B.tcount = r.triangle_count;
            B.cat = r.category; B.mask = r.mask; B.id = r.id;
            // hull radius: farthest core vertex plus the core radius (pre-filter of the inside-body assertion)
            float hull = 0.0f;
            for (uint32_t v = 0; v < r.vertex_count; ++v) {
                float x = in.body_vertices[2 * (r.vertex_offset + v)], y = in.body_vertices[2 * (r.vertex_offset + v) + 1];
                hull = std::max(hull, std::sqrt(x * x + y * y));
            }
            B.pad = hull + r.core_radius;
            ws.hBodyIds[obo + b] = r.id;
            ws.hBodyLayers[obo + b] = r.layer;
        }
        for (uint32_t v = 0; v < in.field_vertex_count; ++v)
            fverts[ofv + v] = make_float2(in.field_vertices[2 * v], in.field_vertices[2 * v + 1]);
        for (uint32_t v = 0; v < in.field_object_id_count; ++v) fids[ofi + v] = in.field_object_ids[v];
        for (uint32_t f = 0; f < in.field_count; ++f) {
            const bp_force_field& r = in.fields[f];
            DField& F = fields[of + f];
            std::memset(&F, 0, sizeof(F));
            F.pos = make_float2(r.position[0], r.position[1]);
            F.cosr = std::cos(r.rotation); F.sinr = std::sin(r.rotation);
            F.falloff = r.falloff; F.strength = r.strength; F.radius = r.radius;
            F.dir = make_float2(r.direction[0], r.direction[1]);
            F.kind = r.kind; F.voff = (uint32_t)(ofv + r.vertex_offset); F.vcount = r.vertex_count;
            F.foff = (uint32_t)(ofi + r.filter_offset); F.fcount = r.filter_count; F.hasFilter = r.has_filter;
        }
        for (uint32_t q = 0; q < in.band_count; ++q) bands[oband + q] = in.bands[q];
        for (uint32_t q = 0; q < in.motor_count; ++q) motors[omotor + q] = in.motors[q];
        if (in.joint_ranges)
            for (uint32_t e = 0; e < in.joint_entity_count; ++e)
                jranges[ojr + e] = make_uint2((uint32_t)(ojp + in.joint_ranges[2 * e]), in.joint_ranges[2 * e + 1]);
        if (in.joint_partners)
            for (uint32_t q = 0; q < in.joint_partner_count; ++q) jpartners[ojp + q] = in.joint_partners[q];
        ob += in.bubble_count; orow += (uint64_t)in.bubble_count * W.k; obrow += (uint64_t)in.body_count * W.k;
        ocon += W.contactCap; os += in.segment_count; obo += in.body_count; obv += in.body_vertex_count;
        obt += in.body_triangle_count; of += in.field_count; ofv += in.field_vertex_count; ofi += in.field_object_id_count;
        oband += in.band_count; omotor += in.motor_count;
        ojr += in.joint_ranges ? in.joint_entity_count : 0; ojp += in.joint_partners ? in.joint_partner_count : 0;
    }

    // device allocations
    cudaError_t err = cudaSuccess;
    cudaStream_t st = ctx->stream;
    DState& S = ws.S;
    ws.dWorlds = ws.alloc<DWorld>(count, err);
    ws.dReports = ws.alloc<bp_step_report>(count, err);
    ws.dAcc = ws.alloc<bp_step_report>(count, err);
    ws.dSizes = ws.alloc<uint32_t>(count, err);
    ws.dTotal = ws.alloc<unsigned long long>(1, err);
    S.worlds = ws.dWorlds;
    S.reports = ws.dReports;
    S.history = ws.alloc<float>((uint64_t)count * kFrameLimit, err);
    S.contactCount = ws.alloc<uint32_t>(count, err);
    S.pos = ws.alloc<float2>(nb, err); S.start = ws.alloc<float2>(nb, err); S.vel = ws.alloc<float2>(nb, err);
    S.acc = ws.alloc<float2>(nb, err); S.a0 = ws.alloc<float2>(nb, err); S.ref = ws.alloc<float2>(nb, err);
    S.rotw = ws.alloc<float2>(nb, err);
    S.phys = ws.alloc<float4>(nb, err);
    S.margin = ws.alloc<float>(nb, err);
    int64_t* dIds = ws.alloc<int64_t>(nb, err);
    S.id = dIds;
    S.flags = ws.alloc<uint32_t>(nb, err); S.result = ws.alloc<uint32_t>(nb, err);
    uint2* dFilter = ws.alloc<uint2>(nb, err);
    S.filter = dFilter;
    S.cell = ws.alloc<longlong2>(nb, err); S.acell = ws.alloc<longlong2>(nb, err);
    S.candRow = ws.alloc<uint32_t>(rows, err); S.candCount = ws.alloc<uint2>(nb, err);
    S.pairTotal = ws.alloc<uint32_t>(nb, err);
    S.adj = ws.alloc<uint32_t>(rows, err); S.deg = ws.alloc<uint32_t>(nb, err);
    S.pPos = ws.alloc<float2>(nb, err); S.pStart = ws.alloc<float2>(nb, err); S.pVel = ws.alloc<float2>(nb, err);
    S.pRotw = ws.alloc<float2>(nb, err); S.pResult = ws.alloc<uint32_t>(nb, err); S.pFlags = ws.alloc<uint32_t>(nb, err);
    DSegment* dSeg = ws.alloc<DSegment>(ns, err);
    S.seg = dSeg;
    S.body = ws.alloc<DBody>(nbo, err); S.pBody = ws.alloc<DBody>(nbo, err);
    float2* dBv = ws.alloc<float2>(nbv, err);
    S.bverts = dBv;
    uint32_t* dBt = ws.alloc<uint32_t>(3 * nbt, err);
    S.btris = dBt;
    S.bodyRow = ws.alloc<uint32_t>(brows, err); S.bodyTotal = ws.alloc<uint32_t>(nbo, err);
    S.tKeys = ws.alloc<unsigned long long>(otree, err); S.tKeysAlt = ws.alloc<unsigned long long>(otree, err);
    S.tCounts = ws.alloc<uint32_t>(16ull * otree, err); S.tNodes = ws.alloc<TreeNode>(otree, err);
    S.tLeafParent = ws.alloc<uint32_t>(otree, err); S.tVisit = ws.alloc<uint32_t>(otree, err);
    S.tValid = ws.alloc<uint32_t>(count, err);
    ws.totalTreeLeaves = otree;
    DField* dF = ws.alloc<DField>(nf, err);
    S.fields = dF;
    float2* dFv = ws.alloc<float2>(nfv, err);
    S.fverts = dFv;
    int64_t* dFi = ws.alloc<int64_t>(nfi, err);
    S.fids = dFi;
    bp_band* dBand = ws.alloc<bp_band>(nband, err);
    S.bands = dBand;
    bp_motor* dMotor = ws.alloc<bp_motor>(nmotor, err);
    S.motors = dMotor;
    uint2* dJr = ws.alloc<uint2>(njr, err);
    S.jranges = dJr;
    int64_t* dJp = ws.alloc<int64_t>(njp, err);
    S.jpartners = dJp;
    S.contacts = ws.alloc<DContact>(contacts, err);
    S.failed = ws.alloc<uint32_t>(count, err);
    S.scanA = ws.alloc<uint32_t>(nb, err); S.scanB = ws.alloc<uint32_t>(nb, err);
    // scheduling: large worlds go to the cooperative path, the others to the persistent kernel's queues
    for (uint32_t w = 0; w < count; ++w) {
        uint32_t n = ws.hWorlds[w].n;
        if (n > kCtaMaxBubbles || (ws.hWorlds[w].flags & BP_WORLD_FORCE_MULTI_CTA)) ws.largeWorlds.push_back(w);
    }
    ws.dCtaList = ws.alloc<uint32_t>(count, err);
    ws.dWarpList = ws.alloc<uint32_t>(count, err);
    ws.dQueue = ws.alloc<uint32_t>(4, err);
    ws.dQueueSingle = ws.alloc<uint32_t>(4, err);
    ws.dCandidates = ws.alloc<uint32_t>(count, err);
    S.bpose = ws.alloc<float4>(nbo, err);
    S.segBox = ws.alloc<RigidBox>(ns, err);
    S.bodyBox = ws.alloc<RigidBox>(nbo, err);
    ws.dSingle = ws.alloc<uint32_t>(count, err);
    for (uint32_t w : ws.largeWorlds) ws.largeMaxN = std::max(ws.largeMaxN, ws.hWorlds[w].n);
    ws.largeB = next_pow2(std::max<uint32_t>(2u * ws.largeMaxN, 64u));
    ws.largeBlocks = ws.largeWorlds.empty() ? 0 : large_max_blocks(kLargeThreads);
    S.gpv = ws.alloc<float>(8ull * std::max(ws.largeBlocks, 1), err);     // 2 parities x 4 regions per block
    S.gpo = ws.alloc<uint32_t>(8ull * std::max(ws.largeBlocks, 1), err);
    S.gbuckets = ws.alloc<uint32_t>(ws.largeWorlds.empty() ? 1 : ws.largeB, err);
    S.gentries = ws.alloc<uint32_t>(std::max<uint32_t>(ws.largeMaxN, 1u), err);
    // entry records of the grid, and one slot per thread of the launch (the row-term passes)
    S.grecords = ws.alloc<float4>(std::max<uint32_t>(std::max<uint32_t>(ws.largeMaxN, 1u),
                                                     (uint32_t)std::max(ws.largeBlocks, 1) * kLargeThreads), err);
    S.barrier = ws.alloc<unsigned int>(2, err);
    S.errorFlag = ws.alloc<uint32_t>(1, err);
#ifdef BP_PHASE_TIMING
    S.phaseCycles = ws.alloc<unsigned long long>((uint64_t)count * kPhaseCount, err);
#else
    S.phaseCycles = nullptr;
#endif
    if (err != cudaSuccess) return cuda_status(err);

    if (ws.measureOnly) return BP_OK;

    std::vector<uint32_t> sizes(count), identity(count);
    for (uint32_t w = 0; w < count; ++w) { sizes[w] = ws.hWorlds[w].n; identity[w] = w; }
    err = upload(ws.dWorlds, ws.hWorlds.data(), count, st);
    if (!err) err = upload(ws.dSizes, sizes.data(), count, st);
    if (!err) err = upload(ws.dSingle, identity.data(), count, st);
    if (!err) err = upload(S.pos, pos.data(), nb, st);
    if (!err) err = upload(S.pPos, pos.data(), nb, st);
    if (!err) err = upload(S.start, start.data(), nb, st);
    if (!err) err = upload(S.pStart, start.data(), nb, st);
    if (!err) err = upload(S.vel, vel.data(), nb, st);
    if (!err) err = upload(S.pVel, vel.data(), nb, st);
    if (!err) err = upload(S.rotw, rotw.data(), nb, st);
    if (!err) err = upload(S.pRotw, rotw.data(), nb, st);
    if (!err) err = upload(S.phys, phys.data(), nb, st);
    if (!err) err = upload(dIds, ids.data(), nb, st);
    if (!err) err = upload(S.flags, flags.data(), nb, st);
    if (!err) err = upload(S.pFlags, flags.data(), nb, st);
    if (!err) err = upload(dFilter, filter.data(), nb, st);
    if (!err) err = upload(dSeg, segs.data(), ns, st);
    if (!err) err = upload(S.body, bodies.data(), nbo, st);
    if (!err) err = upload(S.pBody, bodies.data(), nbo, st);
    if (!err) err = upload(dBv, bverts.data(), nbv, st);
    if (!err) err = upload(dBt, btris.data(), 3 * nbt, st);
    if (!err) err = upload(dF, fields.data(), nf, st);
    if (!err) err = upload(dFv, fverts.data(), nfv, st);
    if (!err) err = upload(dFi, fids.data(), nfi, st);
    if (!err) err = upload(dBand, bands.data(), nband, st);
    if (!err) err = upload(dMotor, motors.data(), nmotor, st);
    if (!err) err = upload(dJr, jranges.data(), njr, st);
    if (!err) err = upload(dJp, jpartners.data(), njp, st);
    if (!err) err = cudaStreamSynchronize(st);
    if (!err && !ws.planOnly) err = schedule(ws, ws.threads, ws.warpMax, ws.groupWidth);
    return cuda_status(err);
}

// Launches one step of every world of the set (or of one world when `only` < nWorlds).
// Blocks of a whole-GPU step of a world of n bubbles: about one thread per bubble (at least 8 blocks), never more
// than fit on the GPU at once. Every block takes part in every grid barrier, so blocks without bubbles only make the
// barriers slower.
// Bubbles per block of the whole-GPU team: kLargeBubblesPerBlock unless BP_LARGE_BUBBLES_PER_BLOCK overrides it (a
// tuning knob: fewer blocks make each grid barrier cheaper and each phase longer).
uint32_t large_bubbles_per_block() {
    static const uint32_t value = [] {
        const char* env = std::getenv("BP_LARGE_BUBBLES_PER_BLOCK");
        const long v = env ? std::strtol(env, nullptr, 10) : 0;
        return v >= 64 && v <= (1 << 16) ? (uint32_t)v : kLargeBubblesPerBlock;
    }();
    return value;
}

int large_blocks_for(const WorldSet& ws, uint32_t n) {
    const uint32_t per = large_bubbles_per_block();
    const int want = (int)((n + per - 1) / per);
    return std::max(1, std::min(ws.largeBlocks, std::max(want, 8)));
}

// The whole-GPU step of world w; a world that builds a tree gets the key sort's histogram memory.
cudaError_t launch_large_world(WorldSet& ws, uint32_t w, cudaStream_t st) {
    return launch_large(ws.S, w, ws.largeB, large_blocks_for(ws, ws.hWorlds[w].n), kLargeThreads,
                        ws.hWorlds[w].tree ? kRadixHistBytes : 0u, st);
}

cudaError_t launch_step(WorldSet& ws, bool perWorld, uint32_t only = 0xffffffffu) {
    cudaError_t err = cudaSuccess;
    cudaStream_t st = ws.ctx->stream;
    auto one = [&](uint32_t w) -> cudaError_t {
        const DWorld& W = ws.hWorlds[w];
        ws.launches++;
        if (W.n > kCtaMaxBubbles || (W.flags & BP_WORLD_FORCE_MULTI_CTA))
            return launch_large_world(ws, w, st);
        QueueArgs q{};
        q.queue = ws.dQueueSingle;
        q.countsOnDevice = 0u;
        q.tree = W.tree;
        uint32_t maxN = std::max<uint32_t>(W.n, 1u);
        uint32_t bytes = workspace_bytes(W.n, W.s, W.nb);
        bool warpTeam = W.n <= ws.warpMax;
        uint32_t wsWords = ws.staging && bytes <= (warpTeam ? kWarpWorkspaceCap : kCtaWorkspaceCap) ? ((bytes + 15u) / 16u) * 4u : 0u;
        if (warpTeam) { q.warpList = ws.dSingle + w; q.nWarp = 1; q.warpMaxN = maxN; q.warpB = grid_buckets(maxN); q.warpWsWords = wsWords; q.groupWidth = 32u; }
        else { q.ctaList = ws.dSingle + w; q.nCta = 1; q.ctaMaxN = maxN; q.ctaB = grid_buckets(maxN); q.ctaWsWords = wsWords; }
        return launch_persistent(ws.S, q, W.n <= ws.warpMax ? 32u : ws.threads, 1u, st);
    };
    if (only < ws.nWorlds) return one(only);
    if (perWorld) {
        for (uint32_t w = 0; w < ws.nWorlds && err == cudaSuccess; ++w) err = one(w);
        return err;
    }
    if (ws.queue.nCta + ws.queue.nWarp) {
        ws.launches++;
        err = launch_persistent(ws.S, ws.queue, ws.threads, ws.blocks, st);
    }
    for (uint32_t w : ws.largeWorlds) {
        if (err != cudaSuccess) break;
        ws.launches++;
        err = launch_large_world(ws, w, st);
    }
    return err;
}

// Snapshot / restore of the dynamic state (for the autotuner's trial steps).
std::vector<std::pair<void*, size_t>> persistent_parts(WorldSet& ws) {
    DState& S = ws.S;
    uint64_t nb = ws.totalBubbles;
    // order of PersistentPart
    return {{S.pos, nb * 8}, {S.start, nb * 8}, {S.vel, nb * 8}, {S.acc, nb * 8}, {S.rotw, nb * 8},
            {S.flags, nb * 4}, {S.result, nb * 4}, {S.pPos, nb * 8}, {S.pStart, nb * 8}, {S.pVel, nb * 8},
            {S.pRotw, nb * 8}, {S.pResult, nb * 4}, {S.pFlags, nb * 4}, {S.body, ws.totalBodies * sizeof(DBody)},
            {S.pBody, ws.totalBodies * sizeof(DBody)}, {S.failed, ws.nWorlds * 4ull}};
}

cudaError_t take_snapshot(WorldSet& ws, Snapshot& snap) {
    snap.parts = persistent_parts(ws);
    cudaError_t err = cudaSuccess;
    for (auto& p : snap.parts) {
        void* c = nullptr;
        if (p.second) {
            err = cudaMalloc(&c, p.second);
            if (!err) err = cudaMemcpyAsync(c, p.first, p.second, cudaMemcpyDeviceToDevice, ws.ctx->stream);
        }
        snap.copies.push_back(c);
        if (err) return err;
    }
    return err;
}
cudaError_t restore_snapshot(WorldSet& ws, Snapshot& snap) {
    cudaError_t err = cudaSuccess;
    for (size_t q = 0; q < snap.parts.size() && !err; ++q)
        if (snap.copies[q]) err = cudaMemcpyAsync(snap.parts[q].first, snap.copies[q], snap.parts[q].second,
                                                  cudaMemcpyDeviceToDevice, ws.ctx->stream);
    return err;
}
void free_snapshot(Snapshot& snap) {
    for (void* c : snap.copies)
        if (c) cudaFree(c);
    snap.copies.clear();
}

// Project autotuner: times one step of the whole batch for each (block width, warp-team threshold) candidate from the
// same saved state and keeps the fastest; the state is restored afterwards so tuning does not advance the simulation.
cudaError_t autotune(WorldSet& ws) {
    if (ws.tuned) return cudaSuccess;
    ws.tuned = true;
    if (ws.fixedThreads) return cudaSuccess;
    Snapshot snap;
    cudaError_t err = take_snapshot(ws, snap);
    cudaStream_t st = ws.ctx->stream;
    // block width x group-queue threshold x group width; combinations whose group grids do not fit are skipped
    const uint32_t widths[] = {256, 512};
    const uint32_t warpMaxes[] = {0, 64, 128, 256, 512, 1024};
    const uint32_t groupWidths[] = {32, 64, 128};
    float best = 1e30f;
    uint32_t bestT = ws.threads, bestW = ws.warpMax, bestG = ws.groupWidth;
    for (uint32_t t : widths) {
        for (uint32_t wm : warpMaxes) {
            for (uint32_t gw : groupWidths) {
                uint32_t cap = 0;
                if (err) break;
                if (wm == 0u && gw != 32u) continue;  // no group queue: the group width does not matter
                if (wm && !group_layout(t, gw, wm, &cap)) continue;
                err = schedule(ws, t, wm, gw);
                for (int rep = 0; rep < 2 && !err; ++rep) {  // the first run warms up
                    err = restore_snapshot(ws, snap);
                    if (err) break;
                    cudaEventRecord(ws.ctx->start, st);
                    err = launch_persistent(ws.S, ws.queue, ws.threads, ws.blocks, st);
                    cudaEventRecord(ws.ctx->stop, st);
                    if (!err) err = cudaEventSynchronize(ws.ctx->stop);
                    float ms = 0.0f;
                    cudaEventElapsedTime(&ms, ws.ctx->start, ws.ctx->stop);
                    if (!err && rep == 1 && ms < best) { best = ms; bestT = t; bestW = wm; bestG = gw; }
                }
            }
        }
    }
    if (!err) err = schedule(ws, bestT, bestW, bestG);
    cudaError_t rerr = restore_snapshot(ws, snap);
    if (!rerr) rerr = cudaStreamSynchronize(st);
    free_snapshot(snap);
    return err ? err : rerr;
}

int read_reports(WorldSet& ws, bp_step_report* out, uint32_t count) {
    cudaError_t err = cudaMemcpyAsync(out, ws.dReports, count * sizeof(bp_step_report), cudaMemcpyDeviceToHost, ws.ctx->stream);
    if (!err) err = cudaStreamSynchronize(ws.ctx->stream);
    return cuda_status(err);
}

int step_set(WorldSet& ws, uint32_t steps, bp_step_report* reports, bool perWorld, bool useGraph, bool perStepReports) {
    if (ws.inflight) return BP_E_INFLIGHT;
    ws.inflight = true;
    struct Clear { bool& f; ~Clear() { f = false; } } clear{ws.inflight};
    DeviceGuard guard(ws.ctx->device);
    cudaStream_t st = ws.ctx->stream;
    cudaError_t err = cudaSuccess;
    if ((ws.flags & BP_BATCH_AUTOTUNE) && !ws.tuned && !perWorld) {
        err = autotune(ws);
        if (err) return cuda_status(err);
    }
    err = cudaMemsetAsync(ws.dAcc, 0, ws.nWorlds * sizeof(bp_step_report), st);
    if (!err) err = cudaMemsetAsync(ws.dTotal, 0, sizeof(unsigned long long), st);
    if (err) return cuda_status(err);
    bool graphed = useGraph && !perWorld && ws.largeWorlds.empty();
    if (graphed && !ws.graph) {
        cudaGraph_t g = nullptr;
        err = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
        if (!err) {
            uint64_t before = ws.launches;
            cudaError_t le = launch_step(ws, false);
            le = le ? le : launch_accumulate(ws.dReports, ws.dAcc, ws.dSizes, ws.dTotal, ws.nWorlds, st);
            le = le ? le : launch_schedule(ws.S, ws.dCandidates, ws.nCandidates, ws.warpMax, kWarpSubsteps, ws.dCtaList,
                                           ws.dWarpList, ws.dQueue, st);
            err = cudaStreamEndCapture(st, &g);
            ws.launches = before;
            if (!err) err = le;
        }
        if (!err) err = cudaGraphInstantiate(&ws.graph, g, 0);
        if (g) cudaGraphDestroy(g);
        if (err) return cuda_status(err);
    }
    uint32_t launchesPerStep = (ws.queue.nCta + ws.queue.nWarp ? 1u : 0u) + (uint32_t)ws.largeWorlds.size();
    int status = BP_OK;
    cudaEventRecord(ws.ctx->start, st);
    for (uint32_t s = 0; s < steps && !err; ++s) {
        if (graphed) {
            err = cudaGraphLaunch(ws.graph, st);
            ws.launches += launchesPerStep;
        } else {
            err = launch_step(ws, perWorld);
            if (!err) err = launch_accumulate(ws.dReports, ws.dAcc, ws.dSizes, ws.dTotal, ws.nWorlds, st);
            if (!err && !perWorld)
                err = launch_schedule(ws.S, ws.dCandidates, ws.nCandidates, ws.warpMax, kWarpSubsteps, ws.dCtaList,
                                      ws.dWarpList, ws.dQueue, st);
        }
        if (perStepReports && reports && !err) {
            int rs = read_reports(ws, reports + (uint64_t)s * ws.nWorlds, ws.nWorlds);
            if (rs) return rs;
            for (uint32_t w = 0; w < ws.nWorlds; ++w)
                if (reports[(uint64_t)s * ws.nWorlds + w].status != BP_OK) status = reports[(uint64_t)s * ws.nWorlds + w].status;
            if (status != BP_OK && ws.nWorlds == 1) break;
        }
    }
    cudaEventRecord(ws.ctx->stop, st);
    if (err) return cuda_status(err);
    unsigned long long total = 0;
    err = cudaMemcpyAsync(&total, ws.dTotal, sizeof(total), cudaMemcpyDeviceToHost, st);
    if (!err && reports && !perStepReports) err = cudaMemcpyAsync(reports, ws.dAcc, ws.nWorlds * sizeof(bp_step_report), cudaMemcpyDeviceToHost, st);
    if (!err) err = cudaStreamSynchronize(st);
    if (!err) {
        uint32_t flag = 0;
        cudaMemcpy(&flag, ws.S.errorFlag, sizeof(flag), cudaMemcpyDeviceToHost);
        if (flag) {
            cudaMemset(ws.S.barrier, 0, 2 * sizeof(unsigned int));
            cudaMemset(ws.S.errorFlag, 0, sizeof(uint32_t));
            return BP_E_TIMEOUT;
        }
    }
    if (err) return cuda_status(err);
    ws.bubbleSubsteps += total;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, ws.ctx->start, ws.ctx->stop);
    if (reports && !perStepReports)
        for (uint32_t w = 0; w < ws.nWorlds; ++w) {
            reports[w].gpu_ms = ms;
            if (reports[w].status != BP_OK && status == BP_OK) status = reports[w].status;
        }
    return status;
}

int read_bubbles(WorldSet& ws, uint32_t world, bp_bubble* out, uint32_t capacity, uint32_t* count) {
    if (world >= ws.nWorlds) return BP_E_INVALID;
    const DWorld& W = ws.hWorlds[world];
    if (count) *count = W.n;
    if (!out) return BP_OK;
    DeviceGuard guard(ws.ctx->device);
    uint32_t m = std::min(W.n, capacity);
    std::vector<float2> pos(m), start(m), vel(m), rotw(m);
    std::vector<uint32_t> result(m), flags(m);
    cudaError_t err = cudaSuccess;
    if (m) {
        err = cudaMemcpy(pos.data(), ws.S.pPos + W.boff, m * 8, cudaMemcpyDeviceToHost);
        if (!err) err = cudaMemcpy(start.data(), ws.S.pStart + W.boff, m * 8, cudaMemcpyDeviceToHost);
        if (!err) err = cudaMemcpy(vel.data(), ws.S.pVel + W.boff, m * 8, cudaMemcpyDeviceToHost);
        if (!err) err = cudaMemcpy(rotw.data(), ws.S.pRotw + W.boff, m * 8, cudaMemcpyDeviceToHost);
        if (!err) err = cudaMemcpy(result.data(), ws.S.pResult + W.boff, m * 4, cudaMemcpyDeviceToHost);
        if (!err) err = cudaMemcpy(flags.data(), ws.S.pFlags + W.boff, m * 4, cudaMemcpyDeviceToHost);
    }
    if (err) return cuda_status(err);
    for (uint32_t i = 0; i < m; ++i) {
        bp_bubble b = ws.hBubbles[W.boff + i];
        b.center[0] = pos[i].x; b.center[1] = pos[i].y;
        b.previous_center[0] = start[i].x; b.previous_center[1] = start[i].y;
        b.velocity[0] = vel[i].x; b.velocity[1] = vel[i].y;
        b.rotation = rotw[i].x; b.angular_velocity = rotw[i].y;
        b.region_result = result[i];
        b.flags = flags[i] & 0xffu;
        out[i] = b;
    }
    return BP_OK;
}

}  // namespace bp_host

static void context_free(bp_context* c) {
    DeviceGuard guard(c->device);
    cudaStreamSynchronize(c->stream);
    cudaEventDestroy(c->start);
    cudaEventDestroy(c->stop);
    cudaStreamDestroy(c->stream);
    delete c;
}

// The context lives until it is released and every world / batch created on it is destroyed, whatever the order of
// the destroy calls.
void bp_host::context_unref(bp_context* c) {
    if (--c->refs == 0 && c->released) context_free(c);
}

// ================================================================================================================
// C ABI
// ================================================================================================================
extern "C" {

int bp_abi_version(void) { return BP_ABI_VERSION; }

const char* bp_status_string(int status) {
    switch (status) {
        case BP_OK: return "ok";
        case BP_E_INVALID: return "invalid snapshot";
        case BP_E_SUBSTEP_LIMIT: return "substep limit exceeded";
        case BP_E_NONFINITE: return "non-finite values";
        case BP_E_CONTACT_VIOLATION: return "contact violation";
        case BP_E_INFLIGHT: return "frame in flight";
        case BP_E_TIMEOUT: return "bounded device wait timed out";
        case BP_E_CUDA: return "CUDA command failed";
        case BP_E_CAPACITY: return "capacity overflow";
        case BP_E_UNAVAILABLE: return "CUDA device unavailable";
        case BP_E_ALLOC: return "allocation failed";
        case BP_E_WORLD_FAILED: return "world failed in an earlier step";
        default: return "unknown status";
    }
}

int bp_device_available(int device) {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) return BP_E_UNAVAILABLE;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return BP_E_UNAVAILABLE;
    return prop.major >= 10 ? BP_OK : BP_E_UNAVAILABLE;
}

int bp_context_create(int device, uint32_t flags, bp_context** out) {
    (void)flags;
    if (!out) return BP_E_INVALID;
    int st = bp_device_available(device);
    if (st != BP_OK) return st;
    DeviceGuard guard(device);
    bp_context* c = new (std::nothrow) bp_context();
    if (!c) return BP_E_ALLOC;
    c->device = device;
    cudaError_t err = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (!err) err = cudaEventCreate(&c->start);
    if (!err) err = cudaEventCreate(&c->stop);
    if (!err) err = cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device);
    if (err) { delete c; return cuda_status(err); }
    prepare_kernels();
    *out = c;
    return BP_OK;
}

int bp_context_destroy(bp_context* c) {
    if (!c) return BP_OK;
    c->released = true;
    if (c->refs == 0) context_free(c);
    return BP_OK;
}

int bp_world_create(bp_context* context, const bp_world_desc* desc, const bp_world_input* input, bp_world** out) {
    if (!context || !desc || !input || !out) return BP_E_INVALID;
    bp_world* w = new (std::nothrow) bp_world();
    if (!w) return BP_E_ALLOC;
    context->refs++;
    int st = build_set(w->set, context, 1, desc, input, true);
    if (st != BP_OK) { delete w; context_unref(context); return st; }
    *out = w;
    return BP_OK;
}

int bp_world_destroy(bp_world* world) {
    if (!world) return BP_OK;
    bp_context* c = world->set.ctx;
    {
        DeviceGuard guard(c->device);
        cudaStreamSynchronize(c->stream);
        delete world;
    }
    context_unref(c);
    return BP_OK;
}

int bp_world_write_bubbles(bp_world* world, const bp_bubble* bubbles, uint32_t count) {
    if (!world || (!bubbles && count)) return BP_E_INVALID;
    WorldSet& ws = world->set;
    if (count != ws.hWorlds[0].n) return BP_E_INVALID;
    for (uint32_t i = 0; i < count; ++i)
        if (bubbles[i].id != ws.hBubbles[i].id) return BP_E_INVALID;
    DeviceGuard guard(ws.ctx->device);
    std::vector<float2> pos(count), start(count), vel(count), rotw(count);
    std::vector<float4> phys(count);
    std::vector<uint32_t> flags(count);
    std::vector<uint2> filter(count);
    for (uint32_t i = 0; i < count; ++i) {
        const bp_bubble& b = bubbles[i];
        pos[i] = make_float2(b.center[0], b.center[1]);
        start[i] = make_float2(b.previous_center[0], b.previous_center[1]);
        vel[i] = make_float2(b.velocity[0], b.velocity[1]);
        rotw[i] = make_float2(b.rotation, b.angular_velocity);
        phys[i] = make_float4(b.radius, b.inverse_mass, b.contact_stiffness, b.damping);
        flags[i] = b.flags & 0xffu;
        filter[i] = make_uint2(b.category, b.mask);
        ws.hBubbles[i] = b;
    }
    cudaStream_t st = ws.ctx->stream;
    cudaError_t err = upload(ws.S.pos, pos.data(), count, st);
    if (!err) err = upload(ws.S.pPos, pos.data(), count, st);
    if (!err) err = upload(ws.S.start, start.data(), count, st);
    if (!err) err = upload(ws.S.pStart, start.data(), count, st);
    if (!err) err = upload(ws.S.vel, vel.data(), count, st);
    if (!err) err = upload(ws.S.pVel, vel.data(), count, st);
    if (!err) err = upload(ws.S.rotw, rotw.data(), count, st);
    if (!err) err = upload(ws.S.pRotw, rotw.data(), count, st);
    if (!err) err = upload(ws.S.phys, phys.data(), count, st);
    if (!err) err = upload(ws.S.flags, flags.data(), count, st);
    if (!err) err = upload(ws.S.pFlags, flags.data(), count, st);
    if (!err) err = upload((uint2*)ws.S.filter, filter.data(), count, st);
    if (!err) err = cudaMemsetAsync(ws.S.failed, 0, sizeof(uint32_t), st);
    if (!err) err = cudaStreamSynchronize(st);
    return cuda_status(err);
}

int bp_world_set_diagnostics(bp_world* world, const bp_world_diagnostics* d) {
    if (!world || !d) return BP_E_INVALID;
    WorldSet& ws = world->set;
    ws.hWorlds[0].injectSubstep = d->inject_substep;
    ws.hWorlds[0].injectPos = make_float2(d->inject_position[0], d->inject_position[1]);
    DeviceGuard guard(ws.ctx->device);
    cudaError_t err = upload(ws.dWorlds, ws.hWorlds.data(), 1, ws.ctx->stream);
    if (!err) err = cudaStreamSynchronize(ws.ctx->stream);
    return cuda_status(err);
}

int bp_world_step(bp_world* world, uint32_t steps, bp_step_report* reports) {
    if (!world) return BP_E_INVALID;
    WorldSet& ws = world->set;
    std::vector<bp_step_report> local(steps ? steps : 1);
    bp_step_report* out = reports ? reports : local.data();
    std::memset(out, 0, sizeof(bp_step_report) * steps);
    DeviceGuard guard(ws.ctx->device);
    cudaStream_t st = ws.ctx->stream;
    int status = BP_OK;
    for (uint32_t s = 0; s < steps; ++s) {
        cudaEventRecord(ws.ctx->start, st);
        cudaError_t err = launch_step(ws, true);
        cudaEventRecord(ws.ctx->stop, st);
        if (err) return cuda_status(err);
        int rs = read_reports(ws, out + s, 1);
        if (rs) return rs;
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, ws.ctx->start, ws.ctx->stop);
        out[s].gpu_ms = ms;
        uint32_t flag = 0;
        cudaMemcpy(&flag, ws.S.errorFlag, sizeof(flag), cudaMemcpyDeviceToHost);
        if (flag) {
            out[s].status = BP_E_TIMEOUT;
            cudaMemset(ws.S.barrier, 0, 2 * sizeof(unsigned int));
            cudaMemset(ws.S.errorFlag, 0, sizeof(uint32_t));
            return BP_E_TIMEOUT;
        }
        ws.bubbleSubsteps += (uint64_t)out[s].substep_count * ws.hWorlds[0].n;
        if (ws.sensorCount && out[s].status == BP_OK) {
            err = launch_sensors(ws.S, ws.hWorlds[0], ws.dSensors, ws.sensorCount, ws.dSensorVerts, ws.dSensorAllowed,
                                 ws.dSensorState, ws.dSensorKinds, ws.dSensorEvents, ws.sensorEventCapacity, ws.dSensorCount, st);
            if (err) return cuda_status(err);
        }
        status = out[s].status;
        if (status != BP_OK) break;
    }
    return status;
}

int bp_world_read_bubbles(bp_world* world, bp_bubble* out, uint32_t capacity, uint32_t* count) {
    if (!world) return BP_E_INVALID;
    return read_bubbles(world->set, 0, out, capacity, count);
}

int bp_world_read_contacts(bp_world* world, bp_contact* out, uint32_t capacity, uint32_t* count) {
    if (!world) return BP_E_INVALID;
    WorldSet& ws = world->set;
    DeviceGuard guard(ws.ctx->device);
    uint32_t c = 0;
    cudaError_t err = cudaMemcpy(&c, ws.S.contactCount, sizeof(c), cudaMemcpyDeviceToHost);
    if (err) return cuda_status(err);
    if (count) *count = c;
    if (!out) return BP_OK;
    uint32_t m = std::min(c, capacity);
    std::vector<DContact> rec(m);
    if (m) err = cudaMemcpy(rec.data(), ws.S.contacts + ws.hWorlds[0].contactOff, m * sizeof(DContact), cudaMemcpyDeviceToHost);
    if (err) return cuda_status(err);
    for (uint32_t q = 0; q < m; ++q) {
        bp_contact& o = out[q];
        std::memset(&o, 0, sizeof(o));
        const DContact& r = rec[q];
        o.participants[0] = ws.hBubbles[r.a].id;
        o.participants[1] = r.kind == 0 ? ws.hBubbles[r.other].id : ws.hSegIds[ws.hWorlds[0].soff + r.other];
        o.kind = r.kind;
        o.feature = r.feature;
        o.normal[0] = r.normal.x; o.normal[1] = r.normal.y;
        o.point[0] = r.point.x; o.point[1] = r.point.y;
        o.impulse = r.impulse;
        o.penetration = r.penetration;
        o.allowed_side = r.allowed;
    }
    return BP_OK;
}

int bp_world_read_candidates(bp_world* world, bp_candidate_key* out, uint32_t capacity, uint32_t* count) {
    if (!world) return BP_E_INVALID;
    WorldSet& ws = world->set;
    const DWorld& W = ws.hWorlds[0];
    DeviceGuard guard(ws.ctx->device);
    std::vector<uint32_t> rows((uint64_t)W.n * W.k), brows((uint64_t)W.nb * W.k), btotal(W.nb), flags(W.n);
    std::vector<uint2> cc(W.n);
    cudaError_t err = cudaSuccess;
    if (W.n) err = cudaMemcpy(rows.data(), ws.S.candRow + W.rowOff, rows.size() * 4, cudaMemcpyDeviceToHost);
    if (!err && W.n) err = cudaMemcpy(cc.data(), ws.S.candCount + W.boff, W.n * sizeof(uint2), cudaMemcpyDeviceToHost);
    if (!err && W.n) err = cudaMemcpy(flags.data(), ws.S.flags + W.boff, W.n * 4, cudaMemcpyDeviceToHost);
    if (!err && W.nb) err = cudaMemcpy(brows.data(), ws.S.bodyRow + W.bodyRowOff, brows.size() * 4, cudaMemcpyDeviceToHost);
    if (!err && W.nb) err = cudaMemcpy(btotal.data(), ws.S.bodyTotal + W.bodyOff, W.nb * 4, cudaMemcpyDeviceToHost);
    if (err) return cuda_status(err);
    std::vector<bp_candidate_key> keys;
    for (uint32_t i = 0; i < W.n; ++i) {
        if (flags[i] & kRemoved) continue;
        for (uint32_t e = 0; e < cc[i].x + cc[i].y; ++e) {
            uint32_t v = rows[(uint64_t)i * W.k + e];
            if (e < cc[i].x) keys.push_back({0u, 0u, ws.hBubbles[i].id, ws.hBubbles[v].id});
            else keys.push_back({1u, 0u, ws.hBubbles[i].id, ws.hSegIds[W.soff + (v & kIndexMask)]});
        }
    }
    for (uint32_t b = 0; b < W.nb; ++b)
        for (uint32_t e = 0; e < std::min(btotal[b], W.k); ++e)
            keys.push_back({2u, 0u, ws.hBubbles[brows[(uint64_t)b * W.k + e]].id, ws.hBodyIds[W.bodyOff + b]});
    std::sort(keys.begin(), keys.end(), [](const bp_candidate_key& a, const bp_candidate_key& b) {
        if (a.kind != b.kind) return a.kind < b.kind;
        if (a.first != b.first) return a.first < b.first;
        return a.second < b.second;
    });
    if (count) *count = (uint32_t)keys.size();
    if (out)
        for (uint32_t q = 0; q < keys.size() && q < capacity; ++q) out[q] = keys[q];
    return BP_OK;
}

int bp_world_read_cells(bp_world* world, int64_t* out, uint32_t capacity, uint32_t* count) {
    if (!world) return BP_E_INVALID;
    WorldSet& ws = world->set;
    const DWorld& W = ws.hWorlds[0];
    if (count) *count = W.n;
    if (!out) return BP_OK;
    DeviceGuard guard(ws.ctx->device);
    uint32_t m = std::min(W.n, capacity);
    cudaError_t err = m ? cudaMemcpy(out, ws.S.cell + W.boff, m * sizeof(longlong2), cudaMemcpyDeviceToHost) : cudaSuccess;
    return cuda_status(err);
}

int bp_world_read_rigid_keys(bp_world* world, uint64_t* out, uint32_t capacity, uint32_t* count) {
    if (!world) return BP_E_INVALID;
    WorldSet& ws = world->set;
    const DWorld& W = ws.hWorlds[0];
    DeviceGuard guard(ws.ctx->device);
    uint32_t valid = 0;
    cudaError_t err = W.tree ? cudaMemcpy(&valid, ws.S.tValid, sizeof(valid), cudaMemcpyDeviceToHost) : cudaSuccess;
    if (err) return cuda_status(err);
    const uint32_t leaves = valid ? W.s + W.nb : 0u;
    if (count) *count = leaves;
    if (!out) return BP_OK;
    uint32_t m = std::min(leaves, capacity);
    err = m ? cudaMemcpy(out, ws.S.tKeys + W.treeOff, m * sizeof(uint64_t), cudaMemcpyDeviceToHost) : cudaSuccess;
    return cuda_status(err);
}

// The world's table of contour directions for sample counts up to `stride` (grown to the largest stride asked for).
static cudaError_t contour_dirs(WorldSet& ws, uint32_t stride, const float2** out) {
    if (stride > ws.contourDirStride) {
        const std::vector<float2> dirs = contour_directions(stride);
        float2* d = nullptr;
        cudaError_t err = cudaMalloc(&d, dirs.size() * sizeof(float2));
        if (!err) err = cudaMemcpy(d, dirs.data(), dirs.size() * sizeof(float2), cudaMemcpyHostToDevice);
        if (err) {
            cudaFree(d);
            return err;
        }
        cudaFree(ws.dContourDirs);
        ws.dContourDirs = d;
        ws.contourDirStride = stride;
    }
    *out = ws.dContourDirs;
    return cudaSuccess;
}

int bp_world_contours(bp_world* world, const bp_contour_config* config, float* points_xy, uint32_t* counts,
                      float* level, float* shape, uint32_t* stride_out, float* gpu_ms) {
    if (!world || !config) return BP_E_INVALID;
    const float maxEdge = config->max_edge, tension = config->surface_tension, clearance = config->clearance;
    if (!(maxEdge > 0.0f) || !std::isfinite(maxEdge) || !(tension >= 0.0f) || !std::isfinite(tension) ||
        !(clearance >= 0.0f) || !std::isfinite(clearance))
        return BP_E_INVALID;
    WorldSet& ws = world->set;
    const DWorld& W = ws.hWorlds[0];
    uint32_t need = 64u;
    for (uint32_t i = 0; i < W.n; ++i) need = std::max(need, contour_samples(ws.hBubbles[W.boff + i].radius, maxEdge, 0xffffffffu));
    const uint32_t stride = config->stride ? config->stride : need;
    if (stride_out) *stride_out = stride;
    if (stride > 1024u) return BP_E_CAPACITY;
    if (gpu_ms) *gpu_ms = 0.0f;
    if ((!points_xy && !counts && !level && !shape) || W.n == 0u) return BP_OK;
    DeviceGuard guard(ws.ctx->device);
    cudaStream_t st = ws.ctx->stream;
    const uint64_t samples = (uint64_t)W.n * stride;
    float2* dPoints = nullptr;
    uint32_t* dCounts = nullptr;
    float* dLevel = nullptr;
    float* dShape = nullptr;
    const float2* dDirs = nullptr;
    cudaError_t err = contour_dirs(ws, stride, &dDirs);
    if (!err) err = cudaMallocAsync(&dPoints, samples * sizeof(float2), st);
    if (!err) err = cudaMallocAsync(&dCounts, (size_t)W.n * sizeof(uint32_t), st);
    if (!err) err = cudaMallocAsync(&dLevel, samples * sizeof(float), st);
    if (!err) err = cudaMallocAsync(&dShape, (size_t)W.n * 6u * sizeof(float), st);
    if (!err) err = cudaEventRecord(ws.ctx->start, st);
    if (!err) err = launch_contours(ws.S, W, maxEdge, tension, clearance, stride, dDirs, dPoints, dCounts, dLevel, dShape, st);
    if (!err) err = cudaEventRecord(ws.ctx->stop, st);
    if (!err && points_xy) err = cudaMemcpyAsync(points_xy, dPoints, samples * sizeof(float2), cudaMemcpyDeviceToHost, st);
    if (!err && counts) err = cudaMemcpyAsync(counts, dCounts, (size_t)W.n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    if (!err && level) err = cudaMemcpyAsync(level, dLevel, samples * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (!err && shape) err = cudaMemcpyAsync(shape, dShape, (size_t)W.n * 6u * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (!err) err = cudaStreamSynchronize(st);
    if (!err && gpu_ms) cudaEventElapsedTime(gpu_ms, ws.ctx->start, ws.ctx->stop);
    for (void* p : {(void*)dPoints, (void*)dCounts, (void*)dLevel, (void*)dShape})
        if (p) cudaFreeAsync(p, st);
    cudaError_t fin = cudaStreamSynchronize(st);
    return cuda_status(err ? err : fin);
}

int bp_world_hit_test(bp_world* world, const bp_contour_config* config, const float* points_xy, uint32_t count,
                      int64_t* ids, int32_t* layers, uint32_t* found) {
    if (!world || !config || (count && (!points_xy || !ids || !layers || !found))) return BP_E_INVALID;
    uint32_t stride = 0;
    int st = bp_world_contours(world, config, nullptr, nullptr, nullptr, nullptr, &stride, nullptr);
    if (st) return st;
    if (count == 0u) return BP_OK;
    WorldSet& ws = world->set;
    const DWorld& W = ws.hWorlds[0];
    DeviceGuard guard(ws.ctx->device);
    cudaStream_t st0 = ws.ctx->stream;
    const uint64_t samples = (uint64_t)std::max(W.n, 1u) * stride;
    std::vector<uint32_t> bubbleLayers(std::max(W.n, 1u));
    for (uint32_t i = 0; i < W.n; ++i) bubbleLayers[i] = ws.hBubbles[W.boff + i].layer;
    float2 *dPoints = nullptr, *dQueries = nullptr;
    uint32_t *dCounts = nullptr, *dBubbleLayers = nullptr, *dSegLayers = nullptr, *dBodyLayers = nullptr;
    uint32_t *dLayers = nullptr, *dFound = nullptr;
    float *dLevel = nullptr, *dShape = nullptr;
    long long* dIds = nullptr;
    const float2* dDirs = nullptr;
    cudaError_t err = contour_dirs(ws, stride, &dDirs);
    if (!err) err = cudaMallocAsync(&dPoints, samples * sizeof(float2), st0);
    if (!err) err = cudaMallocAsync(&dCounts, std::max(W.n, 1u) * sizeof(uint32_t), st0);
    if (!err) err = cudaMallocAsync(&dLevel, samples * sizeof(float), st0);
    if (!err) err = cudaMallocAsync(&dShape, std::max(W.n, 1u) * 6ull * sizeof(float), st0);
    if (!err) err = cudaMallocAsync(&dQueries, count * sizeof(float2), st0);
    if (!err) err = cudaMallocAsync(&dBubbleLayers, bubbleLayers.size() * sizeof(uint32_t), st0);
    if (!err) err = cudaMallocAsync(&dSegLayers, std::max(W.s, 1u) * sizeof(uint32_t), st0);
    if (!err) err = cudaMallocAsync(&dBodyLayers, std::max(W.nb, 1u) * sizeof(uint32_t), st0);
    if (!err) err = cudaMallocAsync(&dIds, count * sizeof(long long), st0);
    if (!err) err = cudaMallocAsync(&dLayers, count * sizeof(uint32_t), st0);
    if (!err) err = cudaMallocAsync(&dFound, count * sizeof(uint32_t), st0);
    if (!err) err = upload(dQueries, (const float2*)points_xy, count, st0);
    if (!err) err = upload(dBubbleLayers, bubbleLayers.data(), W.n, st0);
    if (!err) err = upload(dSegLayers, ws.hSegLayers.data() + W.soff, W.s, st0);
    if (!err) err = upload(dBodyLayers, ws.hBodyLayers.data() + W.bodyOff, W.nb, st0);
    if (!err) err = launch_contours(ws.S, W, config->max_edge, config->surface_tension, config->clearance, stride, dDirs,
                                    dPoints, dCounts, dLevel, dShape, st0);
    if (!err) err = launch_hit_test(ws.S, W, dQueries, count, dPoints, dCounts, dShape, stride, dBubbleLayers, dSegLayers,
                                    dBodyLayers, dIds, dLayers, dFound, st0);
    if (!err) err = cudaMemcpyAsync(ids, dIds, count * sizeof(long long), cudaMemcpyDeviceToHost, st0);
    if (!err) err = cudaMemcpyAsync(layers, dLayers, count * sizeof(uint32_t), cudaMemcpyDeviceToHost, st0);
    if (!err) err = cudaMemcpyAsync(found, dFound, count * sizeof(uint32_t), cudaMemcpyDeviceToHost, st0);
    if (!err) err = cudaStreamSynchronize(st0);
    for (void* p : {(void*)dPoints, (void*)dCounts, (void*)dLevel, (void*)dShape, (void*)dQueries, (void*)dBubbleLayers,
                    (void*)dSegLayers, (void*)dBodyLayers, (void*)dIds, (void*)dLayers, (void*)dFound})
        if (p) cudaFreeAsync(p, st0);
    cudaError_t fin = cudaStreamSynchronize(st0);
    return cuda_status(err ? err : fin);
}

int bp_world_set_sensors(bp_world* world, const bp_sensor* sensors, uint32_t count, const float* vertices_xy,
                         uint32_t vertex_count, const uint8_t* allowed, const uint8_t* overlap_state) {
    if (!world || (count && !sensors) || (vertex_count && !vertices_xy)) return BP_E_INVALID;
    for (uint32_t k = 0; k < count; ++k) {
        const bp_sensor& r = sensors[k];
        if ((uint64_t)r.vertex_offset + r.vertex_count > vertex_count || r.vertex_count == 1u || r.vertex_count == 2u ||
            !std::isfinite(r.position[0]) || !std::isfinite(r.position[1]) || !std::isfinite(r.angle) ||
            !(r.radius >= 0.0f))
            return BP_E_INVALID;
    }
    WorldSet& ws = world->set;
    DeviceGuard guard(ws.ctx->device);
    cudaStream_t st = ws.ctx->stream;
    cudaError_t err = cudaStreamSynchronize(st);
    for (void* p : ws.sensorAllocations) cudaFree(p);
    ws.sensorAllocations.clear();
    ws.sensorCount = 0;
    if (err) return cuda_status(err);
    const uint64_t objects = (uint64_t)ws.hWorlds[0].n + ws.hWorlds[0].nb;
    const uint64_t pairs = (uint64_t)count * objects;
    if (pairs > 0xffffffffull) return BP_E_CAPACITY;
    auto take = [&](size_t bytes) -> void* {
        void* p = nullptr;
        if (err == cudaSuccess) err = cudaMalloc(&p, std::max<size_t>(bytes, 16));
        if (err == cudaSuccess) { ws.sensorAllocations.push_back(p); err = cudaMemsetAsync(p, 0, std::max<size_t>(bytes, 16), st); }
        return p;
    };
    ws.dSensors = take(count * sensor_record_bytes());
    ws.dSensorVerts = (float2*)take(vertex_count * sizeof(float2));
    ws.dSensorAllowed = allowed ? (uint8_t*)take(pairs) : nullptr;
    ws.dSensorState = (uint8_t*)take(pairs);
    ws.dSensorKinds = (uint8_t*)take(pairs);
    ws.dSensorEvents = (bp_sensor_event*)take(pairs * sizeof(bp_sensor_event));
    ws.dSensorCount = (uint32_t*)take(sizeof(uint32_t));
    if (err) return cuda_status(err);
    std::vector<unsigned char> records(count * sensor_record_bytes());
    for (uint32_t k = 0; k < count; ++k) sensor_to_device(sensors[k], records.data() + k * sensor_record_bytes());
    if (count) err = cudaMemcpyAsync(ws.dSensors, records.data(), records.size(), cudaMemcpyHostToDevice, st);
    if (!err && vertex_count) err = cudaMemcpyAsync(ws.dSensorVerts, vertices_xy, vertex_count * sizeof(float2), cudaMemcpyHostToDevice, st);
    if (!err && allowed && pairs) err = cudaMemcpyAsync(ws.dSensorAllowed, allowed, pairs, cudaMemcpyHostToDevice, st);
    if (!err && overlap_state && pairs)
        err = cudaMemcpyAsync(ws.dSensorState, overlap_state, pairs, cudaMemcpyHostToDevice, st);
    if (!err) err = cudaStreamSynchronize(st);
    if (err) return cuda_status(err);
    ws.sensorCount = count;
    ws.sensorEventCapacity = (uint32_t)pairs;
    return BP_OK;
}

int bp_world_read_sensor_events(bp_world* world, bp_sensor_event* out, uint32_t capacity, uint32_t* count) {
    if (!world) return BP_E_INVALID;
    WorldSet& ws = world->set;
    if (!ws.sensorCount) {
        if (count) *count = 0;
        return BP_OK;
    }
    DeviceGuard guard(ws.ctx->device);
    uint32_t c = 0;
    cudaError_t err = cudaStreamSynchronize(ws.ctx->stream);  // the last step's sensor kernels ran on it
    if (!err) err = cudaMemcpy(&c, ws.dSensorCount, sizeof(c), cudaMemcpyDeviceToHost);
    if (err) return cuda_status(err);
    if (count) *count = c;
    const uint32_t m = std::min(std::min(c, capacity), ws.sensorEventCapacity);
    if (out && m) err = cudaMemcpy(out, ws.dSensorEvents, m * sizeof(bp_sensor_event), cudaMemcpyDeviceToHost);
    return cuda_status(err);
}

// ---- contact events ---------------------------------------------------------------------------------------------

}  // extern "C"

namespace {
// Grows the history buffers to hold `keys` pair keys, keeping the current history.
cudaError_t history_reserve(WorldSet::EventState& ev, uint32_t keys) {
    if (keys <= ev.historyCap) return cudaSuccess;
    const uint32_t cap = std::max({keys, 2u * ev.historyCap, 256u});
    unsigned long long* fresh[2] = {nullptr, nullptr};
    cudaError_t err = cudaMalloc(&fresh[0], 2ull * cap * sizeof(unsigned long long));
    if (!err) err = cudaMalloc(&fresh[1], 2ull * cap * sizeof(unsigned long long));
    if (!err && ev.historyCount)
        err = cudaMemcpy(fresh[0], ev.history[ev.current], 2ull * ev.historyCount * sizeof(unsigned long long),
                         cudaMemcpyDeviceToDevice);
    if (err) {
        cudaFree(fresh[0]);
        cudaFree(fresh[1]);
        return err;
    }
    cudaFree(ev.history[0]);
    cudaFree(ev.history[1]);
    ev.history[0] = fresh[0];
    ev.history[1] = fresh[1];
    ev.current = 0;
    ev.historyCap = cap;
    return cudaSuccess;
}

size_t align256(size_t v) { return (v + 255u) & ~(size_t)255u; }
}  // namespace

extern "C" {

int bp_world_set_contact_history(bp_world* world, const int64_t* pairs, uint32_t pair_count) {
    if (!world || (!pairs && pair_count)) return BP_E_INVALID;
    WorldSet& ws = world->set;
    DeviceGuard guard(ws.ctx->device);
    std::vector<std::pair<uint64_t, uint64_t>> keys(pair_count);
    for (uint32_t q = 0; q < pair_count; ++q) {
        const uint64_t a = (uint64_t)pairs[2 * q], b = (uint64_t)pairs[2 * q + 1];
        keys[q] = a <= b ? std::make_pair(a, b) : std::make_pair(b, a);
    }
    std::sort(keys.begin(), keys.end());
    keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
    WorldSet::EventState& ev = ws.events;
    ev.historyCount = 0;
    cudaError_t err = history_reserve(ev, (uint32_t)keys.size());
    if (err) return cuda_status(err);
    std::vector<unsigned long long> flat(2 * keys.size());
    for (size_t q = 0; q < keys.size(); ++q) { flat[2 * q] = keys[q].first; flat[2 * q + 1] = keys[q].second; }
    if (!flat.empty())
        err = cudaMemcpy(ev.history[ev.current], flat.data(), flat.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice);
    if (err) return cuda_status(err);
    ev.historyCount = (uint32_t)keys.size();
    return BP_OK;
}

int bp_world_read_contact_history(bp_world* world, int64_t* pairs, uint32_t capacity, uint32_t* count) {
    if (!world) return BP_E_INVALID;
    WorldSet& ws = world->set;
    const WorldSet::EventState& ev = ws.events;
    if (count) *count = ev.historyCount;
    if (!pairs || !ev.historyCount) return BP_OK;
    DeviceGuard guard(ws.ctx->device);
    const uint32_t m = std::min(capacity, ev.historyCount);
    cudaError_t err = m ? cudaMemcpy(pairs, ev.history[ev.current], 2ull * m * sizeof(int64_t), cudaMemcpyDeviceToHost)
                        : cudaSuccess;
    return cuda_status(err);
}

int bp_world_contact_events(bp_world* world, const int64_t* interested_ids, uint32_t interested_count,
                            const int64_t* removed_ids, uint32_t removed_count, const bp_contact* extra,
                            uint32_t extra_count, float step_seconds, bp_contact_event* out, uint32_t capacity,
                            uint32_t* count) {
    if (!world || (!interested_ids && interested_count) || (!removed_ids && removed_count) ||
        (!extra && extra_count) || (!out && capacity) || !(step_seconds > 0.0f) || !std::isfinite(step_seconds))
        return BP_E_INVALID;
    WorldSet& ws = world->set;
    if (ws.inflight) return BP_E_INFLIGHT;
    DeviceGuard guard(ws.ctx->device);
    cudaStream_t st = ws.ctx->stream;
    const DWorld& W = ws.hWorlds[0];
    uint32_t deviceCount = 0;
    cudaError_t err = cudaMemcpy(&deviceCount, ws.S.contactCount, sizeof(uint32_t), cudaMemcpyDeviceToHost);
    if (err) return cuda_status(err);
    const uint32_t records = deviceCount + extra_count;
    std::vector<int64_t> interested(interested_ids, interested_ids + interested_count);
    std::vector<int64_t> removed(removed_ids, removed_ids + removed_count);
    std::sort(interested.begin(), interested.end());
    std::sort(removed.begin(), removed.end());
    WorldSet::EventState& ev = ws.events;
    err = history_reserve(ev, std::max(records, ev.historyCount));
    if (err) return cuda_status(err);
    uint32_t pow2 = 1;
    while (pow2 < records) pow2 <<= 1;
    // scratch: entries | order | heads | interested | removed | extra | events | counts
    size_t off[9];
    off[0] = 0;
    off[1] = off[0] + align256((size_t)records * event_entry_bytes());
    off[2] = off[1] + align256((size_t)pow2 * 4u);
    off[3] = off[2] + align256((size_t)records * 4u);
    off[4] = off[3] + align256((size_t)interested_count * 8u);
    off[5] = off[4] + align256((size_t)removed_count * 8u);
    off[6] = off[5] + align256((size_t)extra_count * sizeof(bp_contact));
    off[7] = off[6] + align256((size_t)capacity * sizeof(bp_contact_event));
    off[8] = off[7] + align256(2u * sizeof(uint32_t));
    if (off[8] > ev.scratchBytes) {
        cudaFree(ev.scratch);
        ev.scratch = nullptr;
        ev.scratchBytes = 0;
        err = cudaMalloc(&ev.scratch, off[8]);
        if (err) return cuda_status(err);
        ev.scratchBytes = off[8];
    }
    char* base = (char*)ev.scratch;
    if (interested_count)
        err = cudaMemcpyAsync(base + off[3], interested.data(), interested_count * 8ull, cudaMemcpyHostToDevice, st);
    if (!err && removed_count)
        err = cudaMemcpyAsync(base + off[4], removed.data(), removed_count * 8ull, cudaMemcpyHostToDevice, st);
    if (!err && extra_count)
        err = cudaMemcpyAsync(base + off[5], extra, extra_count * sizeof(bp_contact), cudaMemcpyHostToDevice, st);
    if (err) return cuda_status(err);
    uint32_t* counts = (uint32_t*)(base + off[7]);
    EventArgsHost a;
    a.records = ws.S.contacts + W.contactOff;
    a.deviceCount = deviceCount;
    a.extra = (const bp_contact*)(base + off[5]);
    a.extraCount = extra_count;
    a.ids = ws.S.id + W.boff;
    a.segments = ws.S.seg + W.soff;
    a.interested = (const int64_t*)(base + off[3]);
    a.interestedCount = interested_count;
    a.removed = (const int64_t*)(base + off[4]);
    a.removedCount = removed_count;
    a.history = ev.history[ev.current];
    a.historyCount = ev.historyCount;
    a.nextHistory = ev.history[ev.current ^ 1u];
    a.nextHistoryCount = counts + 1;
    a.step = step_seconds;
    a.entries = base + off[0];
    a.order = (uint32_t*)(base + off[1]);
    a.heads = (uint32_t*)(base + off[2]);
    a.out = (bp_contact_event*)(base + off[6]);
    a.capacity = capacity;
    a.count = counts;
    err = launch_contact_events(a, st);
    uint32_t hc[2] = {0u, 0u};
    if (!err) err = cudaMemcpyAsync(hc, counts, sizeof(hc), cudaMemcpyDeviceToHost, st);
    if (!err) err = cudaStreamSynchronize(st);
    if (!err && out && std::min(hc[0], capacity))
        err = cudaMemcpy(out, base + off[6], std::min(hc[0], capacity) * sizeof(bp_contact_event), cudaMemcpyDeviceToHost);
    if (err) return cuda_status(err);
    ev.current ^= 1u;
    ev.historyCount = hc[1];
    if (count) *count = hc[0];
    return BP_OK;
}

int bp_world_read_substeps(bp_world* world, float* out, uint32_t capacity, uint32_t* count) {
    if (!world) return BP_E_INVALID;
    WorldSet& ws = world->set;
    DeviceGuard guard(ws.ctx->device);
    bp_step_report rep;
    int st = read_reports(ws, &rep, 1);
    if (st) return st;
    uint32_t n = std::min<uint32_t>(rep.substep_count, kFrameLimit);
    if (count) *count = n;
    if (!out) return BP_OK;
    cudaError_t err = cudaMemcpy(out, ws.S.history, std::min(n, capacity) * sizeof(float), cudaMemcpyDeviceToHost);
    return cuda_status(err);
}

// ---- batch ----------------------------------------------------------------------------------------------------

int bp_batch_create(bp_context* context, uint32_t world_count, const bp_world_desc* descs, const bp_world_input* inputs,
                    const bp_batch_config* config, bp_batch** out) {
    if (!context || !descs || !inputs || !out || world_count == 0) return BP_E_INVALID;
    bp_batch* b = new (std::nothrow) bp_batch();
    if (!b) return BP_E_ALLOC;
    context->refs++;
    int st = build_set(b->set, context, world_count, descs, inputs, false);
    if (st != BP_OK) { delete b; context_unref(context); return st; }
    if (config) {
        b->set.flags = config->flags;
        if (config->flags & BP_BATCH_NO_STAGING) {
            b->set.staging = false;
            if (schedule(b->set, b->set.threads, b->set.warpMax, b->set.groupWidth) != cudaSuccess) {
                delete b;
                context_unref(context);
                return BP_E_CUDA;
            }
        }
        uint32_t t = config->threads_per_world ? config->threads_per_world : b->set.threads;
        uint32_t wm = config->warp_world_max == 0xffffffffu ? 0u : (config->warp_world_max ? config->warp_world_max : b->set.warpMax);
        uint32_t gw = config->group_width ? config->group_width : b->set.groupWidth;
        uint32_t cap = 0;
        if (t % 32u || t > 512u || wm > kCtaMaxBubbles || (gw != 32u && gw != 64u && gw != 128u && gw != 256u) ||
            gw > t || t % gw || (wm && !group_layout(t, gw, wm, &cap))) {
            delete b;
            context_unref(context);
            return BP_E_INVALID;
        }
        if (config->threads_per_world || config->warp_world_max || config->group_width) {
            b->set.fixedThreads = t;
            if (schedule(b->set, t, wm, gw) != cudaSuccess) { delete b; context_unref(context); return BP_E_CUDA; }
        }
    }
    *out = b;
    return BP_OK;
}

int bp_batch_destroy(bp_batch* batch) {
    if (!batch) return BP_OK;
    bp_context* c = batch->set.ctx;
    {
        DeviceGuard guard(c->device);
        cudaStreamSynchronize(c->stream);
        delete batch;
    }
    context_unref(c);
    return BP_OK;
}

int bp_batch_step(bp_batch* batch, uint32_t steps, bp_step_report* reports) {
    if (!batch) return BP_E_INVALID;
    WorldSet& ws = batch->set;
    bool perWorld = (ws.flags & BP_BATCH_PER_WORLD_LAUNCH) != 0;
    bool graph = (ws.flags & BP_BATCH_USE_GRAPH) != 0;
    int st = step_set(ws, steps, reports, perWorld, graph, false);
    return st;
}

int bp_batch_counters(bp_batch* batch, uint64_t* bubble_count, uint64_t* bubble_substeps, uint64_t* launches) {
    if (!batch) return BP_E_INVALID;
    if (bubble_count) *bubble_count = batch->set.totalBubbles;
    if (bubble_substeps) *bubble_substeps = batch->set.bubbleSubsteps;
    if (launches) *launches = batch->set.launches;
    return BP_OK;
}

int bp_batch_read_bubbles(bp_batch* batch, uint32_t world, bp_bubble* out, uint32_t capacity, uint32_t* count) {
    if (!batch) return BP_E_INVALID;
    return read_bubbles(batch->set, world, out, capacity, count);
}

// The device address of a caller's host buffer of float4 records when the kernels can read or write it directly:
// page-locked memory registered with CUDA (cudaHostAlloc / cudaHostRegister), 16-byte aligned; null otherwise (the
// data then goes through the device staging array with a copy).
static float4* direct_host_records(const void* p) {
    if (((uintptr_t)p & 15u) != 0u) return nullptr;
    cudaPointerAttributes attr{};
    if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (attr.type != cudaMemoryTypeHost || !attr.devicePointer || ((uintptr_t)attr.devicePointer & 15u) != 0u)
        return nullptr;
    return (float4*)attr.devicePointer;
}

int bp_batch_write_state(bp_batch* batch, const float* cv, uint64_t bubble_count) {
    if (!batch || !cv) return BP_E_INVALID;
    WorldSet& ws = batch->set;
    if (bubble_count != ws.totalBubbles) return BP_E_INVALID;
    DeviceGuard guard(ws.ctx->device);
    // page-locked records are read by the kernel across the host link: no staging copy
    if (const float4* direct = direct_host_records(cv))
        return cuda_status(launch_write_state(direct, ws.S.pos, ws.S.vel, ws.S.pPos, ws.S.pVel, bubble_count, ws.ctx->stream));
    cudaError_t err = cudaSuccess;
    if (!ws.dStaging) ws.dStaging = ws.alloc<float4>(ws.totalBubbles, err);
    if (!err) err = cudaMemcpyAsync(ws.dStaging, cv, bubble_count * sizeof(float4), cudaMemcpyHostToDevice, ws.ctx->stream);
    if (!err) err = launch_write_state(ws.dStaging, ws.S.pos, ws.S.vel, ws.S.pPos, ws.S.pVel, bubble_count, ws.ctx->stream);
    return cuda_status(err);
}

int bp_batch_read_state(bp_batch* batch, float* cv, uint64_t bubble_count) {
    if (!batch || !cv) return BP_E_INVALID;
    WorldSet& ws = batch->set;
    if (bubble_count != ws.totalBubbles) return BP_E_INVALID;
    DeviceGuard guard(ws.ctx->device);
    // page-locked records are written by the kernel across the host link: no staging copy
    if (float4* direct = direct_host_records(cv)) {
        cudaError_t err = launch_read_state(direct, ws.S.pPos, ws.S.pVel, bubble_count, ws.ctx->stream);
        if (!err) err = cudaStreamSynchronize(ws.ctx->stream);
        return cuda_status(err);
    }
    cudaError_t err = cudaSuccess;
    if (!ws.dStaging) ws.dStaging = ws.alloc<float4>(ws.totalBubbles, err);
    if (!err) err = launch_read_state(ws.dStaging, ws.S.pPos, ws.S.pVel, bubble_count, ws.ctx->stream);
    if (!err) err = cudaMemcpyAsync(cv, ws.dStaging, bubble_count * sizeof(float4), cudaMemcpyDeviceToHost, ws.ctx->stream);
    if (!err) err = cudaStreamSynchronize(ws.ctx->stream);
    return cuda_status(err);
}

int bp_batch_adjacency_entries(bp_batch* batch, uint64_t* entries) {
    if (!batch || !entries) return BP_E_INVALID;
    WorldSet& ws = batch->set;
    DeviceGuard guard(ws.ctx->device);
    cudaError_t err = cudaMemsetAsync(ws.dTotal, 0, sizeof(unsigned long long), ws.ctx->stream);
    if (!err) err = launch_sum(ws.S.deg, ws.totalBubbles, ws.dTotal, ws.ctx->stream);
    unsigned long long total = 0;
    if (!err) err = cudaMemcpyAsync(&total, ws.dTotal, sizeof(total), cudaMemcpyDeviceToHost, ws.ctx->stream);
    if (!err) err = cudaStreamSynchronize(ws.ctx->stream);
    *entries = total;
    return cuda_status(err);
}

#ifdef BP_PHASE_TIMING
// Profiling builds only: accumulated cycles per phase and world (world_count x kPhaseCount).
int bp_debug_phase_cycles(bp_batch* batch, unsigned long long* out) {
    WorldSet& ws = batch->set;
    cudaError_t err = cudaMemcpy(out, ws.S.phaseCycles, ws.nWorlds * kPhaseCount * sizeof(unsigned long long),
                                 cudaMemcpyDeviceToHost);
    return cuda_status(err);
}
#endif

int bp_batch_tuning(bp_batch* batch, uint32_t* values, uint32_t count) {
    if (!batch || !values) return BP_E_INVALID;
    const WorldSet& ws = batch->set;
    uint32_t v[6] = {ws.threads, ws.warpMax, ws.blocks, ws.queue.nCta, ws.queue.nWarp, ws.groupWidth};
    for (uint32_t q = 0; q < count && q < 6; ++q) values[q] = v[q];
    return BP_OK;
}

// ---- host helpers ----------------------------------------------------------------------------------------------

// NativeStaticPolygonEdges.segments (NativeStaticPolygonEdges.swift:16-72): signed area and collinear merge in double.
int bp_static_polygon_edges(const float* xy, uint32_t count, int64_t first_id, int64_t owner_id, uint32_t has_owner,
                            bp_segment* out, uint32_t capacity, uint32_t* out_count) {
    if (!xy && count) return BP_E_INVALID;
    struct P { float x, y; };
    std::vector<P> pts(count);
    for (uint32_t i = 0; i < count; ++i) pts[i] = {xy[2 * i], xy[2 * i + 1]};
    auto crossd = [](P u, P v) { return (double)u.x * (double)v.y - (double)u.y * (double)v.x; };
    auto subp = [](P a, P b) { return P{a.x - b.x, a.y - b.y}; };
    double area = 0.0;
    if (count >= 3)
        for (uint32_t i = 1; i + 1 < count; ++i) area += crossd(subp(pts[i], pts[0]), subp(pts[i + 1], pts[0]));
    auto segment = [&](int64_t id, P a, P b) {
        bp_segment s;
        std::memset(&s, 0, sizeof(s));
        s.id = id;
        s.owner_id = has_owner ? owner_id : 0;
        s.a[0] = a.x; s.a[1] = a.y; s.b[0] = b.x; s.b[1] = b.y;
        s.flags = has_owner ? BP_SEGMENT_HAS_OWNER : 0u;
        s.category = 1u;
        s.mask = 0xffffffffu;
        return s;
    };
    std::vector<bp_segment> result;
    if (count < 3 || area == 0.0) {
        for (uint32_t i = 0; i < count; ++i) result.push_back(segment(first_id + i, pts[i], pts[(i + 1) % count]));
    } else {
        std::vector<P> ring = pts;
        bool removedAny = true;
        while (removedAny && ring.size() > 3) {
            removedAny = false;
            size_t index = 0;
            while (index < ring.size() && ring.size() > 3) {
                size_t c = ring.size();
                P incoming = subp(ring[index], ring[(index + c - 1) % c]), outgoing = subp(ring[(index + 1) % c], ring[index]);
                double lengths = (double)std::sqrt(incoming.x * incoming.x + incoming.y * incoming.y) *
                                 (double)std::sqrt(outgoing.x * outgoing.x + outgoing.y * outgoing.y);
                double dt = (double)incoming.x * (double)outgoing.x + (double)incoming.y * (double)outgoing.y;
                if (lengths > 0 && dt > 0 && std::fabs(crossd(incoming, outgoing)) <= 1e-5 * lengths) {
                    ring.erase(ring.begin() + index);
                    removedAny = true;
                } else {
                    ++index;
                }
            }
        }
        double orientation = area > 0 ? 1.0 : -1.0;
        size_t c = ring.size();
        for (size_t index = 0; index < c; ++index) {
            P previous = ring[(index + c - 1) % c], a = ring[index], b = ring[(index + 1) % c], next = ring[(index + 2) % c];
            bp_segment s = segment(first_id + (int64_t)index, a, b);
            bool convexStart = crossd(subp(a, previous), subp(b, a)) * orientation > 0;
            bool convexEnd = crossd(subp(b, a), subp(next, b)) * orientation > 0;
            s.flags |= BP_SEGMENT_POLYGON_EDGE | (convexStart ? BP_SEGMENT_CONVEX_START : 0u) | (convexEnd ? BP_SEGMENT_CONVEX_END : 0u);
            s.outward_sign = area > 0 ? -1.0f : 1.0f;
            s.previous_start[0] = previous.x;
            s.previous_start[1] = previous.y;
            result.push_back(s);
        }
    }
    if (out_count) *out_count = (uint32_t)result.size();
    if (out)
        for (uint32_t q = 0; q < result.size() && q < capacity; ++q) out[q] = result[q];
    return result.size() > capacity && out ? BP_E_CAPACITY : BP_OK;
}

int bp_device_contact_law(bp_context* context, uint32_t mode, const float* in, float* out, uint32_t count) {
    if (!context || (!in && count) || (!out && count) || mode > 2) return BP_E_INVALID;
    DeviceGuard guard(context->device);
    float *dIn = nullptr, *dOut = nullptr;
    size_t bytes = (size_t)std::max<uint32_t>(count, 1) * 8 * sizeof(float);
    cudaError_t err = cudaMalloc(&dIn, bytes);
    if (!err) err = cudaMalloc(&dOut, bytes);
    if (!err && count) err = cudaMemcpyAsync(dIn, in, (size_t)count * 8 * sizeof(float), cudaMemcpyHostToDevice, context->stream);
    if (!err) err = launch_contact_law(mode, dIn, dOut, count, context->stream);
    if (!err && count) err = cudaMemcpyAsync(out, dOut, (size_t)count * 8 * sizeof(float), cudaMemcpyDeviceToHost, context->stream);
    if (!err) err = cudaStreamSynchronize(context->stream);
    if (dIn) cudaFree(dIn);
    if (dOut) cudaFree(dOut);
    return cuda_status(err);
}

}  // extern "C"
