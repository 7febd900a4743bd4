// bp_step.cuh - the bubble step on sm_103a: every device function of one world's step and the templates of the two
// persistent kernels (batched worlds, served worlds). The kernels are instantiated in bp_step_variant.cu, one
// (kernel, block width, tree) variant per object file so the large instantiations compile in parallel; the launchers
// and the small kernels live in bp_step.cu.
//
// One world is stepped by one "team" (bp_team.cuh): a group of warps of a block (small worlds, several per block), a
// thread block (medium worlds) or the whole grid of a cooperative launch (one large world). All worlds of a batch run
// in one launch. The team runs the complete step of the reference's single-group kernel nativeSubstepLoopSingleGroup
// (NFK:1236-1307): broadphase, initial forces, the adaptive substep loop with in-step grid rebuilds, and the
// end-of-step work. So a batch costs one launch per step whatever the substep counts of its worlds are.
//
// Per-bubble arithmetic follows NFK / NGK operation order exactly. Reductions pick the largest / smallest value with
// the lower bubble index winning ties, which is order-independent. Row sums that are spread over a warp's lanes
// (warp_rows) are still added by the owning lane in row order. So every team shape gives bit-identical results.
#pragma once
#include <type_traits>

#include "bp_team.cuh"
#include "bp_tree.cuh"

namespace bp {
// Everything up to the variant declarations has internal linkage: each translation unit that instantiates a kernel
// compiles its own copy of the device code.
namespace {

constexpr uint32_t kValid = 0x40000000u;        // bubble is in the grid of the current build
constexpr uint32_t kStartFinite = 0x20000000u;  // the step-start centre is finite (set when the step begins)
constexpr uint32_t kLive = 0xffu;         // mask of the public flags

// Optional per-phase cycle counters (leader thread's clock) for profiling builds (-DBP_PHASE_TIMING).
#ifdef BP_PHASE_TIMING
#define BP_PHASE(id)                                                                                  \
    do {                                                                                              \
        if (team.leader() && S.phaseCycles) {                                                         \
            long long now_ = clock64();                                                               \
            S.phaseCycles[(uint64_t)wi * kPhaseCount + (id)] += (unsigned long long)(now_ - phaseMark); \
            phaseMark = now_;                                                                         \
        }                                                                                             \
    } while (0)
#define BP_PHASE_START long long phaseMark = clock64()
// global time (ns) of a point of the world's step, overwritten every step (slots 24 and 25: start and end)
#define BP_STAMP(state, id)                                                                              \
    do {                                                                                                 \
        if (team.leader() && (state).phaseCycles) {                                                      \
            unsigned long long t_;                                                                       \
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_));                                       \
            (state).phaseCycles[(uint64_t)wi * kPhaseCount + (id)] = t_;                                 \
        }                                                                                                \
    } while (0)
#define BP_SUBPHASE(id)                                                                                     \
    do {                                                                                                    \
        if (team.leader() && S.phaseCycles) {                                                               \
            long long now_ = clock64();                                                                     \
            S.phaseCycles[(uint64_t)subWorld * kPhaseCount + (id)] += \
                (unsigned long long)(now_ - subMark);                                                       \
            subMark = now_;                                                                                 \
        }                                                                                                   \
    } while (0)
#else
#define BP_PHASE(id) do { } while (0)
#define BP_PHASE_START do { } while (0)
#define BP_STAMP(state, id) do { } while (0)
#define BP_SUBPHASE(id) do { } while (0)
#endif

struct Ctl {  // NativeSubstepControl (NFK:22-26), kept identical in every thread of the team
    float timeX, timeY, timeZ, timeW;
    uint32_t cX, cY, cZ, cW;
    int64_t limObj;
    uint32_t limTerm;
};

__device__ __forceinline__ uint32_t grid_hash(long long cx, long long cy, uint32_t buckets) {
    return ((uint32_t)cx * 73856093u ^ (uint32_t)cy * 19349663u) & (buckets - 1u);
}

__device__ __forceinline__ bool removed(const DState& S, uint32_t g) { return (S.flags[g] & kRemoved) != 0u; }

template <class Team> constexpr bool kGridTeam = std::is_same<Team, GridTeam>::value;
// nativeIsStatic / nativeInverseMass / nativeIsForceDriven / nativeEffectiveVelocity, NFK:388-392
__device__ __forceinline__ bool is_static(uint32_t flags, float invMass) {
    return !(invMass > 0.0f) || ((flags & BP_BUBBLE_ENABLED) && (flags & BP_BUBBLE_STATIC));
}
__device__ __forceinline__ float inv_mass(const DState& S, uint32_t g) {
    float im = S.phys[g].y;
    return is_static(S.flags[g], im) ? 0.0f : im;
}
__device__ __forceinline__ float2 eff_vel(const DState& S, uint32_t g) {
    return is_static(S.flags[g], S.phys[g].y) ? f2(0.0f, 0.0f) : S.vel[g];
}

// nativeJointExcluded, NGK:254-258 (entity: bubble index, or bubble count + body index)
__device__ __forceinline__ bool joint_excluded(const DState& S, const DWorld& W, uint32_t entity, int64_t partner) {
    if (entity >= W.njEnt) return false;
    uint2 r = S.jranges[W.jrOff + entity];
    for (uint32_t i = 0; i < r.y; ++i)
        if (S.jpartners[r.x + i] == partner) return true;
    return false;
}

// Field force (nativeFieldForce, NFK:395-409)
__device__ float2 field_force(const DState& S, const DField& f, float2 point) {
    float2 delta = sub(point, f.pos);
    float c = f.cosr, s = f.sinr;
    float2 local = f2(c * delta.x + s * delta.y, -s * delta.x + c * delta.y);
    float distance = len2(local), radius = f.radius;
    if (f.vcount == 0u) {
        if (!(distance <= radius)) return f2(0.0f, 0.0f);
    } else {
        bool inside = false;
        for (uint32_t i = 0; i < f.vcount; ++i) {
            float2 a = S.fverts[f.voff + i], b = S.fverts[f.voff + (i + 1) % f.vcount];
            if ((a.y > local.y) != (b.y > local.y) && local.x < (b.x - a.x) * (local.y - a.y) / (b.y - a.y) + a.x) inside = !inside;
        }
        if (!inside) return f2(0.0f, 0.0f);
    }
    if (f.kind == 0u) return f2(c * f.dir.x - s * f.dir.y, s * f.dir.x + c * f.dir.y);
    if (!(distance > 0.0f)) return f2(0.0f, 0.0f);
    float profile = f.falloff == 0.0f ? 1.0f : powf(fmaxf(0.0f, 1.0f - distance / radius), f.falloff);
    float scale = f.strength * profile / distance;
    return f.kind == 2u ? mul(f2(-delta.y, delta.x), scale) : mul(delta, scale);
}
__device__ bool field_affects(const DState& S, const DField& f, int64_t id) {
    if (!f.hasFilter) return true;
    uint32_t low = f.foff, end = f.foff + f.fcount, high = end;
    while (low < high) {
        uint32_t mid = low + (high - low) / 2;
        if (S.fids[mid] < id) low = mid + 1; else high = mid;
    }
    return low < end && S.fids[low] == id;
}
template <class R> __device__ const R* find_by_bubble(const R* v, uint32_t count, int64_t id) {
    uint32_t low = 0, high = count;
    while (low < high) {
        uint32_t mid = low + (high - low) / 2;
        if (v[mid].bubble_id < id) low = mid + 1; else high = mid;
    }
    return low < count && v[low].bubble_id == id ? v + low : nullptr;
}
// nativeNonContactAcceleration, NFK:450-470, plus the world's gravity acceleration
__device__ float2 non_contact_acc(const DState& S, const DWorld& W, uint32_t g, float2 position) {
    float im = inv_mass(S, g);
    if (!(S.flags[g] & BP_BUBBLE_FORCE_DRIVEN) || !(im > 0.0f)) return f2(0.0f, 0.0f);
    float2 force = W.gforce;
    int64_t id = S.id[g];
    for (uint32_t i = 0; i < W.nf; ++i) {
        DField f = S.fields[W.foff + i];
        if (field_affects(S, f, id)) force = add(force, field_force(S, f, position));
    }
    if (W.nbands) {
        const bp_band* band = find_by_bubble(S.bands + W.bandOff, W.nbands, id);
        if (band) {
            float2 bf = mul(sub(f2(band->target[0], band->target[1]), position), band->stiffness);
            float lim = band->maximum_force, magnitude = len2(bf);
            if (lim > 0.0f && magnitude > lim) bf = mul(bf, lim / magnitude);
            force = add(force, bf);
        }
    }
    if (W.nmotors) {
        const bp_motor* motor = find_by_bubble(S.motors + W.motorOff, W.nmotors, id);
        if (motor) force = add(force, f2(motor->force[0], motor->force[1]));
    }
    float2 a = mul(force, im);
    if (W.gravity.x != 0.0f || W.gravity.y != 0.0f) a = add(a, W.gravity);
    return a;
}

// ------------------------------------------------------------------------------------------------------------------
// Body poses at the current step fraction, memoized once per body (nativeBodyAtFraction, NFK:155-159): every
// (bubble, body) term then reads the same values body_at would compute.
template <class Team> __device__ void refresh_poses(const DState& S, const DWorld& W, const Team& team, float fraction) {
    for (uint32_t bi = team.rank(); bi < W.nb; bi += team.size()) {
        Pose p = body_at(S.body[W.bodyOff + bi], fraction);
        S.bpose[W.bodyOff + bi] = make_float4(p.pos.x, p.pos.y, p.c, p.s);
    }
}
__device__ __forceinline__ Pose cached_pose(const DState& S, const DWorld& W, uint32_t bi) {
    float4 v = S.bpose[W.bodyOff + bi];
    Pose p;
    p.pos = f2(v.x, v.y);
    p.c = v.z;
    p.s = v.w;
    return p;
}

// Per-bubble substep terms (NFK:216-243, 510-614)
// ------------------------------------------------------------------------------------------------------------------
__device__ __forceinline__ const uint32_t* adj_row(const DState& S, const DWorld& W, uint32_t i) {
    return S.adj + W.rowOff + (uint64_t)i * W.k;
}

// One adjacency entry's share of bubble i's contact force and omega^2 (the body of the row loop of
// nativeBubbleContactForce, NFK:216-243, and nativeBubbleOmegaSquared, NFK:510-541, which read the same law
// evaluations): x, y = the force term, z = the omega^2 term, w = which of the two the row sum adds (bit 0 force, bit 1
// omega^2; a wall out of its region adds neither). p, ph and im are bubble i's centre, physical record and inverse mass.
__device__ __forceinline__ float4 contact_term(const DState& S, const DWorld& W, uint32_t i, uint32_t entry, float2 p,
                                               float4 ph, float im) {
    const uint32_t kind = entry >> kKindShift, j = entry & kIndexMask;
    if (kind == 0u) {
        uint32_t low = min(i, j), high = max(i, j);
        uint32_t gl = W.boff + low, gh = W.boff + high;
        float2 delta = sub(S.pos[gh], S.pos[gl]);
        float dist = len2(delta);
        float2 normal = dist > 0.0f ? dvd(delta, dist) : f2(1.0f, 0.0f);
        float4 pl = S.phys[gl], phh = S.phys[gh];
        Law law = pair_law(pl.z, pl.x, phh.z, phh.x, dist);
        float2 v = mul(normal, i == low ? -law.force : law.force);
        if (!(im > 0.0f)) return make_float4(v.x, v.y, 0.0f, __uint_as_float(1u));
        return make_float4(v.x, v.y, law.stiffness * (im + sqrtf(im * inv_mass(S, W.boff + j))), __uint_as_float(3u));
    }
    if (kind == 1u) {
        float2 normal;
        float dist;
        if (!wall_region(S.seg[W.soff + j], p, normal, dist) || !(dist < ph.x)) return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        Law wl = wall_law(ph.z, ph.x, dist);
        float2 v = mul(normal, wl.force);
        return make_float4(v.x, v.y, wl.stiffness * im, __uint_as_float(3u));
    }
    Obstacle o = body_obstacle(S.bverts, S.btris, S.body[W.bodyOff + j], cached_pose(S, W, j), p);
    Law wl = wall_law(ph.z, ph.x, o.distance);
    float2 v = mul(o.normal, wl.force);
    return make_float4(v.x, v.y, wl.stiffness * im, __uint_as_float(3u));
}

// Row entries of a warp's bubbles spread evenly over its lanes. Lane l owns a row of `deg` entries (0 without one);
// the warp's entries are numbered row by row in lane order, and in each round every lane evaluates the next entry,
// `term(o, e)` = entry e of lane o's row, into its slot of `slots` (one float4 per lane of this warp). Each owner then
// hands its own entries' values to `take` in row order, so a row sum adds the same terms in the same order as a
// sequential loop over the row. The whole warp calls this together.
// Exclusive scan of the lanes' row lengths; returns the warp's total.
__device__ __forceinline__ uint32_t warp_row_starts(uint32_t deg, uint32_t& start) {
    const uint32_t lane = threadIdx.x & 31u;
    start = deg;
#pragma unroll
    for (uint32_t d = 1; d < 32u; d <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, start, d);
        if (lane >= d) start += v;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, start, 31);
    start -= deg;
    return total;
}
// The lane whose row holds entry f of the warp's numbering (the last lane whose row starts at or before f), and the
// entry's index in that row.
__device__ __forceinline__ uint32_t warp_row_owner(uint32_t start, uint32_t f, uint32_t& e) {
    uint32_t o = 0;
#pragma unroll
    for (uint32_t step = 16; step; step >>= 1) {
        const uint32_t so = __shfl_sync(0xffffffffu, start, o + step);
        if (so <= f) o += step;
    }
    e = f - __shfl_sync(0xffffffffu, start, o);
    return o;
}

template <class Term, class Take>
__device__ __forceinline__ void warp_rows(uint32_t deg, float4* slots, Term&& term, Take&& take) {
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t start;
    const uint32_t total = warp_row_starts(deg, start);
    for (uint32_t t0 = 0; t0 < total; t0 += 32u) {
        const uint32_t f = t0 + lane;
        uint32_t e;
        const uint32_t o = warp_row_owner(start, f, e);
        if (f < total) slots[lane] = term(o, e);
        __syncwarp();
        const uint32_t lo = max(start, t0), hi = min(start + deg, t0 + 32u);
        for (uint32_t x = lo; x < hi; ++x) take(slots[x - t0]);
        __syncwarp();
    }
}

// The same numbering without a row sum: `visit(o, e)` runs once for every entry e of every lane o's row, spread evenly
// over the lanes (for passes whose per-entry results need no ordered combination). The whole warp calls this together.
template <class Visit>
__device__ __forceinline__ void warp_entries(uint32_t deg, Visit&& visit) {
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t start;
    const uint32_t total = warp_row_starts(deg, start);
    for (uint32_t t0 = 0; t0 < total; t0 += 32u) {
        const uint32_t f = t0 + lane;
        uint32_t e;
        const uint32_t o = warp_row_owner(start, f, e);
        if (f < total) visit(o, e);
    }
}

// Contact force and omega^2 of bubble i0 + lane for every lane of the warp (`has`: the lane's bubble takes part),
// nativeBubbleContactForce + nativeBubbleOmegaSquared with the row entries spread over the warp (warp_rows).
__device__ __forceinline__ float2 warp_contact_terms(const DState& S, const DWorld& W, uint32_t i0, bool has, float im,
                                                     float4* slots, float& omega2) {
    const uint32_t i = i0 + (threadIdx.x & 31u), g = W.boff + i;
    float2 total = f2(0.0f, 0.0f);
    float w2 = 0.0f;
    if (has && im > 0.0f && W.nbands) {
        const bp_band* band = find_by_bubble(S.bands + W.bandOff, W.nbands, S.id[g]);
        if (band) w2 = w2 + band->stiffness * im;
    }
    warp_rows(has ? S.deg[g] : 0u, slots,
              [&](uint32_t o, uint32_t e) {
                  const uint32_t io = i0 + o, go = W.boff + io;
                  return contact_term(S, W, io, adj_row(S, W, io)[e], S.pos[go], S.phys[go], inv_mass(S, go));
              },
              [&](float4 c) {
                  const uint32_t use = __float_as_uint(c.w);
                  if (use & 1u) total = add(total, f2(c.x, c.y));
                  if (use & 2u) w2 = w2 + c.z;
              });
    omega2 = im > 0.0f ? w2 : 0.0f;
    return total;
}

__device__ float omega_squared(const DState& S, const DWorld& W, uint32_t i, float fraction) {
    const uint32_t g = W.boff + i;
    float im = inv_mass(S, g);
    if (!(im > 0.0f)) return 0.0f;
    const float2 p = S.pos[g];
    const float4 ph = S.phys[g];
    float total = 0.0f;
    if (W.nbands) {
        const bp_band* band = find_by_bubble(S.bands + W.bandOff, W.nbands, S.id[g]);
        if (band) total = total + band->stiffness * im;
    }
    const uint32_t* row = adj_row(S, W, i);
    const uint32_t d = S.deg[g];
    for (uint32_t e = 0; e < d; ++e) {
        uint32_t entry = row[e], kind = entry >> kKindShift, j = entry & kIndexMask;
        if (kind == 0u) {
            uint32_t low = min(i, j), high = max(i, j);
            uint32_t gl = W.boff + low, gh = W.boff + high;
            float dist = len2(sub(S.pos[gh], S.pos[gl]));
            float4 pl = S.phys[gl], phh = S.phys[gh];
            Law law = pair_law(pl.z, pl.x, phh.z, phh.x, dist);
            total = total + law.stiffness * (im + sqrtf(im * inv_mass(S, W.boff + j)));
        } else if (kind == 1u) {
            float2 normal;
            float dist;
            if (!wall_region(S.seg[W.soff + j], p, normal, dist) || !(dist < ph.x)) continue;
            total = total + wall_law(ph.z, ph.x, dist).stiffness * im;
        } else {
            Obstacle o = body_obstacle(S.bverts, S.btris, S.body[W.bodyOff + j], cached_pose(S, W, j), p);
            total = total + wall_law(ph.z, ph.x, o.distance).stiffness * im;
        }
    }
    return total;
}

// One adjacency entry's distance bound for a movable bubble at p with the given velocity, radius and |acceleration|
// (the body of the row loop of nativeBubbleDistanceBound, NFK:545-614); +inf for an entry that sets no bound.
__device__ __forceinline__ float distance_term(const DState& S, const DWorld& W, uint32_t entry, float2 p, float2 velocity,
                                               float radius, float accSelf, float hMax) {
    const float inf = __int_as_float(0x7f800000);
    const uint32_t kind = entry >> kKindShift, j = entry & kIndexMask;
    float dist, approach, accSum, reach, bodySpeed = 0.0f;
    if (kind == 0u) {
        uint32_t gj = W.boff + j;
        float2 delta = sub(S.pos[gj], p);
        dist = len2(delta);
        float2 normal = dist > 0.0f ? dvd(delta, dist) : f2(1.0f, 0.0f);
        approach = dot2(sub(velocity, eff_vel(S, gj)), normal);
        accSum = accSelf + len2(S.acc[gj]);
        reach = radius + S.phys[gj].x;
    } else if (kind == 1u) {
        float2 normal;
        if (!wall_region(S.seg[W.soff + j], p, normal, dist)) return inf;
        approach = -dot2(velocity, normal);
        accSum = accSelf;
        reach = radius;
    } else {
        Obstacle o = body_obstacle(S.bverts, S.btris, S.body[W.bodyOff + j], cached_pose(S, W, j), p);
        dist = o.distance;
        approach = -dot2(velocity, o.normal);
        bodySpeed = o.speedBound;
        accSum = accSelf;
        reach = radius;
    }
    bool active = dist < reach;
    float dd = fmaxf(dist, reach * 1e-6f);
    float speed;
    if (active) speed = fabsf(approach) + bodySpeed;
    else {
        if (approach + bodySpeed + accSum * hMax * 0.5f <= 0.0f) return inf;
        speed = approach + bodySpeed;
    }
    float sq = sqrtf(speed * speed + accSum * dd * 0.5f);
    float denominator = sq + speed;
    if (!(denominator > 0.0f)) return inf;
    return dd / (2.0f * denominator);
}

// Distance bound of bubble i0 + lane for every lane of the warp (`has`: the lane's bubble takes part; an immovable
// bubble sets none): the minimum over its row, entries spread over the warp (warp_rows).
__device__ __forceinline__ float warp_distance_bound(const DState& S, const DWorld& W, uint32_t i0, bool has, float hMax,
                                                     float4* slots) {
    const uint32_t g = W.boff + i0 + (threadIdx.x & 31u);
    float best = __int_as_float(0x7f800000);
    const bool movable = has && inv_mass(S, g) > 0.0f;
    warp_rows(movable ? S.deg[g] : 0u, slots,
              [&](uint32_t o, uint32_t e) {
                  const uint32_t io = i0 + o, go = W.boff + io;
                  const float v = distance_term(S, W, adj_row(S, W, io)[e], S.pos[go], S.vel[go], S.phys[go].x,
                                                len2(S.acc[go]), hMax);
                  return make_float4(v, 0.0f, 0.0f, 0.0f);
              },
              [&](float4 c) { best = fminf(best, c.x); });
    return best;
}

__device__ __forceinline__ float margin_bound(const DState& S, uint32_t g) {
    const float inf = __int_as_float(0x7f800000);
    if (!(inv_mass(S, g) > 0.0f)) return inf;
    float left = S.margin[g] - len2(sub(S.pos[g], S.ref[g]));
    if (isnan(left)) return inf;
    if (left <= 0.0f) return 0.0f;
    float speed = len2(S.vel[g]), a = len2(S.acc[g]);
    float denominator = speed + sqrtf(speed * speed + 2.0f * a * left);
    return denominator > 0.0f ? 2.0f * left / denominator : inf;
}

// ------------------------------------------------------------------------------------------------------------------
// Broadphase pieces
// ------------------------------------------------------------------------------------------------------------------
// nativeBubblePairCandidate range test for the pair (low, high) in row `low` (NGK:262-273)
__device__ __forceinline__ bool pair_accepts(const DState& S, const DWorld& W, uint32_t low, uint32_t high) {
    uint32_t gl = W.boff + low, gh = W.boff + high;
    if (!filter_accepts(S.filter[gl], S.filter[gh])) return false;
    if (W.njEnt && joint_excluded(S, W, low, S.id[gh])) return false;
    float reach = S.phys[gl].x + S.phys[gh].x + S.margin[gl] + S.margin[gh] + W.sepTol;
    float2 a = S.pos[gl], b = S.pos[gh];
    return fabsf(a.x - b.x) <= reach && fabsf(a.y - b.y) <= reach;
}
// segment rule of nativeFinishBubbleRow (NGK:279-290)
__device__ __forceinline__ bool segment_accepts(const DState& S, const DWorld& W, uint32_t i, uint32_t sj) {
    uint32_t g = W.boff + i;
    const RigidBox rb = S.segBox[W.soff + sj];
    if (!filter_accepts(S.filter[g], make_uint2(rb.cat, rb.mask))) return false;
    if ((rb.flags & BP_SEGMENT_HAS_OWNER) && W.njEnt && joint_excluded(S, W, i, S.seg[W.soff + sj].owner)) return false;
    float reach = S.phys[g].x + S.margin[g] + W.sepTol;
    float2 lower = sub(f2(rb.box.x, rb.box.y), f2(reach, reach));
    float2 upper = add(f2(rb.box.z, rb.box.w), f2(reach, reach));
    float2 p = S.pos[g];
    return p.x >= lower.x && p.y >= lower.y && p.x <= upper.x && p.y <= upper.y;
}
// bubble obstacle rule of nativeEmitBodyCandidates (NGK:361-378)
__device__ __forceinline__ bool body_is_obstacle(const DBody& b) {
    return (b.flags & BP_BODY_STATIC) ? b.kind != BP_BODY_POLYGON : (b.flags & BP_BODY_KINEMATIC) != 0u;
}
__device__ __forceinline__ bool body_accepts(const DState& S, const DWorld& W, const RigidBox& rb, uint32_t bi, uint32_t i) {
    uint32_t g = W.boff + i;
    if (!filter_accepts(S.filter[g], make_uint2(rb.cat, rb.mask))) return false;
    if (W.njEnt && joint_excluded(S, W, W.n + bi, S.id[g])) return false;
    float2 bodyLow = f2(rb.box.x, rb.box.y);
    float2 bodyHigh = f2(rb.box.z, rb.box.w);
    float reach = S.phys[g].x + fmaxf(S.margin[g], 0.0f);
    float2 c = S.pos[g];
    float2 lo = sub(c, f2(reach, reach)), hi = add(c, f2(reach, reach));
    return !(hi.x < bodyLow.x || hi.y < bodyLow.y || bodyHigh.x < lo.x || bodyHigh.y < lo.y);
}

// Insert `value` into a row kept sorted ascending with at most `limit` entries (nativeInsertCandidate, NGK:238-251).
__device__ __forceinline__ void insert_sorted(uint32_t* row, uint32_t& count, uint32_t limit, uint32_t value) {
    uint32_t loc;
    if (count < limit) loc = count++;
    else {
        if (!(value < row[limit - 1])) return;
        loc = limit - 1;
    }
    while (loc > 0 && value < row[loc - 1]) { row[loc] = row[loc - 1]; --loc; }
    row[loc] = value;
}

__device__ __forceinline__ bool row_contains(const uint32_t* row, uint32_t count, uint32_t value) {
    uint32_t low = 0, high = count;
    while (low < high) {
        uint32_t mid = (low + high) >> 1;
        if (row[mid] < value) low = mid + 1; else high = mid;
    }
    return low < count && row[low] == value;
}

// Visits every bubble j registered in cell (tx, ty) of the hash grid.
template <class F>
__device__ __forceinline__ void for_each_in_cell(const longlong2* cells, const DWorld& W, const uint32_t* buckets,
                                                 const uint32_t* entries, uint32_t B, long long tx, long long ty, F&& f) {
    uint32_t h = grid_hash(tx, ty, B);
    uint32_t begin = h == 0u ? 0u : buckets[h - 1], end = buckets[h];
    for (uint32_t e = begin; e < end; ++e) {
        uint32_t j = entries[e];
        longlong2 c = cells[W.boff + j];
        if (c.x == tx && c.y == ty) f(j);
    }
}

// Body-row hits of bubble i found through the tree: slots are taken in arrival order and put in index order (or
// rebuilt by brute force when the row overflows) by fix_body_row.
__device__ __forceinline__ void body_hit(const DState& S, const DWorld& W, uint32_t bi, uint32_t i) {
    const uint32_t slot = atomicAdd(S.bodyTotal + W.bodyOff + bi, 1u);
    if (slot < W.k) S.bodyRow[W.bodyRowOff + (uint64_t)bi * W.k + slot] = i;
}

// Lower pair (j, i), j < i, of bubble i's adjacency (the pair lives in row j): the same tests as the candidate rule
// of row j; whether row j kept i is checked once every row is built (finish_adjacency).
__device__ __forceinline__ void lower_pair(const DState& S, const DWorld& W, uint32_t i, uint32_t j, uint32_t* adjRow,
                                           uint32_t& kept, uint32_t& total) {
    if (!(S.flags[W.boff + j] & kStartFinite)) return;
    if (!pair_accepts(S, W, j, i)) return;
    ++total;
    insert_sorted(adjRow, kept, W.k, j);
}

// Forward candidate row of bubble i: pairs with j > i, then segments; k smallest keys (NGK:300-330). The same cell
// scan collects the lower pairs j < i into the adjacency row (their count goes to deg until finish_adjacency). With
// the tree, the rigid traversal also registers i in the rows of the bodies that accept it.
template <bool kTree, bool kPrune>
__device__ void emit_row(const DState& S, const DWorld& W, const uint32_t* buckets, const uint32_t* entries,
                         const float4* records, uint32_t B, float cw, uint32_t i, uint32_t& overflow, uint32_t& maxPer) {
    const uint32_t g = W.boff + i, k = W.k;
    uint32_t* row = S.candRow + W.rowOff + (uint64_t)i * k;
    uint32_t* adjRow = S.adj + W.rowOff + (uint64_t)i * k;
    uint32_t lowerKept = 0, lowerTotal = 0;
    if (!(S.flags[g] & kValid) || !(S.flags[g] & kStartFinite)) {
        S.candCount[g] = make_uint2(0u, 0u);
        S.pairTotal[g] = 0u;
        if (S.flags[g] & kValid) {  // a valid cell with a non-finite step start: no row, but lower pairs still count
            const longlong2 c = S.cell[g];
            for (int dx = -1; dx <= 1; ++dx)
                for (int dy = -1; dy <= 1; ++dy)
                    for_each_in_cell(S.cell, W, buckets, entries, B, c.x + dx, c.y + dy, [&](uint32_t j) {
                        if (j < i) lower_pair(S, W, i, j, adjRow, lowerKept, lowerTotal);
                    });
        }
        S.deg[g] = lowerTotal;
        if (kTree && W.nb && !removed(S, g)) {
            // a bubble without a valid cell still meets the body rule (a non-finite centre fails no comparison)
            const float reach = S.phys[g].x + fmaxf(S.margin[g], 0.0f);
            const float2 c = S.pos[g], lo = sub(c, f2(reach, reach)), hi = add(c, f2(reach, reach));
            tree_query(S, W, [&](float4 nb) { return !(hi.x < nb.x || hi.y < nb.y || nb.z < lo.x || nb.w < lo.y); },
                       [&](uint32_t leaf) {
                           if (leaf < W.s) return;
                           const uint32_t bi = leaf - W.s;
                           const RigidBox rb = S.bodyBox[W.bodyOff + bi];
                           if (rb.flags && body_accepts(S, W, rb, bi, i)) body_hit(S, W, bi, i);
                       });
        }
        return;
    }
    longlong2 c = S.cell[g];
    uint32_t count = 0, total = 0;
    // The pair rule (pair_accepts, and lower_pair for j < i) with its box test first, on the entry's record: reach and
    // distances are computed in the same order of operations as the rule, so every decision is the rule's. The entry's
    // own cell is read only for pairs within reach (another cell may share the bucket).
    const float2 pi = S.pos[g];
    const float ri = S.phys[g].x, mi = S.margin[g], tol = W.sepTol;
    const uint2 fi = S.filter[g];
    // With kPrune only the cells of the 3x3 block that meet the square of half-side R around the centre are scanned:
    // they alone can hold a pair within reach, since every r_j + m_j is at most (cw - tol) / 2, so reach <= r_i + m_i +
    // cw / 2 + |tol|; the relative slack covers every rounding of the reach, the box test and the cell coordinates
    // (visiting a cell more is harmless, the rule decides). A non-finite R scans the whole block. This pays where
    // entries are read from global memory; on staged worlds the whole block is scanned.
    int x0 = -1, x1 = 1, y0 = -1, y1 = 1;
    if (kPrune) {
        const float reachMax = ri + mi + 0.5f * cw + fabsf(tol);
        const float R = reachMax + 1e-4f * (fabsf(ri) + fabsf(mi) + cw + fabsf(tol) + fabsf(pi.x) + fabsf(pi.y)) + 1e-3f;
        if (R < cw) {
            const long long lx = (long long)clampf(floorf((pi.x - R) / cw), -4.0e18f, 4.0e18f);
            const long long hx = (long long)clampf(floorf((pi.x + R) / cw), -4.0e18f, 4.0e18f);
            const long long ly = (long long)clampf(floorf((pi.y - R) / cw), -4.0e18f, 4.0e18f);
            const long long hy = (long long)clampf(floorf((pi.y + R) / cw), -4.0e18f, 4.0e18f);
            if (lx >= c.x) x0 = 0;
            if (hx <= c.x) x1 = 0;
            if (ly >= c.y) y0 = 0;
            if (hy <= c.y) y1 = 0;
        }
    }
    // one cell of the scan: entries [begin, end) of the bucket of cell (tx, ty)
    auto scan_cell = [&](const long long tx, const long long ty, const uint32_t begin, const uint32_t end) {
        auto visit = [&](const float4 q, const uint32_t j) {
            if (j == i) return;
            const float reach = j < i ? q.z + ri + q.w + mi + tol : ri + q.z + mi + q.w + tol;
            if (!(fabsf(pi.x - q.x) <= reach && fabsf(pi.y - q.y) <= reach)) return;
            const uint32_t gj = W.boff + j;
            const longlong2 cj = S.cell[gj];
            if (cj.x != tx || cj.y != ty) return;
            if (j < i) {
                if (!(S.flags[gj] & kStartFinite)) return;
                if (!filter_accepts(S.filter[gj], fi)) return;
                if (W.njEnt && joint_excluded(S, W, j, S.id[g])) return;
                ++lowerTotal;
                insert_sorted(adjRow, lowerKept, k, j);
            } else {
                if (!filter_accepts(fi, S.filter[gj])) return;
                if (W.njEnt && joint_excluded(S, W, i, S.id[gj])) return;
                ++total;
                insert_sorted(row, count, k, j);
            }
        };
        uint32_t e = begin;
        if (kPrune)  // entries in global memory: two loads in flight before the first test
            for (; e + 1u < end; e += 2u) {
                const float4 q0 = records[e], q1 = records[e + 1u];
                const uint32_t j0 = entries[e], j1 = entries[e + 1u];
                visit(q0, j0);
                visit(q1, j1);
            }
        for (; e < end; ++e) visit(records[e], entries[e]);
    };
    if (kPrune) {
        // the buckets live in global memory: every cell's bounds are loaded before the first cell is scanned
        uint32_t cb[9], ce[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            const int dx = q / 3 - 1, dy = q % 3 - 1;
            cb[q] = 0u;
            ce[q] = 0u;
            if (dx >= x0 && dx <= x1 && dy >= y0 && dy <= y1) {
                const uint32_t h = grid_hash(c.x + dx, c.y + dy, B);
                cb[q] = h == 0u ? 0u : buckets[h - 1];
                ce[q] = buckets[h];
            }
        }
#pragma unroll
        for (int q = 0; q < 9; ++q) scan_cell(c.x + (q / 3 - 1), c.y + (q % 3 - 1), cb[q], ce[q]);
    } else {
        for (int dx = x0; dx <= x1; ++dx)
            for (int dy = y0; dy <= y1; ++dy) {
                const long long tx = c.x + dx, ty = c.y + dy;
                const uint32_t h = grid_hash(tx, ty, B);
                scan_cell(tx, ty, h == 0u ? 0u : buckets[h - 1], buckets[h]);
            }
    }
    S.deg[g] = lowerTotal;
    const uint32_t pairs = count;
    uint32_t segTotal = 0;
    if (kTree) {
        // segments kept in index order up to the free slots, as the brute-force loop below appends them
        uint32_t* segRow = row + pairs;
        const uint32_t segLimit = k - pairs;
        uint32_t segKept = 0;
        const float2 p = S.pos[g];
        const float reachS = S.phys[g].x + S.margin[g] + W.sepTol;
        const float reachB = S.phys[g].x + fmaxf(S.margin[g], 0.0f);
        const float2 lo = sub(p, f2(reachB, reachB)), hi = add(p, f2(reachB, reachB));
        const bool wantBodies = W.nb != 0u;
        tree_query(S, W,
                   [&](float4 nb) {
                       const bool seg = p.x >= nb.x - reachS && p.y >= nb.y - reachS && p.x <= nb.z + reachS &&
                                        p.y <= nb.w + reachS;
                       const bool body = wantBodies && !(hi.x < nb.x || hi.y < nb.y || nb.z < lo.x || nb.w < lo.y);
                       return seg || body;
                   },
                   [&](uint32_t leaf) {
                       if (leaf < W.s) {
                           if (!segment_accepts(S, W, i, leaf)) return;
                           ++segTotal;
                           if (segLimit) insert_sorted(segRow, segKept, segLimit, (1u << kKindShift) | leaf);
                           return;
                       }
                       const uint32_t bi = leaf - W.s;
                       const RigidBox rb = S.bodyBox[W.bodyOff + bi];
                       if (rb.flags && body_accepts(S, W, rb, bi, i)) body_hit(S, W, bi, i);
                   });
        count += segKept;
    } else {
        for (uint32_t sj = 0; sj < W.s; ++sj) {
            if (!segment_accepts(S, W, i, sj)) continue;
            ++segTotal;
            if (count < k) row[count++] = (1u << kKindShift) | sj;
        }
    }
    S.candCount[g] = make_uint2(pairs, count - pairs);
    S.pairTotal[g] = total;
    uint32_t all = total + segTotal;
    overflow += all - count;
    maxPer = max(maxPer, all);
}

// Body row of body bi built by one warp: the first k accepting bubbles in index order (NGK:350-392).
__device__ void emit_body_row(const DState& S, const DWorld& W, uint32_t bi, uint32_t lane, uint32_t& overflow, uint32_t& maxPer) {
    const RigidBox rb = S.bodyBox[W.bodyOff + bi];
    const uint32_t k = W.k;
    uint32_t* row = S.bodyRow + W.bodyRowOff + (uint64_t)bi * k;
    uint32_t total = 0;
    if (rb.flags) {
        for (uint32_t base = 0; base < W.n; base += 32) {
            uint32_t i = base + lane;
            bool hit = i < W.n && !removed(S, W.boff + i) && body_accepts(S, W, rb, bi, i);
            uint32_t mask = __ballot_sync(0xffffffffu, hit);
            uint32_t rank = __popc(mask & ((1u << lane) - 1u));
            if (hit && total + rank < k) row[total + rank] = i;
            total += __popc(mask);
        }
    }
    if (lane == 0) {
        S.bodyTotal[W.bodyOff + bi] = total;
        overflow += total > k ? total - k : 0u;
        maxPer = max(maxPer, total);
    }
}

// Body row bi after the tree pass: hits arrived in any order; a row that fits is sorted (the first k accepting bubbles
// in index order are then all of them), an overflowing row is rebuilt by the brute-force scan.
__device__ void fix_body_row(const DState& S, const DWorld& W, uint32_t bi, uint32_t lane, uint32_t& overflow, uint32_t& maxPer) {
    const uint32_t total = S.bodyTotal[W.bodyOff + bi];
    if (total > W.k) {
        emit_body_row(S, W, bi, lane, overflow, maxPer);
        return;
    }
    if (lane == 0) {
        uint32_t* row = S.bodyRow + W.bodyRowOff + (uint64_t)bi * W.k;
        for (uint32_t e = 1; e < total; ++e) {
            const uint32_t value = row[e];
            uint32_t loc = e;
            while (loc > 0 && value < row[loc - 1]) { row[loc] = row[loc - 1]; --loc; }
            row[loc] = value;
        }
        maxPer = max(maxPer, total);
    }
}

// Adjacency row of bubble i, sorted by (kind, neighbour), first k kept (NFK:298-331, NCK:222-238).
template <bool kTree>
__device__ void build_adjacency(const DState& S, const DWorld& W, const uint32_t* buckets, const uint32_t* entries,
                                uint32_t B, uint32_t i, uint32_t& overflow, uint32_t& maxPer) {
    const uint32_t g = W.boff + i, k = W.k;
    uint32_t* row = S.adj + W.rowOff + (uint64_t)i * k;
    uint32_t deg = 0, demanded = 0;
    if (removed(S, g)) { S.deg[g] = 0u; return; }
    const uint32_t lowerTotal = S.deg[g];  // lower pairs found by emit_row, the first k of them in the row
    if (lowerTotal <= k) {
        // keep the lower pairs whose row j holds i (only a truncated row j can miss it)
        for (uint32_t e = 0; e < lowerTotal; ++e) {
            const uint32_t j = row[e], gj = W.boff + j;
            if (S.pairTotal[gj] > k && !row_contains(S.candRow + W.rowOff + (uint64_t)j * k, S.candCount[gj].x, i)) continue;
            row[deg++] = j;
            ++demanded;
        }
    } else {
        // more lower pairs than slots: which ones are kept depends on the rows j, so scan again with that check
        longlong2 c = S.cell[g];
        for (int dx = -1; dx <= 1; ++dx)
            for (int dy = -1; dy <= 1; ++dy)
                for_each_in_cell(S.cell, W, buckets, entries, B, c.x + dx, c.y + dy, [&](uint32_t j) {
                    if (j >= i) return;
                    uint32_t gj = W.boff + j;
                    if (!(S.flags[gj] & kStartFinite)) return;
                    if (!pair_accepts(S, W, j, i)) return;
                    if (S.pairTotal[gj] > k && !row_contains(S.candRow + W.rowOff + (uint64_t)j * k, S.candCount[gj].x, i)) return;
                    ++demanded;
                    insert_sorted(row, deg, k, j);
                });
    }
    // own row: pairs (j > i), then segments
    const uint2 cc = S.candCount[g];
    const uint32_t* crow = S.candRow + W.rowOff + (uint64_t)i * k;
    for (uint32_t e = 0; e < cc.x + cc.y; ++e) {
        ++demanded;
        if (deg < k) row[deg++] = crow[e];
    }
    // bodies holding i in their row
    if (kTree) {
        if (W.nb) {
            const float reach = S.phys[g].x + fmaxf(S.margin[g], 0.0f);
            const float2 c = S.pos[g], lo = sub(c, f2(reach, reach)), hi = add(c, f2(reach, reach));
            tree_query(S, W, [&](float4 nb) { return !(hi.x < nb.x || hi.y < nb.y || nb.z < lo.x || nb.w < lo.y); },
                       [&](uint32_t leaf) {
                           if (leaf < W.s) return;
                           const uint32_t bi = leaf - W.s;
                           const RigidBox rb = S.bodyBox[W.bodyOff + bi];
                           if (!rb.flags || !body_accepts(S, W, rb, bi, i)) return;
                           const uint32_t total = S.bodyTotal[W.bodyOff + bi];
                           if (total > k && !row_contains(S.bodyRow + W.bodyRowOff + (uint64_t)bi * k, k, i)) return;
                           ++demanded;
                           insert_sorted(row, deg, k, (2u << kKindShift) | bi);
                       });
        }
    } else for (uint32_t bi = 0; bi < W.nb; ++bi) {
        const RigidBox rb = S.bodyBox[W.bodyOff + bi];
        if (!rb.flags || !body_accepts(S, W, rb, bi, i)) continue;
        uint32_t total = S.bodyTotal[W.bodyOff + bi];
        if (total > k && !row_contains(S.bodyRow + W.bodyRowOff + (uint64_t)bi * k, k, i)) continue;
        ++demanded;
        if (deg < k) row[deg++] = (2u << kKindShift) | bi;
    }
    S.deg[g] = deg;
    overflow += demanded - deg;
    maxPer = max(maxPer, demanded);
}

// ------------------------------------------------------------------------------------------------------------------
// Grid build + candidates + adjacency (one build of nativeBroadphaseInGroup, NFK:1040-1134)
// ------------------------------------------------------------------------------------------------------------------
template <class Team, bool kTree>
__device__ float broadphase(const DState& S, const DWorld& W, const Ctl& c, const Team& team, uint32_t* buckets,
                            uint32_t* entries, float4* records, uint32_t B, uint32_t& buildOverflow, uint32_t& maxPerAll, uint32_t subWorld) {
    const uint32_t n = W.n, T = team.size(), r = team.rank();
#ifdef BP_PHASE_TIMING
    long long subMark = clock64();
#endif
    // a0, margin and x0 (nativeBubbleAcceleration + nativeBubbleMargin, NFK:472-499)
    const float t = fmaxf(c.timeX - c.timeY, 0.0f);
    float cwl = W.sepTol;
    for (uint32_t i = r; i < n; i += T) {
        uint32_t g = W.boff + i;
        if (removed(S, g)) continue;
        float2 p = S.pos[g];
        float2 a0 = non_contact_acc(S, W, g, p);
        S.a0[g] = a0;
        float radius = S.phys[g].x;
        float travel = len2(eff_vel(S, g)) * t + 0.5f * len2(a0) * t * t;
        float m = (W.flags & BP_WORLD_MINIMUM_MARGIN_ONLY) ? 0.25f * radius : fmaxf(1.05f * travel, 0.25f * radius);
        S.margin[g] = m;
        S.ref[g] = p;
        cwl = fmaxf(cwl, 2.0f * (radius + m) + W.sepTol);  // nativePrepareGrid, NGK:163-177
    }
    BP_SUBPHASE(12);
    // The whole-GPU team clears the grid before the cell-width reduction, whose grid barrier then orders the clear
    // before the cells (the last readers of the buckets passed barriers since); the other teams after it.
    if (kGridTeam<Team>) {
        for (uint32_t b = r; b < B; b += T) buckets[b] = 0u;
        if (kTree)
            for (uint32_t bi = r; bi < W.nb; bi += T) S.bodyTotal[W.bodyOff + bi] = 0u;
    }
    float cw = team.fmax(cwl);
    cw = fmaxf(cw, kFltMin);
    if (!kGridTeam<Team>) {
        for (uint32_t b = r; b < B; b += T) buckets[b] = 0u;
        if (kTree)
            for (uint32_t bi = r; bi < W.nb; bi += T) S.bodyTotal[W.bodyOff + bi] = 0u;
        team.sync();
    }
    BP_SUBPHASE(13);
    // cells (nativeBuildGrid, NGK:179-189) and bucket counts
    for (uint32_t i = r; i < n; i += T) {
        uint32_t g = W.boff + i;
        uint32_t f = S.flags[g] & ~kValid;
        float2 p = S.pos[g];
        bool valid = !(f & kRemoved) && finite2(p);
        long long cx = 0, cy = 0;
        if (valid) {
            cx = (long long)clampf(floorf(p.x / cw), -4.0e18f, 4.0e18f);
            cy = (long long)clampf(floorf(p.y / cw), -4.0e18f, 4.0e18f);
            f |= kValid;
            atomicAdd(buckets + grid_hash(cx, cy, B), 1u);
        }
        S.cell[g] = make_longlong2(cx, cy);
        S.flags[g] = f;
    }
    team.sync();
    team.scan_inplace(buckets, B);
    for (uint32_t i = r; i < n; i += T) {
        uint32_t g = W.boff + i;
        if (!(S.flags[g] & kValid)) continue;
        longlong2 cc = S.cell[g];
        uint32_t slot = atomicAdd(buckets + grid_hash(cc.x, cc.y, B), 1u);
        entries[slot] = i;
        const float2 p = S.pos[g];
        records[slot] = make_float4(p.x, p.y, S.phys[g].x, S.margin[g]);
    }
    team.sync();
    BP_SUBPHASE(14);
    uint32_t overflow = 0, maxPer = 0;
    for (uint32_t i = r; i < n; i += T)
        emit_row<kTree, kGridTeam<Team>>(S, W, buckets, entries, records, B, cw, i, overflow, maxPer);
    team.sync();
    BP_SUBPHASE(15);
    {
        const uint32_t lane = threadIdx.x & 31u, warp = r >> 5, warps = T >> 5;
        if (kTree)
            for (uint32_t bi = warp; bi < W.nb; bi += warps) fix_body_row(S, W, bi, lane, overflow, maxPer);
        else
            for (uint32_t bi = warp; bi < W.nb; bi += warps) emit_body_row(S, W, bi, lane, overflow, maxPer);
    }
    // body rows are read by the adjacency rows; without bodies the whole-GPU team skips this grid barrier (the
    // candidate rows' barrier is above). The block and group teams keep it: removing it measured slower there.
    if (W.nb || !kGridTeam<Team>) team.sync();
    BP_SUBPHASE(16);
    for (uint32_t i = r; i < n; i += T) build_adjacency<kTree>(S, W, buckets, entries, B, i, overflow, maxPer);
    team.sync();
    BP_SUBPHASE(17);
    uint32_t red[4] = {overflow, maxPer, 0u, 0u};
    team.template reduce4<2u>(red);
    buildOverflow = red[0];
    maxPerAll = max(maxPerAll, red[1]);
    BP_SUBPHASE(18);
    return cw;
}

// Contact forces from the current state, then the start-of-build acceleration (phase 2, NFK:776-779). Also gives
// each thread its share of the first reduction: (max omega^2, owner) and (min margin bound, owner). `slots` holds one
// float4 per thread of the team (the row terms of warp_rows).
template <class Team>
__device__ void initial_forces(const DState& S, const DWorld& W, const Ctl& c, const Team& team, ValOwner& w2, ValOwner& mg,
                               float4* slots) {
    const float fraction = c.timeX > 0.0f ? clampf(c.timeY / c.timeX, 0.0f, 1.0f) : 1.0f;
    if (W.nb) {
        refresh_poses(S, W, team, fraction);
        team.sync();
    }
    w2 = ValOwner{-1.0f, 0u};
    mg = ValOwner{__int_as_float(0x7f800000), 0u};
    const uint32_t lane = team.rank() & 31u;
    for (uint32_t i0 = team.rank() - lane; i0 < W.n; i0 += team.size()) {  // the whole warp iterates together
        const uint32_t i = i0 + lane, g = W.boff + i;
        const bool has = i < W.n && !removed(S, g);
        float im = has ? inv_mass(S, g) : 0.0f, omega2;
        float2 F = warp_contact_terms(S, W, i0, has, im, slots + (team.rank() - lane), omega2);
        if (!has) continue;
        S.acc[g] = add(mul(F, im), S.a0[g]);
        if (omega2 > w2.v) { w2.v = omega2; w2.o = i; }
        float m = margin_bound(S, g);
        if (m < mg.v) { mg.v = m; mg.o = i; }
    }
    // the next reduction's barrier orders these writes before any reader; the whole-GPU team saves this grid barrier
    if (!kGridTeam<Team>) team.sync();
}

// nativeReduceSubstepInGroup, NFK:625-736
template <class Team>
__device__ void reduce_substep(const DState& S, const DWorld& W, Ctl& c, const Team& team, float* history, ValOwner w2,
                               ValOwner mg, float4* slots) {
    const float inf = __int_as_float(0x7f800000);
    float remaining = c.timeX - c.timeY;
    bool over = !(remaining > 0.0f), stopped = c.cZ != 0u || c.cW != 0u, limited = c.cY >= kFrameLimit;
    if (over || stopped || limited) {
        if (limited && !over && !stopped) c.cW = 1u;
        c.timeZ = 0.0f;
        return;
    }
    const float fraction = c.timeX > 0.0f ? clampf(c.timeY / c.timeX, 0.0f, 1.0f) : 1.0f;
    if (W.flags & BP_WORLD_INJECT_STATE) {
        // an injected position invalidates the partials of the force pass: evaluate the terms afresh
        w2 = ValOwner{-1.0f, 0u};
        mg = ValOwner{inf, 0u};
        for (uint32_t i = team.rank(); i < W.n; i += team.size()) {
            uint32_t g = W.boff + i;
            if (removed(S, g)) continue;
            float v = omega_squared(S, W, i, fraction);
            if (v > w2.v) { w2.v = v; w2.o = i; }
            float m = margin_bound(S, g);
            if (m < mg.v) { mg.v = m; mg.o = i; }
        }
    }
    team.template pick2<true, false>(w2, mg);
    const float stiffnessBound = w2.v > 0.0f ? 1.0f / sqrtf(w2.v) : inf;
    const float hMax = fminf(remaining, stiffnessBound);
    ValOwner db{inf, 0u};
    const uint32_t lane = team.rank() & 31u;
    for (uint32_t i0 = team.rank() - lane; i0 < W.n; i0 += team.size()) {  // the whole warp iterates together
        const uint32_t i = i0 + lane;
        const bool has = i < W.n && !removed(S, W.boff + i);
        float v = warp_distance_bound(S, W, i0, has, hMax, slots + (team.rank() - lane));
        if (has && v < db.v) { db.v = v; db.o = i; }
    }
    db = team.template pick<false>(db);
    if (mg.v <= 0.0f) {
        c.cZ = 1u;
        c.timeZ = 0.0f;
        c.limObj = S.id[W.boff + mg.o];
        c.limTerm = BP_TERM_MARGIN;
        return;
    }
    float split = fmaxf(c.timeW, 1.0f);
    float h = remaining;
    uint32_t term = BP_TERM_REMAINING;
    int64_t object = 0;
    if (split > 1.0f && c.timeX / split < h) h = c.timeX / split;
    if (stiffnessBound / split < h) { h = stiffnessBound / split; term = BP_TERM_STIFFNESS; object = S.id[W.boff + w2.o]; }
    if (db.v / split < h) { h = db.v / split; term = BP_TERM_DISTANCE; object = S.id[W.boff + db.o]; }
    if (mg.v < h) { h = mg.v; term = BP_TERM_MARGIN; object = S.id[W.boff + mg.o]; c.cZ = 1u; }
    h = fmaxf(h, c.timeX * 1e-7f);
    uint32_t frameSubstep = c.cY;
    if (h >= remaining || remaining - h <= c.timeX * 1e-5f) { h = remaining; c.timeY = c.timeX; }
    else c.timeY = c.timeY + h;
    c.timeZ = h;
    c.cX += 1u;
    c.cY = frameSubstep + 1u;
    c.limObj = object;
    c.limTerm = term;
    if (team.leader() && frameSubstep < kFrameLimit) history[frameSubstep] = h;
}

// Phase 0 of nativeIntegratePhase (NFK:784-797): half kick with the previous acceleration, drift, rotation.
__device__ __forceinline__ void kick_drift(const DState& S, const DWorld& W, uint32_t i, float h) {
    const uint32_t g = W.boff + i;
    float im = inv_mass(S, g);
    if (!(im > 0.0f)) return;
    uint32_t f = S.flags[g];
    float halfStep = 0.5f * h;
    float gamma = (f & BP_BUBBLE_FORCE_DRIVEN) ? fmaxf(S.phys[g].w, 0.0f) : 0.0f;
    float decay = expf(-gamma * halfStep), factor = half_impulse(gamma, halfStep);
    float2 velocity = add(mul(S.vel[g], decay), mul(S.acc[g], factor));
    float2 rw = S.rotw[g];
    float angular = rw.y * expf(-gamma * h);
    if (W.nmotors && (f & BP_BUBBLE_FORCE_DRIVEN)) {
        const bp_motor* motor = find_by_bubble(S.motors + W.motorOff, W.nmotors, S.id[g]);
        if (motor && motor->inertia > 0.0f) angular = angular + motor->torque / motor->inertia * half_impulse(gamma, h);
    }
    S.pos[g] = add(S.pos[g], mul(velocity, h));
    S.vel[g] = velocity;
    S.rotw[g] = f2(rw.x + rw.y * h, angular);
}

// Contact forces from the new state and phase 1 (NFK:798-801): a = F / m + a0(x), second half kick. The same pass
// gives omega^2 and the margin bound of the next reduction (same positions, velocities and accelerations it would read).
// Bubble i0 + lane of every lane of the warp (`has`: the lane's bubble is live); the whole warp calls this together.
__device__ __forceinline__ void force_kick(const DState& S, const DWorld& W, uint32_t i0, bool has, float h,
                                           ValOwner& w2, ValOwner& mg, float4* slots) {
    const uint32_t i = i0 + (threadIdx.x & 31u), g = W.boff + i;
    const float im = has ? inv_mass(S, g) : 0.0f;
    float omega2;
    float2 F = warp_contact_terms(S, W, i0, has && im > 0.0f, im, slots, omega2);
    if (!has) return;
    if (!(im > 0.0f)) {
        if (0.0f > w2.v) { w2.v = 0.0f; w2.o = i; }
        return;
    }
    uint32_t f = S.flags[g];
    float halfStep = 0.5f * h;
    float gamma = (f & BP_BUBBLE_FORCE_DRIVEN) ? fmaxf(S.phys[g].w, 0.0f) : 0.0f;
    float decay = expf(-gamma * halfStep), factor = half_impulse(gamma, halfStep);
    float2 a = add(mul(F, im), non_contact_acc(S, W, g, S.pos[g]));
    S.vel[g] = add(mul(S.vel[g], decay), mul(a, factor));
    S.acc[g] = a;
    if (omega2 > w2.v) { w2.v = omega2; w2.o = i; }
    float m = margin_bound(S, g);
    if (m < mg.v) { mg.v = m; mg.o = i; }
}

// ------------------------------------------------------------------------------------------------------------------
// Contact assertion (NFK:865-918): the violation of the lowest bubble index.
// ------------------------------------------------------------------------------------------------------------------
struct Viol {
    uint32_t kind;
    int64_t a, b, edge;
    float distance;
};

template <bool kTree>
__device__ bool assert_bubble(const DState& S, const DWorld& W, const uint32_t* buckets, const uint32_t* entries, uint32_t B,
                              float fraction, uint32_t i, bool fromCandidates, Viol& v) {
    const uint32_t g = W.boff + i;
    float2 center = S.pos[g], start = S.start[g];
    if (!finite2(center) || S.result[g] == 1u || removed(S, g)) return false;
    bool movable = inv_mass(S, g) > 0.0f;
    uint2 fi = S.filter[g];
    uint32_t bestJ = 0xffffffffu;
    float bestD = 0.0f;
    auto checkPair = [&](uint32_t j) {
        if (j <= i || j >= bestJ) return;
        uint32_t gj = W.boff + j;
        if (S.result[gj] == 1u || removed(S, gj)) return;
        if (!filter_accepts(fi, S.filter[gj])) return;
        if (!movable && !(inv_mass(S, gj) > 0.0f)) return;
        float d = len2(sub(S.pos[gj], center));
        if (d <= 0.0f) { bestJ = j; bestD = d; }
    };
    if (fromCandidates) {
        // pairs with d <= 0 are candidates of the last build (see assert_contacts)
        const uint32_t* crow = S.candRow + W.rowOff + (uint64_t)i * W.k;
        const uint32_t pairs = S.candCount[g].x;
        for (uint32_t e = 0; e < pairs; ++e) checkPair(crow[e]);
    } else {
        // pairs with d <= 0 have coincident centres: same or adjacent cell of the current-position grid
        longlong2 c = S.acell[g];
        for (int dx = -1; dx <= 1; ++dx)
            for (int dy = -1; dy <= 1; ++dy)
                for_each_in_cell(S.acell, W, buckets, entries, B, c.x + dx, c.y + dy, checkPair);
    }
    if (bestJ != 0xffffffffu) {
        v.kind = BP_VIOLATION_PAIR; v.a = S.id[g]; v.b = S.id[W.boff + bestJ]; v.edge = 0; v.distance = bestD;
        return true;
    }
    if (!movable) return false;
    // a centre inside the body lies inside its swept box widened to the hull radius (conservative slack for the
    // rounding of the interpolated pose)
    const float cs = 1e-3f + 1e-5f * fmaxf(fabsf(center.x), fabsf(center.y));
    auto insideBody = [&](uint32_t bi) {
        const RigidBox rb = S.bodyBox[W.bodyOff + bi];
        if (!filter_accepts(fi, make_uint2(rb.cat, rb.mask))) return false;
        const float extra = __uint_as_float(rb.pad);
        if (center.x < rb.box.x - extra - cs || center.y < rb.box.y - extra - cs || center.x > rb.box.z + extra + cs ||
            center.y > rb.box.w + extra + cs)
            return false;
        const DBody& b = S.body[W.bodyOff + bi];
        Pose pose = body_at(b, fraction);
        return rigid_inside(S.bverts, S.btris, center, b, pose);
    };
    // the reported body is the lowest index the centre is inside of, whichever way the bodies are visited
    uint32_t insideOf = 0xffffffffu;
    if (kTree) {
        if (W.nb)
            tree_query(S, W,
                       [&](float4 nb) {
                           return !(center.x < nb.x - cs || center.y < nb.y - cs || center.x > nb.z + cs ||
                                    center.y > nb.w + cs);
                       },
                       [&](uint32_t leaf) {
                           if (leaf < W.s || leaf - W.s >= insideOf) return;
                           if (insideBody(leaf - W.s)) insideOf = leaf - W.s;
                       });
    } else {
        for (uint32_t bi = 0; bi < W.nb; ++bi)
            if (insideBody(bi)) { insideOf = bi; break; }
    }
    if (insideOf != 0xffffffffu) {
        v.kind = BP_VIOLATION_INSIDE_BODY; v.a = S.id[g]; v.b = S.body[W.bodyOff + insideOf].id; v.edge = 0; v.distance = 0.0f;
        return true;
    }
    // a crossing point lies on both the chord start -> centre and the edge: their boxes must overlap (conservative
    // margin for rounding) before the exact test runs
    const float2 pathLo = vmin2(start, center), pathHi = vmax2(start, center);
    const float slack = 1e-3f + 1e-5f * fmaxf(fmaxf(fabsf(pathLo.x), fabsf(pathLo.y)), fmaxf(fabsf(pathHi.x), fabsf(pathHi.y)));
    auto crossesEdge = [&](uint32_t e, float& after) {
        const RigidBox rb = S.segBox[W.soff + e];
        if (!(rb.flags & BP_SEGMENT_POLYGON_EDGE)) return false;
        if (rb.box.x > pathHi.x + slack || rb.box.y > pathHi.y + slack || rb.box.z < pathLo.x - slack ||
            rb.box.w < pathLo.y - slack)
            return false;
        if (!filter_accepts(fi, make_uint2(rb.cat, rb.mask))) return false;
        const DSegment& sg = S.seg[W.soff + e];
        float2 edge = sub(sg.b, sg.a);
        float lsq = dot2(edge, edge);
        if (!(lsq > 0.0f)) return false;
        float2 outward = mul(dvd(f2(-edge.y, edge.x), sqrtf(lsq)), sg.outward);
        float before = dot2(sub(start, sg.a), outward);
        after = dot2(sub(center, sg.a), outward);
        if (!(before > 0.0f) || !(after <= 0.0f)) return false;
        float2 crossing = add(start, mul(sub(center, start), before / (before - after)));
        float along = dot2(sub(crossing, sg.a), edge) / lsq;
        return !(along < 0.0f || along > 1.0f);
    };
    // the reported edge is the lowest segment index crossed
    uint32_t crossed = 0xffffffffu;
    float crossedAfter = 0.0f;
    if (kTree) {
        if (W.s)
            tree_query(S, W,
                       [&](float4 nb) {
                           return !(nb.x > pathHi.x + slack || nb.y > pathHi.y + slack || nb.z < pathLo.x - slack ||
                                    nb.w < pathLo.y - slack);
                       },
                       [&](uint32_t leaf) {
                           float after;
                           if (leaf >= W.s || leaf >= crossed) return;
                           if (crossesEdge(leaf, after)) { crossed = leaf; crossedAfter = after; }
                       });
    } else {
        for (uint32_t e = 0; e < W.s; ++e) {
            float after;
            if (crossesEdge(e, after)) { crossed = e; crossedAfter = after; break; }
        }
    }
    if (crossed != 0xffffffffu) {
        const DSegment& sg = S.seg[W.soff + crossed];
        v.kind = BP_VIOLATION_EDGE_SIDE; v.a = S.id[g]; v.b = sg.owner; v.edge = sg.id; v.distance = crossedAfter;
        return true;
    }
    return false;
}

// Hash grid of the current centres (cells of width cw) for the assertion; reuses the bucket memory and keeps its own
// cells so the cells of the last build stay readable.
template <class Team>
__device__ void assertion_grid(const DState& S, const DWorld& W, const Team& team, uint32_t* buckets, uint32_t* entries,
                               uint32_t B, float cw) {
    const uint32_t n = W.n, T = team.size(), r = team.rank();
    const long long none = (long long)0x8000000000000000ull;
    for (uint32_t b = r; b < B; b += T) buckets[b] = 0u;
    team.sync();
    for (uint32_t i = r; i < n; i += T) {
        uint32_t g = W.boff + i;
        float2 p = S.pos[g];
        long long cx = none, cy = 0;
        if (!removed(S, g) && finite2(p)) {
            cx = (long long)clampf(floorf(p.x / cw), -4.0e18f, 4.0e18f);
            cy = (long long)clampf(floorf(p.y / cw), -4.0e18f, 4.0e18f);
            atomicAdd(buckets + grid_hash(cx, cy, B), 1u);
        }
        S.acell[g] = make_longlong2(cx, cy);
    }
    team.sync();
    team.scan_inplace(buckets, B);
    for (uint32_t i = r; i < n; i += T) {
        uint32_t g = W.boff + i;
        longlong2 cc = S.acell[g];
        if (cc.x == none) continue;
        entries[atomicAdd(buckets + grid_hash(cc.x, cc.y, B), 1u)] = i;
    }
    team.sync();
}

// Runs the assertion over the world; the thread that owns the violating bubble of the lowest index writes the details
// into the report. Returns 1 in every thread when a violation exists.
// The pair part can use the candidate rows of the last build instead of a fresh grid when that is complete: two
// centres closer than any rounding can only meet if their build positions were within m_i + m_j plus the distance each
// moved since the build, so when every bubble is within margin + r/2 of its build position the pair passed the
// candidate test (reach = r_i + r_j + m_i + m_j + sepTol). Truncated rows, joint exclusions, injected states and region
// wraps void that argument and take the grid path.
template <class Team, bool kTree>
__device__ uint32_t assert_contacts(const DState& S, const DWorld& W, const Team& team, uint32_t* buckets, uint32_t* entries,
                                    uint32_t B, float cw, float fraction, bp_step_report* rep, bool rowsComplete) {
    uint32_t unsafe = (!rowsComplete || W.njEnt || (W.flags & BP_WORLD_INJECT_STATE)) ? 1u : 0u;
    if (!unsafe) {
        for (uint32_t i = team.rank(); i < W.n; i += team.size()) {
            uint32_t g = W.boff + i;
            if (removed(S, g)) continue;
            if (S.result[g] == 2u || !(len2(sub(S.pos[g], S.ref[g])) <= S.margin[g] + 0.5f * S.phys[g].x)) unsafe = 1u;
        }
        unsafe = team.umax(unsafe);
    }
    const bool fromCandidates = unsafe == 0u;
    if (!fromCandidates) assertion_grid(S, W, team, buckets, entries, B, cw);
    Viol mine{0u, 0, 0, 0, 0.0f};
    ValOwner first{__int_as_float(0x7f800000), 0xffffffffu};
    for (uint32_t i = team.rank(); i < W.n; i += team.size()) {
        Viol v;
        if (assert_bubble<kTree>(S, W, buckets, entries, B, fraction, i, fromCandidates, v)) {
            first.v = 0.0f;
            first.o = i;
            mine = v;
            break;  // later indices of this thread are larger
        }
    }
    ValOwner winner = team.template pick<false>(first);
    if (winner.o != 0xffffffffu && winner.o == first.o) {
        rep->violation_kind = mine.kind;
        rep->violation_objects[0] = mine.a;
        rep->violation_objects[1] = mine.b;
        rep->violation_edge = mine.edge;
        rep->violation_distance = mine.distance;
    }
    return winner.o != 0xffffffffu ? 1u : 0u;
}

// ------------------------------------------------------------------------------------------------------------------
// End of step: region (NPK:536-568), contact records (NGK:683-728 + NCK:146-160 + NFK:261-280)
// ------------------------------------------------------------------------------------------------------------------
__device__ bool apply_region(const DState& S, const DWorld& W, uint32_t g, uint32_t& removedCount, uint32_t& wrapped) {
    uint32_t f = S.flags[g];
    if ((f & kRemoved) || !(f & BP_BUBBLE_ENABLED) || (f & BP_BUBBLE_STATIC)) return true;
    float2 p = S.pos[g];
    float r = S.phys[g].x;
    float2 nearest = vmin2(vmax2(p, W.rmin), W.rmax);
    if (len2(sub(p, nearest)) <= r) return true;
    if (!(f & BP_BUBBLE_WRAP)) { S.result[g] = 1u; ++removedCount; return true; }
    float2 span = add(sub(W.rmax, W.rmin), f2(2.0f * r, 2.0f * r));
    float dl[2] = {0.0f, 0.0f};
    float pp[2] = {p.x, p.y}, lo[2] = {W.rmin.x, W.rmin.y}, hi[2] = {W.rmax.x, W.rmax.y}, sp[2] = {span.x, span.y};
#pragma unroll
    for (int axis = 0; axis < 2; ++axis) {
        if (pp[axis] > hi[axis]) dl[axis] = -sp[axis] * fmaxf(1.0f, ceilf((pp[axis] - r - hi[axis]) / sp[axis]));
        else if (pp[axis] < lo[axis]) dl[axis] = sp[axis] * fmaxf(1.0f, ceilf((lo[axis] - r - pp[axis]) / sp[axis]));
    }
    float2 delta = f2(dl[0], dl[1]);
    float2 w = add(p, delta);
    float2 nw = vmin2(vmax2(w, W.rmin), W.rmax);
    if (len2(sub(w, nw)) > r) delta = add(delta, sub(nw, w));
    float2 np = add(p, delta), ns = add(S.start[g], delta);
    S.pos[g] = np;
    S.start[g] = ns;
    if (!finite2(np) || !finite2(ns)) return false;
    S.result[g] = 2u;
    ++wrapped;
    return true;
}

// Contact record of candidate (i, kind, other); returns false when inactive (penetration <= -sepTol). With kFull
// false only the activity is decided (the geometry up to the penetration; no law, nothing written): the counting pass.
template <bool kFull>
__device__ bool contact_record(const DState& S, const DWorld& W, uint32_t i, uint32_t kind, uint32_t other, DContact& out) {
    const uint32_t g = W.boff + i;
    float2 apos = S.pos[g];
    float4 pa = S.phys[g];
    float ar = pa.x;
    float2 normal, point;
    float pen, allowed = 0.0f;
    uint32_t feature = 0;
    if (kind == 0u) {
        uint32_t go = W.boff + other;
        float2 delta = sub(S.pos[go], apos);
        float d = len2(delta);
        normal = d > 0.0f ? dvd(delta, d) : f2(1.0f, 0.0f);
        point = add(apos, mul(normal, ar));
        pen = ar + S.phys[go].x - d;
    } else {
        const DSegment& sg = S.seg[W.soff + other];
        float2 edge = sub(sg.b, sg.a);
        float lsq = dot2(edge, edge);
        float t = lsq > 0.0f ? clampf(dot2(sub(apos, sg.a), edge) / lsq, 0.0f, 1.0f) : 0.0f;
        point = add(sg.a, mul(edge, t));
        float2 delta = sub(apos, point);
        float d = len2(delta), edgeLength = len2(edge);
        float2 base = edgeLength > 0.0f ? dvd(f2(-edge.y, edge.x), edgeLength) : f2(0.0f, 1.0f);
        float sign = ((S.id[g] ^ sg.id) & 1) == 0 ? 1.0f : -1.0f;
        bool fixedSide = (sg.flags & BP_SEGMENT_ALLOWED_SIDE) != 0u;
        normal = fixedSide ? mul(base, sg.allowed) : (d > 0.0f ? dvd(delta, d) : mul(base, sign));
        allowed = fixedSide ? sg.allowed : 0.0f;
        pen = ar - d;
        if (sg.flags & BP_SEGMENT_POLYGON_EDGE) {
            float2 outward = mul(base, sg.outward);
            float2 start = sg.a, end = sg.b;
            float along = dot2(sub(apos, start), sub(end, start));
            bool convexStart = (sg.flags & BP_SEGMENT_CONVEX_START) != 0u;
            if (convexStart && along <= 0.0f && past_segment_end(apos, sg.prev, start)) feature = 2u;
            else {
                bool interior = along > 0.0f && !past_segment_end(apos, start, end);
                feature = dot2(sub(apos, start), outward) >= 0.0f && interior ? 1u : 0u;
            }
            if (feature == 1u) {
                normal = outward;
                point = sub(apos, mul(outward, dot2(sub(apos, sg.a), outward)));
                pen = ar - dot2(sub(apos, sg.a), outward);
            } else if (feature == 2u) {
                point = sg.a;
                delta = sub(apos, point);
                d = len2(delta);
                normal = d > 0.0f ? dvd(delta, d) : outward;
                pen = ar - d;
            } else {
                normal = outward;
                point = sg.a;
                pen = -kFltMax;
            }
        }
    }
    if (!(pen > -W.sepTol)) return false;
    if (!kFull) return true;
    float force;
    if (kind == 0u) {
        float4 pb = S.phys[W.boff + other];
        force = pair_law(pa.z, ar, pb.z, pb.x, ar + pb.x - pen).force;
    } else {
        force = wall_law(pa.z, ar, ar - pen).force;
    }
    out.a = i;
    out.other = other;
    out.kind = kind;
    out.feature = feature;
    out.normal = normal;
    out.point = point;
    out.impulse = force * W.dt * W.dt;
    out.penetration = pen;
    out.allowed = allowed;
    return true;
}

// ------------------------------------------------------------------------------------------------------------------
// Shared-memory residency: a team that owns a small enough world keeps the world's hot state in its shared-memory
// workspace for the whole step (staged in here, written back when the step publishes). S is redirected so the same
// per-bubble code indexes shared memory; worlds that do not fit run the identical code on global memory.
// ------------------------------------------------------------------------------------------------------------------
template <class T> __device__ __forceinline__ T* carve(char*& p, uint32_t count) {
    T* out = (T*)p;
    p += ((size_t)count * sizeof(T) + 15u) & ~(size_t)15u;
    return out;
}

template <class Team>
__device__ bool stage_world(const DState& G, DState& S, const DWorld& W, const Team& team, uint32_t* ws, uint32_t wsWords) {
    if (ws == nullptr || workspace_bytes(W.n, W.s, W.nb) > wsWords * 4u) return false;
    const uint32_t n = W.n, T = team.size(), r = team.rank();
    char* p = (char*)ws;
    float4* phys = carve<float4>(p, n);
    float2* pos = carve<float2>(p, n);
    float2* vel = carve<float2>(p, n);
    float2* acc = carve<float2>(p, n);
    float2* ref = carve<float2>(p, n);
    float2* a0 = carve<float2>(p, n);
    uint2* filter = carve<uint2>(p, n);
    uint2* candCount = carve<uint2>(p, n);
    float* margin = carve<float>(p, n);
    uint32_t* flags = carve<uint32_t>(p, n);
    uint32_t* deg = carve<uint32_t>(p, n);
    uint32_t* pairTotal = carve<uint32_t>(p, n);
    RigidBox* segBox = carve<RigidBox>(p, W.s);
    RigidBox* bodyBox = carve<RigidBox>(p, W.nb);
    float4* bpose = carve<float4>(p, W.nb);
    for (uint32_t i = r; i < n; i += T) {
        uint32_t g = W.boff + i;
        phys[i] = G.phys[g];
        pos[i] = G.pos[g];
        vel[i] = G.vel[g];
        filter[i] = G.filter[g];
        flags[i] = G.flags[g];
    }
    if (team.shared_leader()) {  // S lives in the team's shared memory: one thread redirects it
        S.phys = phys - W.boff;
        S.pos = pos - W.boff;
        S.vel = vel - W.boff;
        S.acc = acc - W.boff;
        S.ref = ref - W.boff;
        S.a0 = a0 - W.boff;
        S.filter = filter - W.boff;
        S.candCount = candCount - W.boff;
        S.margin = margin - W.boff;
        S.flags = flags - W.boff;
        S.deg = deg - W.boff;
        S.pairTotal = pairTotal - W.boff;
        S.segBox = segBox - W.soff;
        S.bodyBox = bodyBox - W.bodyOff;
        S.bpose = bpose - W.bodyOff;
    }
    team.sync();
    return true;
}

// Boxes of the world's segments and (after the kinematic advance) bodies for this step.
template <class Team> __device__ void build_boxes(const DState& S, const DWorld& W, const Team& team) {
    for (uint32_t j = team.rank(); j < W.s; j += team.size()) {
        const DSegment& sg = S.seg[W.soff + j];
        float2 lo = vmin2(sg.a, sg.b), hi = vmax2(sg.a, sg.b);
        RigidBox rb;
        rb.box = make_float4(lo.x, lo.y, hi.x, hi.y);
        rb.cat = sg.cat; rb.mask = sg.mask; rb.flags = sg.flags; rb.pad = 0u;
        S.segBox[W.soff + j] = rb;
    }
    for (uint32_t bi = team.rank(); bi < W.nb; bi += team.size()) {
        const DBody& b = S.body[W.bodyOff + bi];
        float2 lo = sub(vmin2(b.pos, b.prev), f2(b.radius, b.radius));
        float2 hi = add(vmax2(b.pos, b.prev), f2(b.radius, b.radius));
        RigidBox rb;
        rb.box = make_float4(lo.x, lo.y, hi.x, hi.y);
        rb.cat = b.cat; rb.mask = b.mask; rb.flags = body_is_obstacle(b) ? 1u : 0u;
        rb.pad = __float_as_uint(fmaxf(b.pad - b.radius, 0.0f));  // hull radius beyond the bounding radius
        S.bodyBox[W.bodyOff + bi] = rb;
    }
}

// ------------------------------------------------------------------------------------------------------------------
// One complete step of one world (nativeBeginStep -> substep loop -> end of step)
// ------------------------------------------------------------------------------------------------------------------
// `ts` is the team's TeamState in shared memory (ts.S and ts.W are written here; G may be ts.G).
template <class Team, bool kTreeCapable>
__device__ void world_step(const DState& G, uint32_t wi, const Team& team, uint32_t* buckets, uint32_t* entries,
                           float4* records, uint32_t B,
                           uint32_t* ws, uint32_t wsWords, TeamState& ts) {
    if (team.shared_leader()) {
        ts.W = G.worlds[wi];
        ts.S = G;
    }
    team.shared_sync();
    const DWorld& W = ts.W;
    const uint32_t n = W.n, T = team.size(), r = team.rank();
    bp_step_report* rep = G.reports + wi;
    if (G.failed[wi]) {
        if (team.leader()) { rep->status = BP_E_WORLD_FAILED; rep->substep_count = 0u; }
        team.sync();
        return;
    }
    DState& S = ts.S;
    BP_STAMP(G, 24);
    stage_world(G, S, W, team, ws, wsWords);
    BP_PHASE_START;
    // nativeBeginStep (NFK:285-293)
    uint32_t liveLocal = 0;
    for (uint32_t i = r; i < n; i += T) {
        uint32_t g = W.boff + i;
        uint32_t f = S.flags[g];
        if (f & kRemoved) continue;
        ++liveLocal;
        S.result[g] = 0u;
        const float2 p0 = S.pos[g];
        S.start[g] = p0;
        S.flags[g] = finite2(p0) ? (f | kStartFinite) : (f & ~kStartFinite);
        if ((f & BP_BUBBLE_ENABLED) && (f & BP_BUBBLE_STATIC)) {
            S.vel[g] = f2(0.0f, 0.0f);
            S.rotw[g].y = 0.0f;
        }
    }
    // kinematic advance of static / kinematic bodies (nativeRigidPredict, NPK:65-80)
    for (uint32_t bi = r; bi < W.nb; bi += T) {
        DBody b = S.body[W.bodyOff + bi];
        b.prev = b.pos;
        b.prevAngle = b.angle;
        b.cosPrev = b.cosEnd;
        b.sinPrev = b.sinEnd;
        if (b.flags & BP_BODY_STATIC) {
            b.vel = f2(0.0f, 0.0f);
            b.omega = 0.0f;
        } else {
            b.pos = add(b.pos, mul(b.vel, W.dt));
            b.angle = b.angle + b.omega * W.dt;
            if (b.angle != b.prevAngle) { b.cosEnd = cosf(b.angle); b.sinEnd = sinf(b.angle); }
        }
        S.body[W.bodyOff + bi] = b;
    }
    team.sync();
    build_boxes(S, W, team);
    const uint32_t live = team.sum(liveLocal);
    // the tree-capable instantiation carries the LBVH code; a kernel for worlds without trees is compiled without it
    const bool useTree = kTreeCapable && W.tree && build_rigid_tree(S, W, wi, team);
    Ctl c;
    c.timeX = W.dt;
    c.timeY = live == 0u ? W.dt : 0.0f;
    c.timeZ = 0.0f;
    c.timeW = W.split;
    c.cX = c.cY = c.cZ = c.cW = 0u;
    c.limObj = 0;
    c.limTerm = 0u;
    float* history = S.history + (uint64_t)wi * kFrameLimit;
    uint32_t buildOverflow = 0, overflowMax = 0, maxPer = 0, rebuilds = 0;
    BP_PHASE(0);
    float cw = useTree ? broadphase<Team, true>(S, W, c, team, buckets, entries, records, B, buildOverflow, maxPer, wi)
                       : broadphase<Team, false>(S, W, c, team, buckets, entries, records, B, buildOverflow, maxPer, wi);
    BP_PHASE(1);
    ValOwner w2, mg;
    initial_forces(S, W, c, team, w2, mg, records);
    BP_PHASE(2);
    uint32_t violated = 0u;
    for (uint32_t iteration = 0; iteration < 2u * kFrameLimit + 2u; ++iteration) {
        if (!team.ok()) break;
        reduce_substep(S, W, c, team, history, w2, mg, records);
        BP_PHASE(3);
        const float h = c.timeZ;
        const bool limited = c.cW != 0u, finished = !(c.timeX - c.timeY > 0.0f), rebuild = c.cZ != 0u;
        if (!(h > 0.0f)) {
            if (limited || finished || !rebuild) break;
            c.cX = 0u;
            c.cZ = 0u;
            overflowMax = max(overflowMax, buildOverflow);
            ++rebuilds;
            cw = useTree ? broadphase<Team, true>(S, W, c, team, buckets, entries, records, B, buildOverflow, maxPer, wi)
                         : broadphase<Team, false>(S, W, c, team, buckets, entries, records, B, buildOverflow, maxPer, wi);
            initial_forces(S, W, c, team, w2, mg, records);
            BP_PHASE(1);
            continue;
        }
        const float fraction = c.timeX > 0.0f ? clampf(c.timeY / c.timeX, 0.0f, 1.0f) : 1.0f;
        for (uint32_t i = r; i < n; i += T)
            if (!removed(S, W.boff + i)) kick_drift(S, W, i, h);
        refresh_poses(S, W, team, fraction);
        team.sync();
        w2 = ValOwner{-1.0f, 0u};
        mg = ValOwner{__int_as_float(0x7f800000), 0u};
        for (uint32_t i0 = r - (r & 31u); i0 < n; i0 += T) {  // the whole warp iterates together
            const uint32_t i = i0 + (r & 31u);
            force_kick(S, W, i0, i < n && !removed(S, W.boff + i), h, w2, mg, records + (r - (r & 31u)));
        }
        // The whole-GPU team needs no barrier here: whatever reads other bubbles' new state next (the next reduction,
        // an injection, the assertion, the end of the step, a rebuild's grid reductions) passes one first, and the
        // body poses the force pass reads are rewritten only behind several. The block and group teams keep it:
        // removing it measured slower there.
        if (!kGridTeam<Team>) team.sync();
        BP_PHASE(4);
        if (W.flags & BP_WORLD_INJECT_STATE) {
            if (c.cY == W.injectSubstep + 1u)
                for (uint32_t i = r; i < n; i += T)
                    if (S.id[W.boff + i] == W.injectObject) S.pos[W.boff + i] = W.injectPos;
            team.sync();
        }
        if ((W.flags & BP_WORLD_ASSERT_EVERY_SUBSTEP) && !violated) {
            const float at = c.timeX > 0.0f ? clampf(c.timeY / c.timeX, 0.0f, 1.0f) : 1.0f;
            violated = useTree ? assert_contacts<Team, true>(S, W, team, buckets, entries, B, cw, at, rep, buildOverflow == 0u)
                               : assert_contacts<Team, false>(S, W, team, buckets, entries, B, cw, at, rep, buildOverflow == 0u);
        }
    }
    overflowMax = max(overflowMax, buildOverflow);
    BP_PHASE(5);

    // ---- end of step ----
    uint32_t removedCount = 0, wrapped = 0, nonfinite = 0;
    const bool stepDone = c.cW == 0u;
    if (stepDone && (W.flags & BP_WORLD_HAS_REGION))
        for (uint32_t i = r; i < n; i += T)
            if (!apply_region(S, W, W.boff + i, removedCount, wrapped)) nonfinite = 1u;
    team.sync();
    // contact records: count per bubble, scan, write (kind-major candidate order)
    uint32_t pairsLocal = 0, segsLocal = 0;
    const uint32_t lane = r & 31u;
    if (!kGridTeam<Team>) {
        for (uint32_t i = r; i < n; i += T) {
            uint32_t g = W.boff + i;
            uint32_t cp = 0, cs = 0, active0 = 0, active1 = 0;  // which of the first 64 candidates are active
            if (!removed(S, g)) {
                uint2 cc = S.candCount[g];
                const uint32_t* crow = S.candRow + W.rowOff + (uint64_t)i * W.k;
                DContact tmp;
                for (uint32_t e = 0; e < cc.x + cc.y; ++e) {
                    const uint32_t kind = e < cc.x ? 0u : 1u;
                    if (!contact_record<false>(S, W, i, kind, crow[e] & kIndexMask, tmp)) continue;
                    if (kind == 0u) ++cp; else ++cs;
                    if (e < 32u) active0 |= 1u << e;
                    else if (e < 64u) active1 |= 1u << (e - 32u);
                }
            }
            S.scanA[g] = cp;
            S.scanB[g] = cs;
            // the non-contact accelerations are not needed again this step: their slot keeps the activity bits for
            // the writing pass (stored as raw bits)
            S.a0[g] = f2(__uint_as_float(active0), __uint_as_float(active1));
            pairsLocal += cp;
            segsLocal += cs;
        }
    } else {
        // The whole-GPU team spreads the candidate rows of a warp's bubbles over its lanes (warp_rows); each owner counts
        // its own entries in row order. (The block and group teams measured faster with the plain loop above.)
        for (uint32_t i0 = r - lane; i0 < n; i0 += T) {  // the whole warp iterates together
            const uint32_t i = i0 + lane, g = W.boff + i;
            const bool has = i < n && !removed(S, g);
            const uint2 cc = has ? S.candCount[g] : make_uint2(0u, 0u);
            uint32_t cp = 0, cs = 0, active0 = 0, active1 = 0, e = 0;  // which of the first 64 candidates are active
            warp_rows(cc.x + cc.y, records + (r - lane),
                      [&](uint32_t o, uint32_t eo) {
                          const uint32_t io = i0 + o, go = W.boff + io;
                          const uint32_t kind = eo < S.candCount[go].x ? 0u : 1u;
                          const uint32_t* crow = S.candRow + W.rowOff + (uint64_t)io * W.k;
                          DContact tmp;
                          const bool on = contact_record<false>(S, W, io, kind, crow[eo] & kIndexMask, tmp);
                          return make_float4(on ? 1.0f : 0.0f, 0.0f, 0.0f, 0.0f);
                      },
                      [&](float4 v) {
                          if (v.x != 0.0f) {
                              if (e < cc.x) ++cp; else ++cs;
                              if (e < 32u) active0 |= 1u << e;
                              else if (e < 64u) active1 |= 1u << (e - 32u);
                          }
                          ++e;
                      });
            if (i >= n) continue;
            S.scanA[g] = cp;
            S.scanB[g] = cs;
            // the non-contact accelerations are not needed again this step: their slot keeps the activity bits for the
            // writing pass (stored as raw bits)
            S.a0[g] = f2(__uint_as_float(active0), __uint_as_float(active1));
            pairsLocal += cp;
            segsLocal += cs;
        }
    }
    BP_PHASE(6);
    uint32_t pc[4] = {pairsLocal, segsLocal, 0u, 0u};
    team.template reduce4<0u>(pc);
    const uint32_t pairsAll = pc[0];
    const uint32_t segsAll = pc[1];
    team.scan_inplace(S.scanA + W.boff, n);
    team.scan_inplace(S.scanB + W.boff, n);
    // Records in row order per bubble (pairs at scanA, segments after all pairs at scanB).
    uint32_t droppedLocal = 0;
    auto emit = [&](const DContact& rec, uint32_t slot) {
        if (!finite2(rec.normal) || !finite2(rec.point) || !isfinite(rec.impulse) || !isfinite(rec.penetration)) nonfinite = 1u;
        if (slot < W.contactCap) S.contacts[W.contactOff + slot] = rec;
        else ++droppedLocal;
    };
    if (!kGridTeam<Team>) {
        for (uint32_t i = r; i < n; i += T) {
            uint32_t g = W.boff + i;
            if (removed(S, g)) continue;
            uint2 cc = S.candCount[g];
            const uint32_t* crow = S.candRow + W.rowOff + (uint64_t)i * W.k;
            uint32_t op = S.scanA[g], os = pairsAll + S.scanB[g];
            const float2 bits = S.a0[g];
            const uint32_t active0 = __float_as_uint(bits.x), active1 = __float_as_uint(bits.y);
            DContact rec;
            for (uint32_t e = 0; e < cc.x + cc.y; ++e) {
                uint32_t kind = e < cc.x ? 0u : 1u;
                if (e < 32u ? !((active0 >> e) & 1u) : (e < 64u && !((active1 >> (e - 32u)) & 1u))) continue;
                if (!contact_record<true>(S, W, i, kind, crow[e] & kIndexMask, rec)) continue;
                emit(rec, kind == 0u ? op++ : os++);
            }
        }
    } else {
        // The whole-GPU team spreads the first 64 entries of the warp's rows over its lanes: an active entry's slot is
        // its owner's offset plus the active entries of its kind before it (the activity bits). Entries from 64 on
        // follow in order on the owner's lane.
        for (uint32_t i0 = r - lane; i0 < n; i0 += T) {  // the whole warp iterates together
            const uint32_t i = i0 + lane, g = W.boff + i;
            const bool has = i < n && !removed(S, g);
            const uint2 cc = has ? S.candCount[g] : make_uint2(0u, 0u);
            warp_entries(min(cc.x + cc.y, 64u), [&](uint32_t o, uint32_t e) {
                const uint32_t io = i0 + o, go = W.boff + io;
                const float2 bits = S.a0[go];
                const unsigned long long active =
                    (unsigned long long)__float_as_uint(bits.x) | ((unsigned long long)__float_as_uint(bits.y) << 32);
                if (!((active >> e) & 1ull)) return;
                const uint32_t pairs = S.candCount[go].x, kind = e < pairs ? 0u : 1u;
                const uint32_t* crow = S.candRow + W.rowOff + (uint64_t)io * W.k;
                DContact rec;
                if (!contact_record<true>(S, W, io, kind, crow[e] & kIndexMask, rec)) return;
                const unsigned long long below = active & ((1ull << e) - 1ull);
                const unsigned long long pairMask = pairs >= 64u ? ~0ull : ((1ull << pairs) - 1ull);
                const uint32_t slot = kind == 0u ? S.scanA[go] + (uint32_t)__popcll(below)
                                                 : pairsAll + S.scanB[go] + (uint32_t)__popcll(below & ~pairMask);
                emit(rec, slot);
            });
            if (!has || cc.x + cc.y <= 64u) continue;
            const float2 bits = S.a0[g];
            const unsigned long long active =
                (unsigned long long)__float_as_uint(bits.x) | ((unsigned long long)__float_as_uint(bits.y) << 32);
            const unsigned long long pairMask = cc.x >= 64u ? ~0ull : ((1ull << cc.x) - 1ull);
            uint32_t op = S.scanA[g] + (uint32_t)__popcll(active & pairMask);
            uint32_t os = pairsAll + S.scanB[g] + (uint32_t)__popcll(active & ~pairMask);
            const uint32_t* crow = S.candRow + W.rowOff + (uint64_t)i * W.k;
            DContact rec;
            for (uint32_t e = 64u; e < cc.x + cc.y; ++e) {
                const uint32_t kind = e < cc.x ? 0u : 1u;
                if (!contact_record<true>(S, W, i, kind, crow[e] & kIndexMask, rec)) continue;
                emit(rec, kind == 0u ? op++ : os++);
            }
        }
    }
    BP_PHASE(7);
    // non-finite state (nativeCheckFinite, NPK:5-27)
    for (uint32_t i = r; i < n; i += T) {
        uint32_t g = W.boff + i;
        if (removed(S, g)) continue;
        if (!finite2(S.pos[g]) || !finite2(S.start[g]) || !finite2(S.vel[g]) || !finite2(S.rotw[g])) nonfinite = 1u;
    }
    uint32_t nf[4] = {nonfinite, droppedLocal, 0u, 0u};
    team.template reduce4<1u>(nf);
    const uint32_t anyNonfinite = nf[0];
    const uint32_t contactDropped = nf[1];
    BP_PHASE(8);
    if (!violated && stepDone && !(W.flags & BP_WORLD_NO_END_ASSERTION))
        violated = useTree ? assert_contacts<Team, true>(S, W, team, buckets, entries, B, cw, 1.0f, rep, buildOverflow == 0u)
                           : assert_contacts<Team, false>(S, W, team, buckets, entries, B, cw, 1.0f, rep, buildOverflow == 0u);
    BP_PHASE(9);
    int status = BP_OK;
    if (c.cW != 0u) status = BP_E_SUBSTEP_LIMIT;
    else if (anyNonfinite) status = BP_E_NONFINITE;
    else if (violated) status = BP_E_CONTACT_VIOLATION;
    uint32_t candLocal = 0, bodyCandLocal = 0;
    for (uint32_t i = r; i < n; i += T) {
        uint2 cc = S.candCount[W.boff + i];
        if (!removed(S, W.boff + i)) candLocal += cc.x + cc.y;
    }
    for (uint32_t bi = r; bi < W.nb; bi += T) bodyCandLocal += min(S.bodyTotal[W.bodyOff + bi], W.k);
    uint32_t counts4[4] = {removedCount, wrapped, candLocal, bodyCandLocal};
    team.template reduce4<0u>(counts4);
    const uint32_t removedAll = counts4[0];
    const uint32_t wrappedAll = counts4[1];
    const uint32_t candAll = counts4[2];
    const uint32_t bodyCandAll = counts4[3];
    if (team.leader()) {
        rep->status = status;
        rep->substep_count = c.cY;
        rep->rebuild_count = rebuilds;
        rep->candidate_count = candAll;
        rep->body_candidate_count = bodyCandAll;
        rep->candidate_overflow = overflowMax;
        rep->max_candidates_per_object = maxPer;
        rep->contact_count = min(pairsAll + segsAll, W.contactCap);
        rep->limiter_term = c.limTerm;
        rep->limiter_object = c.limObj;
        rep->cell_width = cw;
        rep->removed_count = removedAll;
        rep->wrapped_count = wrappedAll;
        rep->contact_overflow = contactDropped;
        if (!violated) {
            rep->violation_kind = 0u;
            rep->violation_objects[0] = 0;
            rep->violation_objects[1] = 0;
            rep->violation_edge = 0;
            rep->violation_distance = 0.0f;
        }
        S.contactCount[wi] = min(pairsAll + segsAll, W.contactCap);
    }
    // publish on success, restore the published state on failure (CompleteStep.swift:5-7); staged state goes back
    // to global memory here
    if (status == BP_OK) {
        for (uint32_t i = r; i < n; i += T) {
            uint32_t g = W.boff + i;
            uint32_t f = S.flags[g] & ~(kValid | kStartFinite);
            if (G.result[g] == 1u) f |= kRemoved;
            float2 p = S.pos[g], v = S.vel[g];
            G.flags[g] = f;
            G.pFlags[g] = f;
            G.pos[g] = p;
            G.pPos[g] = p;
            G.vel[g] = v;
            G.pVel[g] = v;
            G.acc[g] = S.acc[g];
            G.pStart[g] = G.start[g];
            G.pRotw[g] = G.rotw[g];
            G.pResult[g] = G.result[g];
            G.candCount[g] = S.candCount[g];
            G.pairTotal[g] = S.pairTotal[g];
            G.deg[g] = S.deg[g];
            G.cell[g] = S.cell[g];
        }
        for (uint32_t bi = r; bi < W.nb; bi += T) G.pBody[W.bodyOff + bi] = G.body[W.bodyOff + bi];
    } else {
        for (uint32_t i = r; i < n; i += T) {
            uint32_t g = W.boff + i;
            G.flags[g] = G.pFlags[g];
            G.pos[g] = G.pPos[g];
            G.start[g] = G.pStart[g];
            G.vel[g] = G.pVel[g];
            G.rotw[g] = G.pRotw[g];
            G.result[g] = G.pResult[g];
            G.candCount[g] = S.candCount[g];
            G.pairTotal[g] = S.pairTotal[g];
            G.deg[g] = S.deg[g];
            G.cell[g] = S.cell[g];
        }
        for (uint32_t bi = r; bi < W.nb; bi += T) G.body[W.bodyOff + bi] = G.pBody[W.bodyOff + bi];
        if (team.leader()) G.failed[wi] = 1u;
    }
    BP_PHASE(10);
    BP_STAMP(G, 25);
}

// ------------------------------------------------------------------------------------------------------------------
// Kernels
// ------------------------------------------------------------------------------------------------------------------
extern __shared__ __align__(16) uint32_t g_dynamic_smem[];

static_assert(sizeof(BlockScratch) <= 4u * kGroupScratchWords, "a group's reduction scratch fits its slice");

// Entry records of a CTA world's grid: after its bucket ends and entries (grid_words).
__device__ __forceinline__ float4* cta_records(const QueueArgs& q) {
    return (float4*)(g_dynamic_smem + round4_words(q.ctaB + q.ctaMaxN));
}

// Persistent step kernel: blocks pull worlds from two queues. First the block splits into groups of q.groupWidth
// threads (one warp or more), and every group pulls worlds of the group queue on its own, so a block keeps
// blockDim / groupWidth worlds in flight; then CTA-team worlds (largest first) are stepped by the whole block. Dynamic
// shared memory holds the hash grid: for a CTA world B bucket ends then its entries (then its workspace); for the group
// queue one slice per group (group_slice_words).
template <class Next>
__device__ __forceinline__ void group_queue(const QueueArgs& q, uint32_t nGroup, BlockScratch& blockSh, uint32_t* next,
                                            Next&& step) {
    if (nGroup == 0u) return;
    const uint32_t width = q.groupWidth > 32u ? q.groupWidth : 32u, group = threadIdx.x / width;
    uint32_t* mine = g_dynamic_smem + group * group_slice_words(q);
    const uint32_t scratch = group_scratch_words(width);
    TeamState& ts = *(TeamState*)mine;
    GroupTeam team{scratch > kTeamStateWords ? (BlockScratch*)(mine + kTeamStateWords) : &blockSh,
                   GroupShape{group * width, width, 1u + group}};
    uint32_t* grid = mine + scratch;
    float4* records = (float4*)(grid + round4_words(q.warpB + q.warpMaxN));
    uint32_t* ws = q.warpWsWords ? grid + grid_words(q.warpB, q.warpMaxN, width) : nullptr;
    for (;;) {
        if (team.leader()) next[group] = atomicAdd(q.queue + 1, 1u);
        team.sync();
        const uint32_t slot = next[group];
        team.sync();
        if (slot >= nGroup) break;
        step(q.warpList[slot], team, grid, grid + q.warpB, records, ws, ts);
        team.sync();
    }
}

template <int kThreads, bool kTree>
__global__ void __launch_bounds__(kThreads, 2) persistent_step_kernel(DState S, QueueArgs q) {
    __shared__ BlockScratch sh;
    __shared__ uint32_t next[kThreads / 32];
    __shared__ TeamState ctaState;
    CtaTeam cta{&sh};
    const uint32_t nCta = q.countsOnDevice ? *(volatile uint32_t*)(q.queue + 2) : q.nCta;
    const uint32_t nGroup = q.countsOnDevice ? *(volatile uint32_t*)(q.queue + 3) : q.nWarp;
    // The group queue goes first: its worlds are cheap but slow to finish (many in flight per SM), and taken last they
    // left a long drain at the end of the launch; the block-team queue ends with its cheapest worlds instead. The first
    // block barrier of the block-team loop waits for every group of the block.
    group_queue(q, nGroup, sh, next, [&](uint32_t wi, const GroupTeam& team, uint32_t* buckets, uint32_t* entries,
                                         float4* records, uint32_t* ws, TeamState& ts) {
        world_step<GroupTeam, kTree>(S, wi, team, buckets, entries, records, q.warpB, ws, q.warpWsWords, ts);
    });
    for (;;) {
        if (threadIdx.x == 0) next[0] = atomicAdd(q.queue, 1u);
        __syncthreads();
        const uint32_t slot = next[0];
        __syncthreads();
        if (slot >= nCta) break;
        world_step<CtaTeam, kTree>(S, q.ctaList[slot], cta, g_dynamic_smem, g_dynamic_smem + q.ctaB, cta_records(q), q.ctaB,
                                   q.ctaWsWords ? g_dynamic_smem + grid_words(q.ctaB, q.ctaMaxN, blockDim.x) : nullptr, q.ctaWsWords,
                                   ctaState);
        __syncthreads();
    }
}

// Served step kernel: the same two queues over a batch of resident worlds that each keep their own device arrays.
// Entry e of the batch is world 0 of the state `sets[entrySlot[e]]`; its report goes to reports[e].
template <int kThreads, bool kTree>
__global__ void __launch_bounds__(kThreads, 2) served_step_kernel(const DState* sets, const uint32_t* entrySlot,
                                                                   bp_step_report* reports, QueueArgs q) {
    __shared__ BlockScratch sh;
    __shared__ uint32_t next[kThreads / 32];
    __shared__ TeamState ctaState;
    CtaTeam cta{&sh};
    // Block-team worlds first: a serving batch is a few worlds, and its latency is that of its largest world, which
    // must start at once (the batched kernel, which steps thousands of worlds for throughput, takes the groups first).
    for (;;) {
        if (threadIdx.x == 0) next[0] = atomicAdd(q.queue, 1u);
        __syncthreads();
        const uint32_t slot = next[0];
        __syncthreads();
        if (slot >= q.nCta) break;
        const uint32_t e = q.ctaList[slot];
        if (threadIdx.x == 0) {
            ctaState.G = sets[entrySlot[e]];
            ctaState.G.reports = reports + e;
        }
        __syncthreads();
        world_step<CtaTeam, kTree>(ctaState.G, 0u, cta, g_dynamic_smem, g_dynamic_smem + q.ctaB, cta_records(q), q.ctaB,
                                   q.ctaWsWords ? g_dynamic_smem + grid_words(q.ctaB, q.ctaMaxN, blockDim.x) : nullptr, q.ctaWsWords,
                                   ctaState);
        __syncthreads();
    }
    group_queue(q, q.nWarp, sh, next, [&](uint32_t e, const GroupTeam& team, uint32_t* buckets, uint32_t* entries,
                                          float4* records, uint32_t* ws, TeamState& ts) {
        if (team.leader()) {
            ts.G = sets[entrySlot[e]];
            ts.G.reports = reports + e;
        }
        team.sync();
        world_step<GroupTeam, kTree>(ts.G, 0u, team, buckets, entries, records, q.warpB, ws, q.warpWsWords, ts);
    });
}

}  // namespace

// Launchers of one kernel variant (defined in bp_step_variant.cu, once per variant): a launch with `threads` threads
// per block (at most the variant's width), the persistent kernel's blocks per SM at a dynamic shared-memory size, and
// `prepare`, which raises the kernel's dynamic shared-memory limit.
#define BP_STEP_VARIANTS(X) X(128, 0) X(256, 0) X(512, 0) X(128, 1) X(256, 1) X(512, 1)
#define BP_DECLARE_VARIANT(T, R)                                                                                     \
    cudaError_t persistent_launch_##T##_##R(const DState& S, const QueueArgs& q, uint32_t threads, uint32_t blocks,  \
                                            size_t smem, cudaStream_t stream);                                      \
    int persistent_blocks_per_sm_##T##_##R(uint32_t threads, size_t smem);                                           \
    cudaError_t persistent_prepare_##T##_##R(int maxSmem);                                                           \
    cudaError_t served_launch_##T##_##R(const DState* sets, const uint32_t* entrySlot, bp_step_report* reports,      \
                                        const QueueArgs& q, uint32_t threads, uint32_t blocks, size_t smem,         \
                                        cudaStream_t stream);                                                       \
    cudaError_t served_prepare_##T##_##R(int maxSmem);
BP_STEP_VARIANTS(BP_DECLARE_VARIANT)

}  // namespace bp
