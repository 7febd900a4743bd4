// bp_events.cu - contact began / ended events of a step on the device (the reference's contact transitions,
// NativePublicWorld.swift:340-391, which it runs on its CPU after reading the contact cache back; here one block
// compacts them from the step's contact records in device memory).
//
// A record (the step's bubble-bubble and bubble-segment records, then the caller's extra records) counts when its
// penetration or impulse is positive and either object has contact interest. Its pair key orders the two object ids
// as unsigned 64-bit values; records of one key are summed in record order (penetration-weighted point, weight,
// normal from the key's first object, impulse / step), which is what the reference's dictionary of sums does. Keys
// are sorted with (key, record index) as the sort key, so the sum of each key visits its records in record order and
// the event list is deterministic. Events: began for the keys not in the history (ascending), then ended for the
// history keys (ascending) that are gone or lost an object (a pair whose objects were both removed reports nothing).
// The new history is the current keys without removed objects.
#include "bp_host.h"

namespace bp {

struct EventEntry {
    unsigned long long k0, k1;  // pair key, k0 <= k1 as unsigned
    float px, py, w, nx, ny, imp;
    uint32_t record, pad;
};

__device__ __forceinline__ bool key_less(unsigned long long a0, unsigned long long a1, unsigned long long b0,
                                         unsigned long long b1) {
    return a0 < b0 || (a0 == b0 && a1 < b1);
}

__device__ __forceinline__ bool sorted_contains(const long long* ids, uint32_t count, long long id) {
    uint32_t lo = 0, hi = count;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (ids[mid] < id) lo = mid + 1; else hi = mid;
    }
    return lo < count && ids[lo] == id;
}

// Position of key (k0, k1) in a sorted list of key pairs (2 words per key), or `count` when absent.
__device__ __forceinline__ uint32_t key_find(const unsigned long long* keys, uint32_t count, unsigned long long k0,
                                             unsigned long long k1) {
    uint32_t lo = 0, hi = count;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (key_less(keys[2 * mid], keys[2 * mid + 1], k0, k1)) lo = mid + 1; else hi = mid;
    }
    return (lo < count && keys[2 * lo] == k0 && keys[2 * lo + 1] == k1) ? lo : count;
}

// Block-wide exclusive scan of one value per thread (blockDim.x <= 1024, a multiple of 32).
__device__ uint32_t event_block_scan(uint32_t x, uint32_t* total, uint32_t* sh) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t incl = x;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= (uint32_t)off) incl += y;
    }
    __syncthreads();
    if (lane == 31u) sh[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const uint32_t y = lane < nw ? sh[lane] : 0u;
        uint32_t s = y;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t z = __shfl_up_sync(0xffffffffu, s, off);
            if (lane >= (uint32_t)off) s += z;
        }
        if (lane < nw) sh[lane] = s - y;
        if (lane == nw - 1) sh[32] = s;
    }
    __syncthreads();
    *total = sh[32];
    return sh[warp] + incl - x;
}

struct EventArgs {
    const DContact* records;      // the step's records (index form), `deviceCount` of them
    uint32_t deviceCount;
    const bp_contact* extra;      // caller's records (ids form, kind 2), `extraCount` of them
    uint32_t extraCount;
    const int64_t* ids;           // bubble ids of the world (by bubble index)
    const DSegment* segments;     // the world's segments (by segment index)
    const long long* interested;  // sorted ids with contact interest
    uint32_t interestedCount;
    const long long* removed;     // sorted ids removed in this step
    uint32_t removedCount;
    const unsigned long long* history;  // sorted keys of the previous step
    uint32_t historyCount;
    unsigned long long* nextHistory;    // out: sorted keys of this step
    uint32_t* nextHistoryCount;
    float step;
    EventEntry* entries;          // scratch: one per record
    uint32_t* order;              // scratch: pow2 >= records
    uint32_t* heads;              // scratch: compacted current keys (entry index of each key's first record)
    bp_contact_event* out;
    uint32_t capacity;
    uint32_t* count;
};

__global__ void __launch_bounds__(1024) contact_events_kernel(EventArgs a) {
    __shared__ uint32_t sh[33];
    const uint32_t R = a.deviceCount + a.extraCount, T = blockDim.x, t = threadIdx.x;
    // 1. one entry per counting record
    for (uint32_t r = t; r < R; r += T) {
        long long first, second;
        float2 nff, point;
        float pen, impulse;
        bool ok = true;
        if (r < a.deviceCount) {
            const DContact c = a.records[r];
            first = a.ids[c.a];
            if (c.kind == 0u) {
                second = a.ids[c.other];
                nff = c.normal;  // from bubble a to bubble b
            } else {
                const DSegment& sg = a.segments[c.other];
                ok = (sg.flags & BP_SEGMENT_HAS_OWNER) != 0u;
                second = sg.owner;
                nff = make_float2(-c.normal.x, -c.normal.y);  // the record's normal points from the segment to the bubble
            }
            point = c.point;
            pen = c.penetration;
            impulse = c.impulse;
        } else {
            const bp_contact& c = a.extra[r - a.deviceCount];
            first = c.participants[0];
            second = c.participants[1];
            nff = make_float2(c.normal[0], c.normal[1]);
            point = make_float2(c.point[0], c.point[1]);
            pen = c.penetration;
            impulse = c.impulse;
        }
        ok = ok && (pen > 0.0f || impulse > 0.0f);
        ok = ok && (sorted_contains(a.interested, a.interestedCount, first) ||
                    sorted_contains(a.interested, a.interestedCount, second));
        EventEntry e;
        const unsigned long long uf = (unsigned long long)first, us = (unsigned long long)second;
        const bool firstLow = uf <= us;
        e.k0 = ok ? (firstLow ? uf : us) : ~0ull;
        e.k1 = ok ? (firstLow ? us : uf) : ~0ull;
        const float w = fmaxf(pen, 0.0f) + 1e-4f;
        e.w = w;
        e.px = point.x * w;
        e.py = point.y * w;
        e.nx = firstLow ? nff.x : -nff.x;
        e.ny = firstLow ? nff.y : -nff.y;
        e.imp = impulse / a.step;
        e.record = ok ? r : 0xffffffffu;
        e.pad = 0u;
        a.entries[r] = e;
    }
    uint32_t P = 1;
    while (P < R) P <<= 1;
    for (uint32_t i = t; i < P; i += T) a.order[i] = i < R ? i : 0xffffffffu;
    __syncthreads();
    // 2. bitonic sort of entry indices by (key, record); dropped records and padding go last
    auto before = [&](uint32_t x, uint32_t y) {  // x strictly before y
        if (y == 0xffffffffu) return x != 0xffffffffu;
        if (x == 0xffffffffu) return false;
        const EventEntry& ex = a.entries[x];
        const EventEntry& ey = a.entries[y];
        if (ex.k0 != ey.k0) return ex.k0 < ey.k0;
        if (ex.k1 != ey.k1) return ex.k1 < ey.k1;
        return ex.record < ey.record;
    };
    for (uint32_t size = 2; size <= P; size <<= 1) {
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
            for (uint32_t i = t; i < P; i += T) {
                const uint32_t j = i ^ stride;
                if (j > i) {
                    const bool up = (i & size) == 0;
                    const uint32_t x = a.order[i], y = a.order[j];
                    if (before(y, x) == up) { a.order[i] = y; a.order[j] = x; }
                }
            }
            __syncthreads();
        }
    }
    // 3. the first record of each key sums its key's records in record order; heads are compacted in key order
    uint32_t running = 0;
    const uint32_t per = (R + T - 1) / T;
    const uint32_t lo = min(t * per, R), hi = min(lo + per, R);
    for (uint32_t i = lo; i < hi; ++i) {
        const uint32_t x = a.order[i];
        if (x == 0xffffffffu || a.entries[x].record == 0xffffffffu) continue;
        const bool head = i == 0 || a.entries[a.order[i - 1]].k0 != a.entries[x].k0 ||
                          a.entries[a.order[i - 1]].k1 != a.entries[x].k1;
        running += head ? 1u : 0u;
    }
    uint32_t heads;
    uint32_t slot = event_block_scan(running, &heads, sh);
    for (uint32_t i = lo; i < hi; ++i) {
        const uint32_t x = a.order[i];
        if (x == 0xffffffffu || a.entries[x].record == 0xffffffffu) continue;
        const bool head = i == 0 || a.entries[a.order[i - 1]].k0 != a.entries[x].k0 ||
                          a.entries[a.order[i - 1]].k1 != a.entries[x].k1;
        if (!head) continue;
        float px = 0.0f, py = 0.0f, w = 0.0f, nx = 0.0f, ny = 0.0f, imp = 0.0f;
        for (uint32_t m = i; m < R; ++m) {
            const uint32_t y = a.order[m];
            if (y == 0xffffffffu) break;
            const EventEntry& e = a.entries[y];
            if (e.record == 0xffffffffu || e.k0 != a.entries[x].k0 || e.k1 != a.entries[x].k1) break;
            px = px + e.px;
            py = py + e.py;
            w = w + e.w;
            nx = nx + e.nx;
            ny = ny + e.ny;
            imp = imp + e.imp;
        }
        EventEntry& h = a.entries[x];  // the head keeps its key's sums (its own contribution was read above)
        h.px = px; h.py = py; h.w = w; h.nx = nx; h.ny = ny; h.imp = imp;
        a.heads[slot++] = x;
    }
    __syncthreads();
    // 4. began: current keys not in the history; ended: history keys gone or with a removed object. Each thread
    // takes a contiguous chunk of both lists, so scans of its counts place the events in key order.
    const uint32_t C = heads, H = a.historyCount;
    auto gone = [&](uint32_t q) {
        const unsigned long long k0 = a.history[2 * q], k1 = a.history[2 * q + 1];
        const bool r0 = sorted_contains(a.removed, a.removedCount, (long long)k0);
        const bool r1 = sorted_contains(a.removed, a.removedCount, (long long)k1);
        if (r0 && r1) return false;  // nobody is left to tell
        if (r0 || r1) return true;
        for (uint32_t lo2 = 0, hi2 = C;;) {  // binary search over the compacted current keys
            if (lo2 >= hi2) return true;
            const uint32_t mid = (lo2 + hi2) >> 1;
            const EventEntry& e = a.entries[a.heads[mid]];
            if (key_less(e.k0, e.k1, k0, k1)) lo2 = mid + 1;
            else if (e.k0 == k0 && e.k1 == k1) return false;
            else hi2 = mid;
        }
    };
    const uint32_t perC = (C + T - 1) / T, cLo = min(t * perC, C), cHi = min(cLo + perC, C);
    const uint32_t perH = (H + T - 1) / T, hLo = min(t * perH, H), hHi = min(hLo + perH, H);
    uint32_t myBegan = 0, myEnded = 0, myKeep = 0;
    for (uint32_t c = cLo; c < cHi; ++c) {
        const EventEntry& e = a.entries[a.heads[c]];
        myBegan += key_find(a.history, H, e.k0, e.k1) == H ? 1u : 0u;
        const bool removedObject = sorted_contains(a.removed, a.removedCount, (long long)e.k0) ||
                                   sorted_contains(a.removed, a.removedCount, (long long)e.k1);
        myKeep += removedObject ? 0u : 1u;
    }
    for (uint32_t q = hLo; q < hHi; ++q) myEnded += gone(q) ? 1u : 0u;
    uint32_t totalBegan, totalEnded, totalKeep;
    uint32_t beganAt = event_block_scan(myBegan, &totalBegan, sh);
    uint32_t endedAt = event_block_scan(myEnded, &totalEnded, sh) + totalBegan;
    uint32_t keepAt = event_block_scan(myKeep, &totalKeep, sh);
    for (uint32_t c = cLo; c < cHi; ++c) {
        const EventEntry& e = a.entries[a.heads[c]];
        if (key_find(a.history, H, e.k0, e.k1) == H) {
            if (beganAt < a.capacity) {
                bp_contact_event ev{};
                ev.kind = 0u;
                ev.objects[0] = (int64_t)e.k0;
                ev.objects[1] = (int64_t)e.k1;
                ev.point[0] = e.px / e.w;
                ev.point[1] = e.py / e.w;
                const float length = sqrtf(e.nx * e.nx + e.ny * e.ny);
                ev.normal[0] = length > 0.0f ? e.nx / length : 0.0f;
                ev.normal[1] = length > 0.0f ? e.ny / length : 0.0f;
                ev.impulse = e.imp;
                a.out[beganAt] = ev;
            }
            ++beganAt;
        }
        const bool removedObject = sorted_contains(a.removed, a.removedCount, (long long)e.k0) ||
                                   sorted_contains(a.removed, a.removedCount, (long long)e.k1);
        if (!removedObject) {
            a.nextHistory[2 * keepAt] = e.k0;
            a.nextHistory[2 * keepAt + 1] = e.k1;
            ++keepAt;
        }
    }
    for (uint32_t q = hLo; q < hHi; ++q) {
        if (!gone(q)) continue;
        if (endedAt < a.capacity) {
            bp_contact_event ev{};
            ev.kind = 1u;
            ev.objects[0] = (int64_t)a.history[2 * q];
            ev.objects[1] = (int64_t)a.history[2 * q + 1];
            a.out[endedAt] = ev;
        }
        ++endedAt;
    }
    if (t == 0) {
        *a.count = totalBegan + totalEnded;
        *a.nextHistoryCount = totalKeep;
    }
}

cudaError_t launch_contact_events(const EventArgsHost& h, cudaStream_t stream) {
    EventArgs a;
    a.records = h.records;
    a.deviceCount = h.deviceCount;
    a.extra = h.extra;
    a.extraCount = h.extraCount;
    a.ids = h.ids;
    a.segments = h.segments;
    a.interested = (const long long*)h.interested;
    a.interestedCount = h.interestedCount;
    a.removed = (const long long*)h.removed;
    a.removedCount = h.removedCount;
    a.history = h.history;
    a.historyCount = h.historyCount;
    a.nextHistory = h.nextHistory;
    a.nextHistoryCount = h.nextHistoryCount;
    a.step = h.step;
    a.entries = (EventEntry*)h.entries;
    a.order = h.order;
    a.heads = h.heads;
    a.out = h.out;
    a.capacity = h.capacity;
    a.count = h.count;
    contact_events_kernel<<<1, 1024, 0, stream>>>(a);
    return cudaGetLastError();
}

size_t event_entry_bytes() { return sizeof(EventEntry); }

}  // namespace bp
