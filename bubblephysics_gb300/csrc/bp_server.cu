// bp_server.cu - serving loop over resident worlds (bp_server_* in include/bubblephysics.h).
//
// Every registered world keeps a deep copy of its input on the host. A world that a request needs becomes resident:
// its device arrays come from the server's stream-ordered memory pool (cheap to take and give back), and its state
// descriptor (DState) goes to a slot of a device table. A batch is a list of slots: one launch of the served step
// kernel steps them all, each world by a block or a warp like the persistent batched kernel, with reports written per
// batch entry and copied back on the batch's stream. Several batches can be in flight on different streams; a world
// is never in two at once. When the device budget is full, idle worlds leave in least-recently-used order: their
// step-to-step state (PersistentPart) is copied byte for byte into pinned host memory and copied back on return, so
// eviction never changes a result.
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <new>
#include <thread>
#include <vector>

#include "bp_host.h"

using namespace bp;
using namespace bp_host;

static_assert(sizeof(bp_server_config) == 40, "bp_server_config layout");
static_assert(sizeof(bp_server_completion) == 136, "bp_server_completion layout");
static_assert(sizeof(bp_server_stats) == 80, "bp_server_stats layout");

namespace {

constexpr uint64_t kDefaultBudget = 120ull << 30;
constexpr uint32_t kDefaultStreams = 8;          // batches in flight: a new arrival rarely waits for a free stream
constexpr uint32_t kDefaultServeThreads = 512;    // the widest block: the largest worlds bound a batch's latency

double host_clock() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Request {
    uint64_t id;
    uint32_t steps, done, substeps;
    double submitted;
    bp_step_report last;
};

struct ServedWorld {
    bp_world_desc desc{};
    std::vector<bp_bubble> bubbles;
    std::vector<bp_segment> segments;
    std::vector<bp_body> bodies;
    std::vector<float> bodyVertices, fieldVertices;
    std::vector<uint32_t> bodyTriangles, jointRanges;
    std::vector<bp_force_field> fields;
    std::vector<int64_t> fieldIds, jointPartners;
    std::vector<bp_band> bands;
    std::vector<bp_motor> motors;
    uint32_t jointEntities = 0;
    bool hasJoints = false;

    std::unique_ptr<WorldSet> set;  // resident when set
    int slot = -1;
    uint64_t bytes = 0;             // device bytes when resident
    void* saved = nullptr;          // pinned copy of the persistent parts after an eviction
    size_t savedBytes = 0;
    bool hasSaved = false;
    std::deque<Request> pending;
    bool inflight = false;
    uint64_t lastUse = 0;

    bp_world_input input() const {
        bp_world_input in{};
        in.bubbles = bubbles.data(); in.bubble_count = (uint32_t)bubbles.size();
        in.segments = segments.data(); in.segment_count = (uint32_t)segments.size();
        in.bodies = bodies.data(); in.body_count = (uint32_t)bodies.size();
        in.body_vertices = bodyVertices.data(); in.body_vertex_count = (uint32_t)(bodyVertices.size() / 2);
        in.body_triangles = bodyTriangles.data(); in.body_triangle_count = (uint32_t)(bodyTriangles.size() / 3);
        in.fields = fields.data(); in.field_count = (uint32_t)fields.size();
        in.field_vertices = fieldVertices.data(); in.field_vertex_count = (uint32_t)(fieldVertices.size() / 2);
        in.field_object_ids = fieldIds.data(); in.field_object_id_count = (uint32_t)fieldIds.size();
        in.bands = bands.data(); in.band_count = (uint32_t)bands.size();
        in.motors = motors.data(); in.motor_count = (uint32_t)motors.size();
        in.joint_ranges = hasJoints ? jointRanges.data() : nullptr; in.joint_entity_count = jointEntities;
        in.joint_partners = hasJoints ? jointPartners.data() : nullptr;
        in.joint_partner_count = (uint32_t)jointPartners.size();
        return in;
    }
};

template <class T> std::vector<T> copy_of(const T* p, uint64_t count) {
    return p && count ? std::vector<T>(p, p + count) : std::vector<T>();
}

// One batch in flight: its stream, events, the device lists of the launch and the host copy of its reports.
struct Flight {
    cudaStream_t stream = nullptr;
    cudaEvent_t start = nullptr, done = nullptr;
    uint32_t* dLists = nullptr;          // ctaList[cap] | warpList[cap] | entrySlot[cap] | queue[4]
    bp_step_report* dReports = nullptr;
    uint32_t* hLists = nullptr;          // pinned staging of the lists
    bp_step_report* hReports = nullptr;  // pinned
    std::vector<uint32_t> worlds;        // batch entry -> world
    bool busy = false;
};

}  // namespace

struct bp_server {
    bp_context* ctx = nullptr;
    bp_server_config cfg{};
    cudaMemPool_t pool = nullptr;
    std::vector<std::unique_ptr<ServedWorld>> worlds;
    DState* dSets = nullptr;             // one state descriptor per slot (slots = max_worlds)
    std::vector<int> freeSlots;
    std::vector<Flight> flights;
    uint32_t cap = 0;                    // entries of a batch
    uint64_t residentBytes = 0, clockTick = 0, nextRequest = 1;
    uint32_t resident = 0;
    std::deque<bp_server_completion> finished;
    uint64_t admissions = 0, evictions = 0, batches = 0, batchedWorlds = 0, requestsDone = 0, bubbleSubsteps = 0;
    double deviceMs = 0.0;
    std::map<uint64_t, uint32_t> blocksFor;  // full-GPU block count per (tree, threads, shared memory)
};

namespace {

void complete(bp_server* s, uint32_t w, Request& r, int status) {
    bp_server_completion c{};
    c.request_id = r.id;
    c.world = w;
    c.status = status;
    c.steps = r.done;
    c.substeps = r.substeps;
    c.submitted_s = r.submitted;
    c.completed_s = host_clock();
    c.report = r.last;
    s->finished.push_back(c);
    s->requestsDone++;
}

cudaError_t evict(bp_server* s, uint32_t w) {
    ServedWorld& sw = *s->worlds[w];
    auto parts = persistent_parts(*sw.set);
    size_t total = 0;
    for (auto& p : parts) total += p.second;
    cudaError_t err = cudaSuccess;
    if (!sw.saved || sw.savedBytes < total) {
        if (sw.saved) cudaFreeHost(sw.saved);
        sw.saved = nullptr;
        err = cudaHostAlloc(&sw.saved, total, cudaHostAllocDefault);
        if (err) return err;
        sw.savedBytes = total;
    }
    size_t off = 0;
    for (auto& p : parts) {
        if (p.second) err = cudaMemcpyAsync((char*)sw.saved + off, p.first, p.second, cudaMemcpyDeviceToHost, s->ctx->stream);
        if (err) return err;
        off += p.second;
    }
    err = cudaStreamSynchronize(s->ctx->stream);
    if (err) return err;
    sw.hasSaved = true;
    sw.set.reset();  // device arrays go back to the pool on the context stream
    s->residentBytes -= sw.bytes;
    s->freeSlots.push_back(sw.slot);
    sw.slot = -1;
    s->resident--;
    s->evictions++;
    return cudaSuccess;
}

// Least recently used resident world with nothing to do, or -1.
int eviction_victim(bp_server* s) {
    int best = -1;
    for (uint32_t w = 0; w < s->worlds.size(); ++w) {
        const ServedWorld& sw = *s->worlds[w];
        if (!sw.set || sw.inflight || !sw.pending.empty()) continue;
        if (best < 0 || sw.lastUse < s->worlds[best]->lastUse) best = (int)w;
    }
    return best;
}

// Makes world w resident if the budget allows (evicting idle worlds as needed). 1 admitted, 0 no room, <0 error.
int admit(bp_server* s, uint32_t w) {
    ServedWorld& sw = *s->worlds[w];
    bp_world_input in = sw.input();
    if (!sw.bytes) {
        WorldSet probe;
        probe.ctx = s->ctx;
        probe.measureOnly = true;
        int st = build_set(probe, s->ctx, 1, &sw.desc, &in, false);
        if (st) return -st;
        sw.bytes = probe.deviceBytes;
    }
    while (s->residentBytes + sw.bytes > s->cfg.hbm_budget_bytes || s->freeSlots.empty()) {
        int victim = eviction_victim(s);
        if (victim < 0) return 0;
        cudaError_t err = evict(s, (uint32_t)victim);
        if (err) return -cuda_status(err);
    }
    std::unique_ptr<WorldSet> set(new (std::nothrow) WorldSet());
    if (!set) return -BP_E_ALLOC;
    set->pool = s->pool;
    set->planOnly = true;
    int st = build_set(*set, s->ctx, 1, &sw.desc, &in, false);
    if (st) return -st;
    cudaError_t err = cudaSuccess;
    if (sw.hasSaved) {
        auto parts = persistent_parts(*set);
        size_t off = 0;
        for (auto& p : parts) {
            if (p.second) err = cudaMemcpyAsync(p.first, (const char*)sw.saved + off, p.second, cudaMemcpyHostToDevice,
                                                s->ctx->stream);
            if (err) return -cuda_status(err);
            off += p.second;
        }
    }
    sw.slot = s->freeSlots.back();
    s->freeSlots.pop_back();
    err = cudaMemcpyAsync(s->dSets + sw.slot, &set->S, sizeof(DState), cudaMemcpyHostToDevice, s->ctx->stream);
    if (!err) err = cudaStreamSynchronize(s->ctx->stream);  // the batch streams see a complete world
    if (err) return -cuda_status(err);
    sw.bytes = set->deviceBytes;
    sw.set = std::move(set);
    s->residentBytes += sw.bytes;
    s->resident++;
    s->admissions++;
    return 1;
}

// Results of every batch whose device work has ended.
int collect(bp_server* s, bool wait, uint32_t& completed) {
    for (Flight& f : s->flights) {
        if (!f.busy) continue;
        cudaError_t q = wait ? cudaEventSynchronize(f.done) : cudaEventQuery(f.done);
        if (q == cudaErrorNotReady) continue;
        if (q != cudaSuccess) return cuda_status(q);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, f.start, f.done);
        s->deviceMs += ms;
        for (uint32_t e = 0; e < f.worlds.size(); ++e) {
            const uint32_t w = f.worlds[e];
            ServedWorld& sw = *s->worlds[w];
            const bp_step_report& rep = f.hReports[e];
            Request& r = sw.pending.front();
            r.done++;
            r.substeps += rep.substep_count;
            r.last = rep;
            s->bubbleSubsteps += (uint64_t)rep.substep_count * sw.bubbles.size();
            sw.inflight = false;
            sw.lastUse = ++s->clockTick;
            if (rep.status != BP_OK || r.done == r.steps) {
                complete(s, w, r, rep.status);
                sw.pending.pop_front();
                ++completed;
            }
        }
        f.worlds.clear();
        f.busy = false;
    }
    return BP_OK;
}

uint32_t ready_worlds(bp_server* s, std::vector<uint32_t>& out, uint32_t limit) {
    out.clear();
    for (uint32_t w = 0; w < s->worlds.size() && out.size() < limit; ++w) {
        const ServedWorld& sw = *s->worlds[w];
        if (sw.set && !sw.inflight && !sw.pending.empty()) out.push_back(w);
    }
    return (uint32_t)out.size();
}

// Launches one batch over `entries` on flight f: the host splits the worlds into the block and group queues (largest
// first) and sizes the shared memory as the batched schedule does.
int launch(bp_server* s, Flight& f, const std::vector<uint32_t>& entries) {
    const bool perWorld = (s->cfg.flags & BP_SERVER_PER_WORLD) != 0;
    const uint32_t warpMax = s->cfg.warp_world_max;
    const uint32_t n = (uint32_t)entries.size();
    uint32_t* cta = f.hLists;
    uint32_t* warp = f.hLists + s->cap;
    uint32_t* slot = f.hLists + 2 * s->cap;
    uint32_t nCta = 0, nWarp = 0, maxCta = 0, maxWarp = 0, ctaWs = 0, warpWs = 0, tree = 0;
    std::vector<uint32_t> order(entries.size());
    for (uint32_t e = 0; e < n; ++e) order[e] = e;
    auto sizeOf = [&](uint32_t e) { return s->worlds[entries[e]]->set->hWorlds[0].n; };
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return sizeOf(a) > sizeOf(b); });
    for (uint32_t e : order) {
        const DWorld& W = s->worlds[entries[e]]->set->hWorlds[0];
        slot[e] = (uint32_t)s->worlds[entries[e]]->slot;
        tree |= W.tree;
        if (W.n <= warpMax) { warp[nWarp++] = e; maxWarp = std::max(maxWarp, W.n); }
        else { cta[nCta++] = e; maxCta = std::max(maxCta, W.n); }
    }
    const uint32_t threads = perWorld && nCta == 0 ? 32u : s->cfg.threads_per_world;
    const uint32_t groupWidth = std::min(s->cfg.group_width, threads);
    const uint32_t ctaGridBytes = team_grid_bytes(maxCta, threads);
    const uint32_t ctaCap = std::min(kCtaWorkspaceCap, kMaxDynamicSmem - std::min(kMaxDynamicSmem, ctaGridBytes));
    uint32_t warpCap = 0;
    if (maxWarp && !group_layout(threads, groupWidth, maxWarp, &warpCap)) return BP_E_INVALID;
    for (uint32_t e = 0; e < n; ++e) {
        const DWorld& W = s->worlds[entries[e]]->set->hWorlds[0];
        const uint32_t bytes = workspace_bytes(W.n, W.s, W.nb);
        if (W.n <= warpMax) { if (bytes <= warpCap) warpWs = std::max(warpWs, bytes); }
        else if (bytes <= ctaCap) ctaWs = std::max(ctaWs, bytes);
    }
    QueueArgs q{};
    q.ctaList = f.dLists;
    q.warpList = f.dLists + s->cap;
    q.queue = f.dLists + 3 * s->cap;
    q.nCta = nCta;
    q.nWarp = nWarp;
    q.ctaMaxN = maxCta;
    q.ctaB = maxCta ? grid_buckets(maxCta) : 0u;
    q.warpMaxN = maxWarp;
    q.warpB = maxWarp ? grid_buckets(maxWarp) : 0u;
    q.countsOnDevice = 0u;
    q.tree = tree;
    q.ctaWsWords = ((ctaWs + 3u) / 4u + 3u) & ~3u;
    q.warpWsWords = ((warpWs + 3u) / 4u + 3u) & ~3u;
    q.groupWidth = groupWidth;
    const uint32_t groupsPerBlock = std::max(threads / groupWidth, 1u);
    const uint64_t key = ((uint64_t)q.tree << 63) | ((uint64_t)threads << 32) | persistent_smem(q, threads);
    auto known = s->blocksFor.find(key);
    const uint32_t full = known != s->blocksFor.end() ? known->second : (s->blocksFor[key] = persistent_blocks(q, threads));
    // a small batch takes only the blocks it can use, so batches on other streams keep the rest of the GPU
    uint32_t blocks = perWorld ? 1u : std::min(full, nCta + (nWarp + groupsPerBlock - 1u) / groupsPerBlock);
    blocks = std::max(blocks, 1u);
    cudaError_t err = cudaMemcpyAsync(f.dLists, f.hLists, 3ull * s->cap * sizeof(uint32_t), cudaMemcpyHostToDevice, f.stream);
    if (!err) err = cudaEventRecord(f.start, f.stream);
    if (!err) err = launch_served(s->dSets, f.dLists + 2 * s->cap, f.dReports, q, threads, blocks, f.stream);
    if (!err) err = cudaMemcpyAsync(f.hReports, f.dReports, n * sizeof(bp_step_report), cudaMemcpyDeviceToHost, f.stream);
    if (!err) err = cudaEventRecord(f.done, f.stream);
    if (err) return cuda_status(err);
    f.worlds = entries;
    f.busy = true;
    for (uint32_t w : entries) s->worlds[w]->inflight = true;
    s->batches++;
    s->batchedWorlds += n;
    return BP_OK;
}

int round_of(bp_server* s, uint32_t wait_us, uint32_t& completed) {
    DeviceGuard guard(s->ctx->device);
    int st = collect(s, false, completed);
    if (st) return st;
    // admission: worlds of waiting requests, oldest request first
    std::vector<std::pair<double, uint32_t>> want;
    for (uint32_t w = 0; w < s->worlds.size(); ++w) {
        const ServedWorld& sw = *s->worlds[w];
        if (!sw.set && !sw.pending.empty()) want.push_back({sw.pending.front().submitted, w});
    }
    std::sort(want.begin(), want.end());
    for (auto& p : want) {
        int a = admit(s, p.second);
        if (a < 0) return -a;
        if (a == 0) break;  // keep arrival order: later worlds wait too
    }
    // launches: every free stream takes the ready worlds (one world at a time on the plain path)
    const bool perWorld = (s->cfg.flags & BP_SERVER_PER_WORLD) != 0;
    std::vector<uint32_t> ready;
    for (Flight& f : s->flights) {
        if (f.busy) continue;
        if (!ready_worlds(s, ready, perWorld ? 1u : s->cap)) break;
        st = launch(s, f, ready);
        if (st) return st;
    }
    if (completed == 0 && wait_us > 0) {
        const double until = host_clock() + wait_us * 1e-6;
        bool any = false;
        for (Flight& f : s->flights) any |= f.busy;
        while (any && host_clock() < until) {
            for (Flight& f : s->flights)
                if (f.busy && cudaEventQuery(f.done) == cudaSuccess) { any = false; break; }
            if (any) std::this_thread::yield();
        }
        st = collect(s, false, completed);
    }
    return st;
}

void server_free(bp_server* s) {
    DeviceGuard guard(s->ctx->device);
    for (Flight& f : s->flights) {
        if (f.stream) cudaStreamSynchronize(f.stream);
        if (f.start) cudaEventDestroy(f.start);
        if (f.done) cudaEventDestroy(f.done);
        if (f.dLists) cudaFree(f.dLists);
        if (f.dReports) cudaFree(f.dReports);
        if (f.hLists) cudaFreeHost(f.hLists);
        if (f.hReports) cudaFreeHost(f.hReports);
        if (f.stream) cudaStreamDestroy(f.stream);
    }
    for (auto& w : s->worlds) {
        w->set.reset();
        if (w->saved) cudaFreeHost(w->saved);
    }
    cudaStreamSynchronize(s->ctx->stream);
    if (s->dSets) cudaFree(s->dSets);
    if (s->pool) cudaMemPoolDestroy(s->pool);
    bp_context* c = s->ctx;
    delete s;
    context_unref(c);
}

}  // namespace

extern "C" {

double bp_server_clock(void) { return host_clock(); }

int bp_server_create(bp_context* context, const bp_server_config* config, bp_server** out) {
    if (!context || !config || !out || config->max_worlds == 0) return BP_E_INVALID;
    bp_server* s = new (std::nothrow) bp_server();
    if (!s) return BP_E_ALLOC;
    s->ctx = context;
    context->refs++;
    s->cfg = *config;
    if (!s->cfg.hbm_budget_bytes) s->cfg.hbm_budget_bytes = kDefaultBudget;
    if (!s->cfg.streams) s->cfg.streams = kDefaultStreams;
    if (!s->cfg.threads_per_world) s->cfg.threads_per_world = kDefaultServeThreads;
    if (!s->cfg.warp_world_max) s->cfg.warp_world_max = kDefaultWarpMax;
    if (!s->cfg.group_width) s->cfg.group_width = kDefaultGroupWidth;
    const uint32_t gw = s->cfg.group_width;
    const uint32_t tw = s->cfg.threads_per_world;
    if ((tw != 128 && tw != 256 && tw != 512) || (gw != 32 && gw != 64 && gw != 128 && gw != 256) ||
        gw > tw || tw % gw) {
        server_free(s);
        return BP_E_INVALID;
    }
    if (s->cfg.flags & BP_SERVER_PER_WORLD) { s->cfg.streams = 1; s->cfg.max_batch_worlds = 1; }
    s->cap = s->cfg.max_batch_worlds ? std::min(s->cfg.max_batch_worlds, s->cfg.max_worlds) : s->cfg.max_worlds;
    DeviceGuard guard(context->device);
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = context->device;
    cudaError_t err = cudaMemPoolCreate(&s->pool, &props);
    if (!err) {
        uint64_t keep = ~0ull;  // freed worlds stay in the pool for the next admission
        err = cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    if (!err) err = cudaMalloc(&s->dSets, (size_t)s->cfg.max_worlds * sizeof(DState));
    s->flights.resize(s->cfg.streams);
    for (Flight& f : s->flights) {
        if (!err) err = cudaStreamCreateWithFlags(&f.stream, cudaStreamNonBlocking);
        if (!err) err = cudaEventCreate(&f.start);
        if (!err) err = cudaEventCreate(&f.done);
        if (!err) err = cudaMalloc(&f.dLists, (3ull * s->cap + 4) * sizeof(uint32_t));
        if (!err) err = cudaMalloc(&f.dReports, (size_t)s->cap * sizeof(bp_step_report));
        if (!err) err = cudaHostAlloc(&f.hLists, 3ull * s->cap * sizeof(uint32_t), cudaHostAllocDefault);
        if (!err) err = cudaHostAlloc(&f.hReports, (size_t)s->cap * sizeof(bp_step_report), cudaHostAllocDefault);
    }
    if (err) {
        server_free(s);
        return cuda_status(err);
    }
    for (int slot = (int)s->cfg.max_worlds - 1; slot >= 0; --slot) s->freeSlots.push_back(slot);
    *out = s;
    return BP_OK;
}

int bp_server_destroy(bp_server* server) {
    if (server) server_free(server);
    return BP_OK;
}

int bp_server_add_world(bp_server* s, const bp_world_desc* desc, const bp_world_input* input, uint32_t* world) {
    if (!s || !desc || !input) return BP_E_INVALID;
    if (s->worlds.size() >= s->cfg.max_worlds) return BP_E_CAPACITY;
    int st = validate(*desc, *input);
    if (st) return st;
    if (input->bubble_count > kCtaMaxBubbles || (desc->flags & BP_WORLD_FORCE_MULTI_CTA)) return BP_E_CAPACITY;
    std::unique_ptr<ServedWorld> sw(new (std::nothrow) ServedWorld());
    if (!sw) return BP_E_ALLOC;
    const bp_world_input& in = *input;
    sw->desc = *desc;
    sw->bubbles = copy_of(in.bubbles, in.bubble_count);
    sw->segments = copy_of(in.segments, in.segment_count);
    sw->bodies = copy_of(in.bodies, in.body_count);
    sw->bodyVertices = copy_of(in.body_vertices, 2ull * in.body_vertex_count);
    sw->bodyTriangles = copy_of(in.body_triangles, 3ull * in.body_triangle_count);
    sw->fields = copy_of(in.fields, in.field_count);
    sw->fieldVertices = copy_of(in.field_vertices, 2ull * in.field_vertex_count);
    sw->fieldIds = copy_of(in.field_object_ids, in.field_object_id_count);
    sw->bands = copy_of(in.bands, in.band_count);
    sw->motors = copy_of(in.motors, in.motor_count);
    sw->hasJoints = in.joint_ranges != nullptr;
    sw->jointEntities = in.joint_ranges ? in.joint_entity_count : 0u;
    sw->jointRanges = copy_of(in.joint_ranges, 2ull * sw->jointEntities);
    sw->jointPartners = copy_of(in.joint_partners, in.joint_partner_count);
    if (world) *world = (uint32_t)s->worlds.size();
    s->worlds.push_back(std::move(sw));
    return BP_OK;
}

int bp_server_submit(bp_server* s, uint32_t world, uint32_t steps, uint64_t* request_id) {
    if (!s || world >= s->worlds.size() || steps == 0) return BP_E_INVALID;
    Request r{};
    r.id = s->nextRequest++;
    r.steps = steps;
    r.submitted = host_clock();
    s->worlds[world]->pending.push_back(r);
    if (request_id) *request_id = r.id;
    return BP_OK;
}

int bp_server_progress(bp_server* s, uint32_t wait_us, uint32_t* completed) {
    if (!s) return BP_E_INVALID;
    uint32_t done = 0;
    int st = round_of(s, wait_us, done);
    if (completed) *completed = done;
    return st;
}

int bp_server_poll(bp_server* s, bp_server_completion* out, uint32_t capacity, uint32_t* count) {
    if (!s) return BP_E_INVALID;
    if (!out) {  // how many are waiting to be taken
        if (count) *count = (uint32_t)s->finished.size();
        return BP_OK;
    }
    uint32_t m = 0;
    while (m < capacity && !s->finished.empty()) {
        out[m++] = s->finished.front();
        s->finished.pop_front();
    }
    if (count) *count = m;
    return BP_OK;
}

int bp_server_pending(bp_server* s, uint32_t* waiting, uint32_t* in_flight) {
    if (!s) return BP_E_INVALID;
    uint32_t wq = 0, fl = 0;
    for (auto& w : s->worlds) {
        wq += (uint32_t)w->pending.size();
        fl += w->inflight ? 1u : 0u;
    }
    if (waiting) *waiting = wq;
    if (in_flight) *in_flight = fl;
    return BP_OK;
}

int bp_server_read_bubbles(bp_server* s, uint32_t world, bp_bubble* out, uint32_t capacity, uint32_t* count) {
    if (!s || world >= s->worlds.size()) return BP_E_INVALID;
    ServedWorld& sw = *s->worlds[world];
    if (sw.inflight) return BP_E_INFLIGHT;
    if (sw.set) return read_bubbles(*sw.set, 0, out, capacity, count);
    const uint32_t n = (uint32_t)sw.bubbles.size();
    if (count) *count = n;
    if (!out) return BP_OK;
    const uint32_t m = std::min(n, capacity);
    if (!sw.hasSaved) {
        std::memcpy(out, sw.bubbles.data(), m * sizeof(bp_bubble));
        return BP_OK;
    }
    // published state inside the pinned copy (parts in PersistentPart order, bubble arrays first)
    const size_t per[kPartBody] = {8, 8, 8, 8, 8, 4, 4, 8, 8, 8, 8, 4, 4};
    size_t at[kPartBody];
    size_t off = 0;
    for (int p = 0; p < kPartBody; ++p) { at[p] = off; off += per[p] * n; }
    const char* base = (const char*)sw.saved;
    for (uint32_t i = 0; i < m; ++i) {
        bp_bubble b = sw.bubbles[i];
        const float* pos = (const float*)(base + at[kPartPubPos]) + 2 * i;
        const float* start = (const float*)(base + at[kPartPubStart]) + 2 * i;
        const float* vel = (const float*)(base + at[kPartPubVel]) + 2 * i;
        const float* rotw = (const float*)(base + at[kPartPubRotw]) + 2 * i;
        b.center[0] = pos[0]; b.center[1] = pos[1];
        b.previous_center[0] = start[0]; b.previous_center[1] = start[1];
        b.velocity[0] = vel[0]; b.velocity[1] = vel[1];
        b.rotation = rotw[0]; b.angular_velocity = rotw[1];
        b.region_result = ((const uint32_t*)(base + at[kPartPubResult]))[i];
        b.flags = ((const uint32_t*)(base + at[kPartPubFlags]))[i] & 0xffu;
        out[i] = b;
    }
    return BP_OK;
}

int bp_server_read_stats(bp_server* s, bp_server_stats* out) {
    if (!s || !out) return BP_E_INVALID;
    std::memset(out, 0, sizeof(*out));
    out->worlds = (uint32_t)s->worlds.size();
    out->resident = s->resident;
    out->resident_bytes = s->residentBytes;
    out->hbm_budget_bytes = s->cfg.hbm_budget_bytes;
    out->admissions = s->admissions;
    out->evictions = s->evictions;
    out->batches = s->batches;
    out->batched_worlds = s->batchedWorlds;
    out->requests_done = s->requestsDone;
    out->bubble_substeps = s->bubbleSubsteps;
    out->device_ms = s->deviceMs;
    return BP_OK;
}

}  // extern "C"
