// bp_host.h - host-side structures shared by the C ABI (bp_capi.cu) and the serving loop (bp_server.cu): the
// context, the WorldSet that owns the device arrays of one world or of a batch, and the launchers of bp_step.cu.
#pragma once

#include <algorithm>
#include <cstdint>
#include <utility>
#include <vector>

#include "bp_device.cuh"

namespace bp {
cudaError_t launch_persistent(const DState& S, const QueueArgs& q, uint32_t threads, uint32_t blocks, cudaStream_t stream);
uint32_t persistent_blocks(const QueueArgs& q, uint32_t threads);
size_t persistent_smem(const QueueArgs& q, uint32_t threads);
cudaError_t launch_schedule(const DState& S, const uint32_t* candidates, uint32_t count, uint32_t warpMax,
                            uint32_t warpSubsteps, uint32_t* ctaList, uint32_t* warpList, uint32_t* queue, cudaStream_t stream);
int large_max_blocks(int threads);
cudaError_t launch_large(const DState& S, uint32_t wi, uint32_t B, int blocks, int threads, size_t smem,
                         cudaStream_t stream);
cudaError_t launch_contact_law(uint32_t mode, const float* in, float* out, uint32_t count, cudaStream_t stream);
cudaError_t launch_accumulate(const bp_step_report* reports, bp_step_report* acc, const uint32_t* sizes,
                              unsigned long long* total, uint32_t count, cudaStream_t stream);
cudaError_t launch_write_state(const float4* in, float2* pos, float2* vel, float2* ppos, float2* pvel, uint64_t n,
                               cudaStream_t stream);
cudaError_t launch_read_state(float4* out, const float2* ppos, const float2* pvel, uint64_t n, cudaStream_t stream);
void prepare_kernels();
cudaError_t launch_served(const DState* sets, const uint32_t* entrySlot, bp_step_report* reports, const QueueArgs& q,
                          uint32_t threads, uint32_t blocks, cudaStream_t stream);
cudaError_t launch_sum(const uint32_t* v, uint64_t n, unsigned long long* total, cudaStream_t stream);
cudaError_t launch_hit_test(const DState& S, const DWorld& W, const float2* queries, uint32_t queryCount,
                            const float2* cpoints, const uint32_t* ccounts, const float* shape, uint32_t stride,
                            const uint32_t* bubbleLayers, const uint32_t* segLayers, const uint32_t* bodyLayers,
                            long long* ids, uint32_t* layers, uint32_t* found, cudaStream_t stream);
cudaError_t launch_sensors(const DState& S, const DWorld& W, const void* sensors, uint32_t sensorCount,
                           const float2* verts, const uint8_t* allowed, uint8_t* state, uint8_t* kinds,
                           bp_sensor_event* events, uint32_t capacity, uint32_t* count, cudaStream_t stream);
size_t sensor_record_bytes();
void sensor_to_device(const bp_sensor& in, void* out);
// Contact began / ended events of one world's last step (bp_events.cu). Scratch: `entries` (event_entry_bytes() per
// record), `order` (a power of two >= records words), `heads` (records words).
struct EventArgsHost {
    const DContact* records;
    uint32_t deviceCount;
    const bp_contact* extra;
    uint32_t extraCount;
    const int64_t* ids;
    const DSegment* segments;
    const int64_t* interested;
    uint32_t interestedCount;
    const int64_t* removed;
    uint32_t removedCount;
    const unsigned long long* history;
    uint32_t historyCount;
    unsigned long long* nextHistory;
    uint32_t* nextHistoryCount;
    float step;
    void* entries;
    uint32_t* order;
    uint32_t* heads;
    bp_contact_event* out;
    uint32_t capacity;
    uint32_t* count;
};
cudaError_t launch_contact_events(const EventArgsHost& args, cudaStream_t stream);
size_t event_entry_bytes();
std::vector<float2> contour_directions(uint32_t stride);
cudaError_t launch_contours(const DState& S, const DWorld& W, float maxEdge, float tension, float clearance,
                            uint32_t stride, const float2* dirs, float2* points, uint32_t* counts, float* level,
                            float* shape, cudaStream_t stream);
}  // namespace bp

struct bp_context {
    int refs = 0;            // live worlds and batches that use this context
    bool released = false;   // bp_context_destroy was called; freed when the last user goes
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t start = nullptr, stop = nullptr;
    std::vector<cudaStream_t> side;
    int sms = 0;
};

namespace bp_host {
using namespace bp;

constexpr uint32_t kCtaMaxBubbles = 4096;
constexpr int kLargeThreads = 512;
constexpr uint32_t kLargeBubblesPerBlock = 512;  // bubbles per block of the whole-GPU team (one per thread)
constexpr uint32_t kDefaultThreads = 256;
constexpr uint32_t kDefaultWarpMax = 64;
constexpr uint32_t kWarpSubsteps = 16;   // a world that took more substeps last step gets a whole block
// shared-memory workspace of a block team: with the grid of 1,024-bubble worlds and its records a block takes 92 KB
// (2 blocks per SM, L1 keeps ~60 KB)
constexpr uint32_t kCtaWorkspaceCap = 64u * 1024u;
constexpr uint32_t kWarpWorkspaceCap = 10u * 1024u;  // per warp of a group team
constexpr uint32_t kDefaultGroupWidth = 32;
constexpr uint32_t kMaxDynamicSmem = 200u * 1024u;   // per block, set on the kernels by prepare_kernels()
constexpr uint32_t kTreeMinLeaves = 128;             // segments + bodies from which rigid candidates use the LBVH

struct DeviceGuard {
    int previous = -1;
    explicit DeviceGuard(int device) {
        cudaGetDevice(&previous);
        if (previous != device) cudaSetDevice(device);
    }
    ~DeviceGuard() {
        int now = -1;
        cudaGetDevice(&now);
        if (previous >= 0 && now != previous) cudaSetDevice(previous);
    }
};

inline uint32_t next_pow2(uint32_t v) {
    uint32_t p = 1;
    while (p < v) p <<= 1;
    return p;
}
inline uint32_t grid_buckets(uint32_t maxN) { return next_pow2(std::max<uint32_t>(2u * maxN, 32u)); }
// Shared-memory bytes of the hash grid (bucket ends, entries, entry records) of a team of `width` threads for worlds of
// up to maxN bubbles.
inline uint32_t team_grid_bytes(uint32_t maxN, uint32_t width) {
    return maxN ? 4u * grid_words(grid_buckets(maxN), maxN, width) : 0u;
}
inline uint32_t round4(uint32_t v) { return (v + 3u) & ~3u; }

inline int cuda_status(cudaError_t e) {
    if (e == cudaSuccess) return BP_OK;
    if (e == cudaErrorMemoryAllocation) return BP_E_ALLOC;
    return BP_E_CUDA;
}

template <class T> cudaError_t upload(T* dst, const T* src, uint64_t count, cudaStream_t stream) {
    if (count == 0) return cudaSuccess;
    return cudaMemcpyAsync(dst, src, count * sizeof(T), cudaMemcpyHostToDevice, stream);
}

struct WorldSet {
    bp_context* ctx = nullptr;
    uint32_t nWorlds = 0;
    uint32_t flags = 0;
    uint32_t fixedThreads = 0;
    std::vector<DWorld> hWorlds;
    std::vector<bp_bubble> hBubbles;        // as uploaded (static fields for readback)
    std::vector<int64_t> hSegIds, hBodyIds;
    std::vector<uint32_t> hSegLayers, hBodyLayers;  // drawing layers (hit tests)
    uint64_t totalBubbles = 0, totalRows = 0, totalBodyRows = 0, totalContacts = 0;
    uint32_t totalSegments = 0, totalBodies = 0;
    uint64_t totalTreeLeaves = 0;
    DState S{};
    DWorld* dWorlds = nullptr;
    bp_step_report* dReports = nullptr;
    bp_step_report* dAcc = nullptr;
    uint32_t* dSizes = nullptr;
    unsigned long long* dTotal = nullptr;
    float4* dStaging = nullptr;
    std::vector<void*> allocations;
    // scheduling: worlds stepped by a block (CTA team) or by a group of groupWidth threads (group queue), largest
    // first
    std::vector<uint32_t> ctaWorlds, warpWorlds;
    uint32_t* dCtaList = nullptr;
    uint32_t* dWarpList = nullptr;
    uint32_t* dQueue = nullptr;
    uint32_t* dQueueSingle = nullptr;       // queue of the one-world launches of the per-world path
    uint32_t* dCandidates = nullptr;        // worlds of the persistent kernel (all but the large ones)
    uint32_t nCandidates = 0;
    uint32_t threads = kDefaultThreads;
    bool staging = true;                    // keep worlds resident in shared memory during a step
    uint32_t warpMax = kDefaultWarpMax;     // worlds of at most this many bubbles go to the group queue
    uint32_t groupWidth = kDefaultGroupWidth;
    uint32_t blocks = 0;
    QueueArgs queue{};
    std::vector<uint32_t> largeWorlds;
    uint32_t largeB = 0, largeMaxN = 0;
    int largeBlocks = 0;
    uint32_t* dSingle = nullptr;            // world index list for per-world launches
    cudaGraphExec_t graph = nullptr;
    bool tuned = false;
    bool inflight = false;
    uint64_t bubbleSubsteps = 0, launches = 0;
    std::vector<float> lastHistory;

    // sensors of a single world (bp_world_set_sensors): device records, vertices, per-pair state and event kinds,
    // the event list of the last step and its length
    void* dSensors = nullptr;
    float2* dSensorVerts = nullptr;
    uint8_t* dSensorAllowed = nullptr;  // null: every pair
    uint8_t* dSensorState = nullptr;
    uint8_t* dSensorKinds = nullptr;
    bp_sensor_event* dSensorEvents = nullptr;
    uint32_t* dSensorCount = nullptr;
    uint32_t sensorCount = 0, sensorEventCapacity = 0;
    std::vector<void*> sensorAllocations;
    // contact events (bp_world_contact_events): the history of pair keys (double-buffered on the device), the scratch
    // of the compaction and the staging of its inputs and outputs, grown as needed
    struct EventState {
        unsigned long long* history[2] = {nullptr, nullptr};
        uint32_t historyCap = 0, historyCount = 0, current = 0;
        void* scratch = nullptr;
        size_t scratchBytes = 0;
    } events;
    // contour sample directions of every count up to contourDirStride (contour_directions), uploaded on first use
    float2* dContourDirs = nullptr;
    uint32_t contourDirStride = 0;
    cudaMemPool_t pool = nullptr;           // stream-ordered pool (server worlds); null: plain cudaMalloc
    bool planOnly = false;                  // server worlds: built without the batch schedule
    bool measureOnly = false;               // count the device bytes of a build without allocating or uploading
    uint64_t deviceBytes = 0;               // bytes of the allocations below

    ~WorldSet() {
        if (graph) cudaGraphExecDestroy(graph);
        for (void* p : sensorAllocations) cudaFree(p);
        cudaFree(events.history[0]);
        cudaFree(events.history[1]);
        cudaFree(events.scratch);
        cudaFree(dContourDirs);
        for (void* p : allocations) {
            if (pool) cudaFreeAsync(p, ctx->stream);
            else cudaFree(p);
        }
    }
    template <class T> T* alloc(uint64_t count, cudaError_t& err) {
        if (err != cudaSuccess) return nullptr;
        void* p = nullptr;
        size_t bytes = std::max<uint64_t>(count, 1) * sizeof(T);
        if (measureOnly) {
            deviceBytes += bytes;
            return nullptr;
        }
        err = pool ? cudaMallocFromPoolAsync(&p, bytes, pool, ctx->stream) : cudaMalloc(&p, bytes);
        if (err != cudaSuccess) return nullptr;
        allocations.push_back(p);
        deviceBytes += bytes;
        err = cudaMemsetAsync(p, 0, bytes, ctx->stream);
        return (T*)p;
    }
};

struct Snapshot {
    std::vector<std::pair<void*, size_t>> parts;
    std::vector<void*> copies;
};

int validate(const bp_world_desc& d, const bp_world_input& in);
int build_set(WorldSet& ws, bp_context* ctx, uint32_t count, const bp_world_desc* descs, const bp_world_input* inputs,
              bool single);
cudaError_t schedule(WorldSet& ws, uint32_t threads, uint32_t warpMax, uint32_t groupWidth);
// Shared-memory layout of the group queue for `threads`-wide blocks of groupWidth-thread groups whose largest world
// has maxN bubbles: false when even the grids do not fit; *wsCap = the workspace bytes a group can stage.
bool group_layout(uint32_t threads, uint32_t groupWidth, uint32_t maxN, uint32_t* wsCap);
// Device arrays whose contents carry over from one step to the next (what a snapshot or an eviction keeps), in this
// order: live state, published state, bodies, failed flags.
enum PersistentPart {
    kPartPos, kPartStart, kPartVel, kPartAcc, kPartRotw, kPartFlags, kPartResult,
    kPartPubPos, kPartPubStart, kPartPubVel, kPartPubRotw, kPartPubResult, kPartPubFlags,
    kPartBody, kPartPubBody, kPartFailed, kPartCount
};
std::vector<std::pair<void*, size_t>> persistent_parts(WorldSet& ws);
int read_bubbles(WorldSet& ws, uint32_t world, bp_bubble* out, uint32_t capacity, uint32_t* count);
void context_unref(bp_context* c);

}  // namespace bp_host
