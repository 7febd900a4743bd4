// bp_noalloc.cu - the allocation-free single-world step (bp_world_step_noalloc).
#include "bp_step.cuh"

// ==================================================================================================================
// Allocation-free single-world step.
//
// Some callers cannot allocate device memory at the moment they step a world: code that runs inside a host framework
// that owns every device allocation through its own pool (game engines, plugin hosts), real-time threads that must not
// take the driver's allocation locks, or memory-capped processes that reserved all the device memory they may use up
// front. bp_world_step_noalloc serves them: the caller passes device buffers for the inputs and outputs, and every
// working array of the step is carved out of one file-scope device array of fixed size, so the call itself allocates
// nothing. The array exists once per GPU that loads the library and stays until the process exits.
// ==================================================================================================================

#define BP_NOALLOC_MAX_BUBBLES 1024u
#define BP_NOALLOC_MAX_SEGMENTS 256u
#define BP_NOALLOC_MAX_CANDIDATE_LIMIT 32u
#define BP_NOALLOC_CONTACTS_PER_BUBBLE 4u

namespace bp {
namespace {

constexpr uint32_t kNaN = BP_NOALLOC_MAX_BUBBLES;
constexpr uint32_t kNaS = BP_NOALLOC_MAX_SEGMENTS;
constexpr uint32_t kNaK = BP_NOALLOC_MAX_CANDIDATE_LIMIT;
constexpr uint32_t kNaContacts = kNaN * BP_NOALLOC_CONTACTS_PER_BUBBLE + 64u;
constexpr uint32_t kNoAllocThreads = 256;  // one block steps the world

// Carves the scratch layout (all offsets 256-byte aligned) from `base`; with base == 0 it returns the size.
struct NoAllocLayout {
    size_t bytes = 0;
    template <class T> constexpr T* take(char* base, size_t count) {
        size_t off = bytes;
        bytes += (count * sizeof(T) + 255u) & ~(size_t)255u;
        return base ? (T*)(base + off) : nullptr;
    }
    DWorld* world = nullptr;
    constexpr DState make(char* base) {
        DState S{};
        world = take<DWorld>(base, 1);
        S.worlds = world;
        S.history = take<float>(base, kFrameLimit);
        S.contactCount = take<uint32_t>(base, 1);
        S.pos = take<float2>(base, kNaN); S.start = take<float2>(base, kNaN); S.vel = take<float2>(base, kNaN);
        S.acc = take<float2>(base, kNaN); S.a0 = take<float2>(base, kNaN); S.ref = take<float2>(base, kNaN);
        S.rotw = take<float2>(base, kNaN);
        S.phys = take<float4>(base, kNaN);
        S.margin = take<float>(base, kNaN);
        S.id = take<int64_t>(base, kNaN);
        S.flags = take<uint32_t>(base, kNaN); S.result = take<uint32_t>(base, kNaN);
        S.filter = take<uint2>(base, kNaN);
        S.cell = take<longlong2>(base, kNaN); S.acell = take<longlong2>(base, kNaN);
        S.candRow = take<uint32_t>(base, (size_t)kNaN * kNaK); S.candCount = take<uint2>(base, kNaN);
        S.pairTotal = take<uint32_t>(base, kNaN);
        S.adj = take<uint32_t>(base, (size_t)kNaN * kNaK); S.deg = take<uint32_t>(base, kNaN);
        S.pPos = take<float2>(base, kNaN); S.pStart = take<float2>(base, kNaN); S.pVel = take<float2>(base, kNaN);
        S.pRotw = take<float2>(base, kNaN); S.pResult = take<uint32_t>(base, kNaN); S.pFlags = take<uint32_t>(base, kNaN);
        S.seg = take<DSegment>(base, kNaS);
        S.segBox = take<RigidBox>(base, kNaS);
        S.contacts = take<DContact>(base, kNaContacts);
        S.failed = take<uint32_t>(base, 1);
        S.scanA = take<uint32_t>(base, kNaN); S.scanB = take<uint32_t>(base, kNaN);
        return S;
    }
};

constexpr size_t noalloc_bytes() {
    // 1024 bubbles: ~0.5 MB of state and rows, 4160 contact records, 256 segments; rounded up generously
    return (size_t)1 << 20;
}

constexpr size_t noalloc_layout_bytes() {
    NoAllocLayout layout;
    layout.make(nullptr);
    return layout.bytes;
}
static_assert(noalloc_layout_bytes() <= noalloc_bytes(), "the scratch layout must fit the fixed device array");

}  // namespace

// The scratch array itself: 1 MiB, 256-byte aligned. Host code must not use its name as an address.
static __device__ __align__(256) unsigned char g_noalloc_scratch[noalloc_bytes()];

// Unpacks the caller's records into the scratch state, steps `steps` times, packs the bubbles back (in place).
__global__ void __launch_bounds__(kNoAllocThreads) noalloc_step_kernel(DState S, DWorld W, bp_bubble* bubbles, const bp_segment* segments,
                                                           uint32_t steps, bp_step_report* reports, uint32_t B) {
    __shared__ BlockScratch sh;
    __shared__ TeamState ts;
    CtaTeam team{&sh};
    const uint32_t n = W.n, T = blockDim.x, r = threadIdx.x;
    if (r == 0) {
        *const_cast<DWorld*>(S.worlds) = W;
        S.failed[0] = 0u;
        S.contactCount[0] = 0u;
    }
    for (uint32_t i = r; i < n; i += T) {
        const bp_bubble b = bubbles[i];
        S.pos[i] = make_float2(b.center[0], b.center[1]);
        S.start[i] = make_float2(b.previous_center[0], b.previous_center[1]);
        S.vel[i] = make_float2(b.velocity[0], b.velocity[1]);
        S.rotw[i] = make_float2(b.rotation, b.angular_velocity);
        S.phys[i] = make_float4(b.radius, b.inverse_mass, b.contact_stiffness, b.damping);
        const_cast<int64_t*>(S.id)[i] = b.id;
        uint32_t f = (b.flags & 0xffu) | (b.region_result == 1u ? kRemoved : 0u);
        S.flags[i] = f;
        S.result[i] = b.region_result == 1u ? 1u : 0u;
        const_cast<uint2*>(S.filter)[i] = make_uint2(b.category, b.mask);
        S.pPos[i] = S.pos[i]; S.pStart[i] = S.start[i]; S.pVel[i] = S.vel[i]; S.pRotw[i] = S.rotw[i];
        S.pResult[i] = S.result[i]; S.pFlags[i] = f;
    }
    for (uint32_t j = r; j < W.s; j += T) {
        const bp_segment g = segments[j];
        DSegment d;
        d.a = make_float2(g.a[0], g.a[1]); d.b = make_float2(g.b[0], g.b[1]);
        d.prev = make_float2(g.previous_start[0], g.previous_start[1]);
        d.outward = g.outward_sign; d.allowed = g.allowed_side;
        d.flags = g.flags; d.cat = g.category; d.mask = g.mask; d.pad = 0u;
        d.id = g.id; d.owner = g.owner_id;
        const_cast<DSegment*>(S.seg)[j] = d;
    }
    // ids must be strictly ascending (what bp_world_create checks on the host): otherwise nothing is stepped and
    // every report says BP_E_INVALID
    uint32_t unsorted = 0u;
    for (uint32_t i = r + 1; i < n; i += T) unsorted |= bubbles[i - 1].id < bubbles[i].id ? 0u : 1u;
    if (__syncthreads_or(unsorted)) {
        for (uint32_t q = r; q < steps; q += T) {
            bp_step_report invalid{};
            invalid.status = BP_E_INVALID;
            reports[q] = invalid;
        }
        return;
    }
    uint32_t* buckets = g_dynamic_smem;
    uint32_t* entries = g_dynamic_smem + B;
    float4* records = (float4*)(g_dynamic_smem + round4_words(B + (n ? n : 1u)));
    uint32_t* ws = g_dynamic_smem + grid_words(B, n ? n : 1u, blockDim.x);
    const uint32_t wsWords = workspace_bytes(n, W.s, 0u) / 4u + 4u;
    for (uint32_t s = 0; s < steps; ++s) {
        if (r == 0) {
            bp_step_report zero{};
            reports[s] = zero;
            ts.G = S;
            ts.G.reports = reports + s;
        }
        __syncthreads();
        world_step<CtaTeam, false>(ts.G, 0u, team, buckets, entries, records, B, ws, wsWords, ts);
        __syncthreads();
        if (S.failed[0]) {  // a failed step publishes nothing and stops the world: later steps report it
            for (uint32_t q = s + 1 + r; q < steps; q += T) {
                bp_step_report failedReport{};
                failedReport.status = BP_E_WORLD_FAILED;
                reports[q] = failedReport;
            }
            break;
        }
    }
    __syncthreads();
    for (uint32_t i = r; i < n; i += T) {
        bp_bubble b = bubbles[i];
        b.center[0] = S.pPos[i].x; b.center[1] = S.pPos[i].y;
        b.previous_center[0] = S.pStart[i].x; b.previous_center[1] = S.pStart[i].y;
        b.velocity[0] = S.pVel[i].x; b.velocity[1] = S.pVel[i].y;
        b.rotation = S.pRotw[i].x; b.angular_velocity = S.pRotw[i].y;
        b.region_result = S.pResult[i];
        bubbles[i] = b;
    }
}

}  // namespace bp

extern "C" int bp_world_step_noalloc(const bp_world_desc* desc, bp_bubble* bubbles, uint32_t bubble_count,
                                     const bp_segment* segments, uint32_t segment_count, uint32_t steps,
                                     bp_step_report* reports, void* stream) {
    using namespace bp;
    if (!desc || (!bubbles && bubble_count) || (!segments && segment_count) || (!reports && steps)) return BP_E_INVALID;
    const uint32_t k = desc->candidate_limit == 0 ? kNaK : desc->candidate_limit;
    if (bubble_count > kNaN || segment_count > kNaS || k > kNaK) return BP_E_CAPACITY;
    if (!(desc->time_step > 0.0f) || !isfinite(desc->time_step)) return BP_E_INVALID;
    if (steps == 0) return BP_OK;
    // The array's device address is looked up on every call, with the caller's device current: it is a host-side
    // lookup that allocates nothing, and it stays right when the context was torn down and made again (the module
    // is then loaded anew and the array may sit elsewhere). The shared-memory attribute is set the same way.
    void* base = nullptr;
    cudaError_t err = cudaGetSymbolAddress(&base, g_noalloc_scratch);
    if (err != cudaSuccess || !base) return BP_E_CUDA;
    if (cudaFuncSetAttribute(noalloc_step_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024) != cudaSuccess)
        return BP_E_CUDA;
    NoAllocLayout layout;
    DState S = layout.make((char*)base);
    DWorld W{};
    W.boff = 0; W.n = bubble_count; W.soff = 0; W.s = segment_count;
    W.k = k;
    W.flags = desc->flags & ~(uint32_t)(BP_WORLD_INJECT_STATE | BP_WORLD_FORCE_MULTI_CTA);
    W.contactCap = bubble_count * BP_NOALLOC_CONTACTS_PER_BUBBLE + 64u;
    W.rowOff = 0; W.bodyRowOff = 0; W.contactOff = 0;
    W.dt = desc->time_step; W.sepTol = desc->separation_tolerance; W.contactTol = desc->contact_tolerance;
    W.split = desc->substep_split_multiplier;
    W.rmin = make_float2(desc->region[0], desc->region[1]);
    W.rmax = make_float2(desc->region[2], desc->region[3]);
    W.gforce = make_float2(desc->global_force[0], desc->global_force[1]);
    W.gravity = make_float2(desc->gravity[0], desc->gravity[1]);
    const uint32_t maxN = bubble_count ? bubble_count : 1u;
    uint32_t B = 32u;
    while (B < 2u * maxN) B <<= 1;
    const size_t smem = ((size_t)grid_words(B, maxN, kNoAllocThreads) + workspace_bytes(bubble_count, segment_count, 0u) / 4u + 4u) * 4u;
    noalloc_step_kernel<<<1, kNoAllocThreads, smem, (cudaStream_t)stream>>>(S, W, bubbles, segments, steps, reports, B);
    return cudaGetLastError() == cudaSuccess ? BP_OK : BP_E_CUDA;
}
