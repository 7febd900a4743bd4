// bp_step.cu - launchers of the bubble step (bp_step.cuh) and its small kernels: the whole-GPU cooperative step of one
// large world, the on-device scheduler of the batched queues, and the contact-law known-answer kernel. The persistent
// kernels themselves are compiled per variant in bp_step_variant.cu.
#include "bp_step.cuh"

namespace bp {

// Cooperative launch: every block steps world `wi` together; the hash grid lives in global memory.
__global__ void __launch_bounds__(512) large_step_kernel(DState S, uint32_t wi, uint32_t B) {
    __shared__ BlockScratch sh;
    __shared__ TeamState ts;
    GridTeam team{&sh, S.barrier, S.errorFlag, S.gpv, S.gpo, nullptr, 0u, false};
    world_step<GridTeam, true>(S, wi, team, S.gbuckets, S.gentries, S.grecords, B, nullptr, 0u, ts);
}

// Contact law known-answer kernel: mode 0 eps(q), 1 wall law, 2 pair law; 8 floats in / out per case.
__global__ void contact_law_kernel(uint32_t mode, const float* in, float* out, uint32_t count) {
    uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= count) return;
    const float* a = in + 8 * c;
    float* o = out + 8 * c;
    for (int q = 0; q < 8; ++q) o[q] = 0.0f;
    if (mode == 0u) o[0] = eps_from_ratio(a[0]);
    else if (mode == 1u) { Law l = wall_law(a[0], a[1], a[2]); o[0] = l.force; o[1] = l.epsA; o[2] = l.stiffness; }
    else { Law l = pair_law(a[0], a[1], a[2], a[3], a[4]); o[0] = l.force; o[1] = l.epsA; o[2] = l.epsB; o[3] = l.stiffness; }
}

// ------------------------------------------------------------------------------------------------------------------
// Host launchers
// ------------------------------------------------------------------------------------------------------------------
// On-device scheduler, run after every batched step: predicted cost of a world = bubbles x (last step's substeps + 2)
// (the +2 stands for the grid build and the end-of-step work); worlds are sorted by cost, most expensive first, and
// split into the warp queue (at most warpMax bubbles and at most warpSubsteps substeps last step) and the CTA queue.
// One block; keys (inverted cost << 32 | world) are sorted bitonically in shared memory.
__global__ void __launch_bounds__(1024) schedule_kernel(const DWorld* worlds, const bp_step_report* reports,
                                                        const uint32_t* failed, const uint32_t* candidates, uint32_t count,
                                                        uint32_t warpMax, uint32_t warpSubsteps, uint32_t* ctaList,
                                                        uint32_t* warpList, uint32_t* queue) {
    extern __shared__ unsigned long long keys[];
    __shared__ BlockScratch sh;
    uint32_t P = 1;
    while (P < count) P <<= 1;
    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
        unsigned long long key = ~0ull;
        if (i < count) {
            uint32_t w = candidates[i];
            uint32_t n = worlds[w].n;
            uint32_t sub = failed[w] ? 0u : reports[w].substep_count;
            unsigned long long cost = failed[w] ? 0ull : (unsigned long long)n * (sub + 2u);
            uint32_t c32 = cost > 0xffffffffull ? 0xffffffffu : (uint32_t)cost;
            key = ((unsigned long long)(0xffffffffu - c32) << 32) | w;
        }
        keys[i] = key;
    }
    __syncthreads();
    for (uint32_t size = 2; size <= P; size <<= 1) {
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
            for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
                uint32_t j = i ^ stride;
                if (j > i) {
                    bool up = (i & size) == 0;
                    unsigned long long a = keys[i], b = keys[j];
                    if ((a > b) == up) { keys[i] = b; keys[j] = a; }
                }
            }
            __syncthreads();
        }
    }
    // stable split into the two queues, in cost order
    uint32_t nCta = 0, nWarp = 0;
    for (uint32_t base = 0; base < count; base += blockDim.x) {
        uint32_t i = base + threadIdx.x;
        uint32_t w = 0, isWarp = 0, valid = i < count ? 1u : 0u;
        if (valid) {
            w = (uint32_t)(keys[i] & 0xffffffffull);
            uint32_t sub = reports[w].substep_count;
            isWarp = (worlds[w].n <= warpMax && sub <= warpSubsteps) ? 1u : 0u;
        }
        uint32_t tw, tc;
        uint32_t pw = block_excl_scan(valid & isWarp, &tw, sh);
        uint32_t pc = block_excl_scan(valid & (isWarp ^ 1u), &tc, sh);
        if (valid) {
            if (isWarp) warpList[nWarp + pw] = w;
            else ctaList[nCta + pc] = w;
        }
        nWarp += tw;
        nCta += tc;
    }
    if (threadIdx.x == 0) { queue[2] = nCta; queue[3] = nWarp; }
}

cudaError_t launch_schedule(const DState& S, const uint32_t* candidates, uint32_t count, uint32_t warpMax,
                            uint32_t warpSubsteps, uint32_t* ctaList, uint32_t* warpList, uint32_t* queue, cudaStream_t stream) {
    if (count == 0u || count > 16384u) return cudaSuccess;
    uint32_t P = 1;
    while (P < count) P <<= 1;
    schedule_kernel<<<1, 1024, (size_t)P * sizeof(unsigned long long), stream>>>(
        S.worlds, S.reports, S.failed, candidates, count, warpMax, warpSubsteps, ctaList, warpList, queue);
    return cudaGetLastError();
}

size_t persistent_smem(const QueueArgs& q, uint32_t threads) {
    size_t cta = (size_t)(q.nCta ? grid_words(q.ctaB, q.ctaMaxN, threads) + q.ctaWsWords : 0);
    size_t warp = (size_t)(q.nWarp ? (threads / (q.groupWidth ? q.groupWidth : 32u)) * group_slice_words(q) : 0);
    return (cta > warp ? cta : warp) * sizeof(uint32_t);
}

// Block width of the variant that serves `threads` (128, 256 or 512).
static uint32_t variant_width(uint32_t threads) { return threads <= 128u ? 128u : threads <= 256u ? 256u : 512u; }

cudaError_t launch_persistent(const DState& S, const QueueArgs& q, uint32_t threads, uint32_t blocks, cudaStream_t stream) {
    if (q.nCta + q.nWarp == 0u) return cudaSuccess;
    size_t smem = persistent_smem(q, threads);
    if (smem > 200u * 1024u) return cudaErrorInvalidValue;  // schedule() keeps every configuration below this
    cudaError_t err = cudaMemsetAsync(q.queue, 0, 2 * sizeof(uint32_t), stream);
    if (err) return err;
    const uint32_t width = variant_width(threads), tree = q.tree ? 1u : 0u;
#define BP_LAUNCH_PERSISTENT(T, R) \
    if (width == T && tree == R) return persistent_launch_##T##_##R(S, q, threads, blocks, smem, stream);
    BP_STEP_VARIANTS(BP_LAUNCH_PERSISTENT)
#undef BP_LAUNCH_PERSISTENT
    return cudaErrorInvalidValue;
}

cudaError_t launch_served(const DState* sets, const uint32_t* entrySlot, bp_step_report* reports, const QueueArgs& q,
                          uint32_t threads, uint32_t blocks, cudaStream_t stream) {
    if (q.nCta + q.nWarp == 0u) return cudaSuccess;
    size_t smem = persistent_smem(q, threads);
    if (smem > 200u * 1024u) return cudaErrorInvalidValue;
    cudaError_t err = cudaMemsetAsync(q.queue, 0, 2 * sizeof(uint32_t), stream);
    if (err) return err;
    const uint32_t width = variant_width(threads), tree = q.tree ? 1u : 0u;
#define BP_LAUNCH_SERVED(T, R) \
    if (width == T && tree == R) return served_launch_##T##_##R(sets, entrySlot, reports, q, threads, blocks, smem, stream);
    BP_STEP_VARIANTS(BP_LAUNCH_SERVED)
#undef BP_LAUNCH_SERVED
    return cudaErrorInvalidValue;
}

// Blocks of the persistent kernel that fit on the GPU at once (the grid size of a full launch).
uint32_t persistent_blocks(const QueueArgs& q, uint32_t threads) {
    int device = 0, sms = 0, perSm = 0;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    size_t smem = persistent_smem(q, threads);
    const uint32_t width = variant_width(threads), tree = q.tree ? 1u : 0u;
#define BP_OCCUPANCY(T, R) \
    if (width == T && tree == R) perSm = persistent_blocks_per_sm_##T##_##R(threads, smem);
    BP_STEP_VARIANTS(BP_OCCUPANCY)
#undef BP_OCCUPANCY
    return (uint32_t)(sms * (perSm > 0 ? perSm : 1));
}

// Function attributes are set once per process before any launch (never inside a stream capture).
void prepare_kernels() {
    static bool done = false;
    if (done) return;
    done = true;
#define BP_PREPARE(T, R)                          \
    persistent_prepare_##T##_##R(200 * 1024); \
    served_prepare_##T##_##R(200 * 1024);
    BP_STEP_VARIANTS(BP_PREPARE)
#undef BP_PREPARE
    cudaFuncSetAttribute(schedule_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 16384 * 8);
}

int large_max_blocks(int threads) {
    int device = 0, sms = 0, perSm = 0;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, large_step_kernel, threads, 0);
    return sms * (perSm > 0 ? perSm : 1);
}

cudaError_t launch_large(const DState& S, uint32_t wi, uint32_t B, int blocks, int threads, size_t smem,
                         cudaStream_t stream) {
    // the grid barrier counts arrivals from zero in every launch (the block count differs between worlds)
    cudaError_t err = cudaMemsetAsync(S.barrier, 0, sizeof(unsigned int), stream);
    if (err != cudaSuccess) return err;
    DState copy = S;
    void* args[] = {&copy, &wi, &B};
    return cudaLaunchCooperativeKernel((const void*)large_step_kernel, dim3(blocks), dim3(threads), args, smem, stream);
}

cudaError_t launch_contact_law(uint32_t mode, const float* in, float* out, uint32_t count, cudaStream_t stream) {
    if (count == 0u) return cudaSuccess;
    contact_law_kernel<<<(count + 127) / 128, 128, 0, stream>>>(mode, in, out, count);
    return cudaGetLastError();
}

}  // namespace bp
