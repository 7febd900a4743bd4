// bp_step_variant.cu - one variant of the persistent step kernels per object file. The build compiles this file once
// per (kernel, block width, tree) with -DBP_VARIANT_KIND=0 (batched worlds, persistent_step_kernel) or 1 (served
// worlds, served_step_kernel), -DBP_VARIANT_THREADS=128|256|512 and -DBP_VARIANT_TREE=0|1; each object defines the
// launchers of its variant declared in bp_step.cuh. The instantiations are the largest functions of the library, and
// one per translation unit lets them compile in parallel.
#include "bp_step.cuh"

#if !defined(BP_VARIANT_KIND) || !defined(BP_VARIANT_THREADS) || !defined(BP_VARIANT_TREE)
#error "bp_step_variant.cu is compiled once per variant with BP_VARIANT_KIND, BP_VARIANT_THREADS and BP_VARIANT_TREE"
#endif

#define BP_CAT3(a, b, c) a##_##b##_##c
#define BP_NAME(prefix, t, r) BP_CAT3(prefix, t, r)
#define BP_FN(prefix) BP_NAME(prefix, BP_VARIANT_THREADS, BP_VARIANT_TREE)

namespace bp {

#if BP_VARIANT_KIND == 0

cudaError_t BP_FN(persistent_launch)(const DState& S, const QueueArgs& q, uint32_t threads, uint32_t blocks,
                                     size_t smem, cudaStream_t stream) {
    persistent_step_kernel<BP_VARIANT_THREADS, BP_VARIANT_TREE != 0><<<blocks, threads, smem, stream>>>(S, q);
    return cudaGetLastError();
}

int BP_FN(persistent_blocks_per_sm)(uint32_t threads, size_t smem) {
    int perSm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, persistent_step_kernel<BP_VARIANT_THREADS, BP_VARIANT_TREE != 0>,
                                                  threads, smem);
    return perSm;
}

cudaError_t BP_FN(persistent_prepare)(int maxSmem) {
    return cudaFuncSetAttribute(persistent_step_kernel<BP_VARIANT_THREADS, BP_VARIANT_TREE != 0>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, maxSmem);
}

#else

cudaError_t BP_FN(served_launch)(const DState* sets, const uint32_t* entrySlot, bp_step_report* reports,
                                 const QueueArgs& q, uint32_t threads, uint32_t blocks, size_t smem,
                                 cudaStream_t stream) {
    served_step_kernel<BP_VARIANT_THREADS, BP_VARIANT_TREE != 0>
        <<<blocks, threads, smem, stream>>>(sets, entrySlot, reports, q);
    return cudaGetLastError();
}

cudaError_t BP_FN(served_prepare)(int maxSmem) {
    return cudaFuncSetAttribute(served_step_kernel<BP_VARIANT_THREADS, BP_VARIANT_TREE != 0>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, maxSmem);
}

#endif

}  // namespace bp
