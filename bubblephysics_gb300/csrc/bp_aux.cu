// bp_aux.cu - small device kernels around the step: per-call report accumulation and the bulk state transfer used by
// the host-buffer (end-to-end) path.
#include <algorithm>

#include "bp_device.cuh"

namespace bp {

// Folds one step's reports into the per-call accumulator: the first failure sticks, substep counts add up, and the
// bubble-substeps of the step are summed into *total (bubbles x substeps, one warp-reduced atomic per warp).
__global__ void accumulate_kernel(const bp_step_report* rep, bp_step_report* acc, const uint32_t* sizes,
                                  unsigned long long* total, uint32_t count) {
    uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long local = 0;
    if (w < count) {
        bp_step_report r = rep[w];
        bp_step_report a = acc[w];
        uint32_t sum = a.substep_count + r.substep_count;
        uint32_t rebuilds = a.rebuild_count + r.rebuild_count;
        if (a.status == BP_OK) a = r;
        a.substep_count = sum;
        a.rebuild_count = rebuilds;
        acc[w] = a;
        local = (unsigned long long)sizes[w] * r.substep_count;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) local += __shfl_xor_sync(0xffffffffu, local, off);
    if ((threadIdx.x & 31u) == 0u && local) atomicAdd(total, local);
}

__global__ void write_state_kernel(const float4* in, float2* pos, float2* vel, float2* ppos, float2* pvel, uint64_t n) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 v = in[i];
    float2 p = make_float2(v.x, v.y), u = make_float2(v.z, v.w);
    pos[i] = p; ppos[i] = p; vel[i] = u; pvel[i] = u;
}

__global__ void read_state_kernel(float4* out, const float2* ppos, const float2* pvel, uint64_t n) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float2 p = ppos[i], u = pvel[i];
    out[i] = make_float4(p.x, p.y, u.x, u.y);
}

// Sum of n 32-bit values (v 16-byte aligned: a device allocation), four per 16-byte load, then the tail.
__global__ void sum_kernel(const uint32_t* v, uint64_t n, unsigned long long* total) {
    unsigned long long local = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x, first = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t quads = n / 4u;
    const uint4* q = (const uint4*)v;
    for (uint64_t i = first; i < quads; i += stride) {
        const uint4 x = q[i];
        local += (unsigned long long)x.x + x.y + x.z + x.w;
    }
    for (uint64_t i = quads * 4u + first; i < n; i += stride) local += v[i];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) local += __shfl_xor_sync(0xffffffffu, local, off);
    if ((threadIdx.x & 31u) == 0u && local) atomicAdd(total, local);
}

cudaError_t launch_sum(const uint32_t* v, uint64_t n, unsigned long long* total, cudaStream_t stream) {
    if (!n) return cudaSuccess;
    // one 16-byte load per thread where the values allow, at most 8 blocks per SM of 152
    const uint64_t blocks = std::min<uint64_t>(std::max<uint64_t>((n / 4u + 255u) / 256u, 1u), 152u * 8u);
    sum_kernel<<<(unsigned)blocks, 256, 0, stream>>>(v, n, total);
    return cudaGetLastError();
}

cudaError_t launch_accumulate(const bp_step_report* reports, bp_step_report* acc, const uint32_t* sizes,
                              unsigned long long* total, uint32_t count, cudaStream_t stream) {
    accumulate_kernel<<<(count + 255) / 256, 256, 0, stream>>>(reports, acc, sizes, total, count);
    return cudaGetLastError();
}
cudaError_t launch_write_state(const float4* in, float2* pos, float2* vel, float2* ppos, float2* pvel, uint64_t n,
                               cudaStream_t stream) {
    if (!n) return cudaSuccess;
    write_state_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(in, pos, vel, ppos, pvel, n);
    return cudaGetLastError();
}
cudaError_t launch_read_state(float4* out, const float2* ppos, const float2* pvel, uint64_t n, cudaStream_t stream) {
    if (!n) return cudaSuccess;
    read_state_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(out, ppos, pvel, n);
    return cudaGetLastError();
}

}  // namespace bp
