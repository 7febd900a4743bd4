// bp_team.cuh - execution teams for the world step: a CTA (one world per thread block), a group of warps of a block
// (one world per group, several groups per block) or the whole grid of a cooperative launch (one large world). All
// provide sync, deterministic (value, owner) reductions with the lower index winning ties, exclusive scans and sums. The grid barrier is bounded: a wait that runs out sets the error
// flag and every block leaves the kernel at its next check, so no launch can spin forever.
#pragma once

#include "bp_device.cuh"

namespace bp {

constexpr unsigned long long kBarrierSpinLimit = 20000000ull;  // about 1-4 s of __nanosleep(32) polls

struct ValOwner {
    float v;
    uint32_t o;
};

__device__ __forceinline__ ValOwner pick_max(ValOwner a, ValOwner b) {
    return (b.v > a.v || (b.v == a.v && b.o < a.o)) ? b : a;
}
__device__ __forceinline__ ValOwner pick_min(ValOwner a, ValOwner b) {
    return (b.v < a.v || (b.v == a.v && b.o < a.o)) ? b : a;
}

template <bool kMax> __device__ __forceinline__ ValOwner warp_pick(ValOwner x) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        ValOwner y;
        y.v = __shfl_xor_sync(0xffffffffu, x.v, off);
        y.o = __shfl_xor_sync(0xffffffffu, x.o, off);
        x = kMax ? pick_max(x, y) : pick_min(x, y);
    }
    return x;
}

__device__ __forceinline__ uint32_t warp_sum(uint32_t x) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
    return x;
}
__device__ __forceinline__ uint32_t warp_max(uint32_t x) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) x = max(x, __shfl_xor_sync(0xffffffffu, x, off));
    return x;
}
__device__ __forceinline__ float warp_fmax(float x) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) x = fmaxf(x, __shfl_xor_sync(0xffffffffu, x, off));
    return x;
}
__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t x) {
    const uint32_t lane = threadIdx.x & 31u;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= (uint32_t)off) x += y;
    }
    return x;
}

// Shared scratch used by the block-level primitives (one per CTA).
struct BlockScratch {
    float fv[32];
    uint32_t uo[32];
    float fv2[32];
    uint32_t uo2[32];
    uint32_t u[33];
    float bcastF[4];
    uint32_t bcastU[8];
    uint32_t u4[4][33];
};

// Threads that reduce together: the whole block (BlockShape), or a group of consecutive warps of it (GroupShape),
// synchronised by a named barrier of its own so the groups of a block run independently. Every reduction below ends
// with a synchronisation of the shape, so it also orders the shared-memory writes made before it.
struct BlockShape {
    __device__ __forceinline__ uint32_t tid() const { return threadIdx.x; }
    __device__ __forceinline__ uint32_t count() const { return blockDim.x; }
    __device__ __forceinline__ void sync() const { __syncthreads(); }
};
struct GroupShape {
    uint32_t base;   // first thread of the group (a multiple of 32)
    uint32_t width;  // threads in the group (a multiple of 32)
    uint32_t id;     // named barrier of the group (1..15); a one-warp group synchronises with __syncwarp
    __device__ __forceinline__ uint32_t tid() const { return threadIdx.x - base; }
    __device__ __forceinline__ uint32_t count() const { return width; }
    __device__ __forceinline__ void sync() const {
        if (width == 32u) __syncwarp();
        else asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(width) : "memory");
    }
};

// Four sums (kMaxMask bit c set: maximum instead of sum for component c) in one reduction over the shape.
template <uint32_t kMaxMask, class Shape>
__device__ __forceinline__ void shape_reduce4(uint32_t (&v)[4], BlockScratch& sh, const Shape& g) {
    const uint32_t lane = threadIdx.x & 31u, warp = g.tid() >> 5, nw = (g.count() + 31u) >> 5;
#pragma unroll
    for (int c = 0; c < 4; ++c) v[c] = ((kMaxMask >> c) & 1u) ? warp_max(v[c]) : warp_sum(v[c]);
    if (nw == 1u) { g.sync(); return; }
    g.sync();
    if (lane == 0) {
#pragma unroll
        for (int c = 0; c < 4; ++c) sh.u4[c][warp] = v[c];
    }
    g.sync();
    if (warp == 0) {
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            uint32_t y = lane < nw ? sh.u4[c][lane] : 0u;
            y = ((kMaxMask >> c) & 1u) ? warp_max(y) : warp_sum(y);
            if (lane == 0) sh.u4[c][32] = y;
        }
    }
    g.sync();
#pragma unroll
    for (int c = 0; c < 4; ++c) v[c] = sh.u4[c][32];
}
template <uint32_t kMaxMask> __device__ __forceinline__ void block_reduce4(uint32_t (&v)[4], BlockScratch& sh) {
    shape_reduce4<kMaxMask>(v, sh, BlockShape{});
}

// (value, owner) reduction over the shape; result broadcast to every thread.
template <bool kMax, class Shape> __device__ __forceinline__ ValOwner shape_pick(ValOwner x, BlockScratch& sh, const Shape& g) {
    const uint32_t lane = threadIdx.x & 31u, warp = g.tid() >> 5, nw = (g.count() + 31u) >> 5;
    x = warp_pick<kMax>(x);
    if (nw == 1u) { g.sync(); return x; }
    g.sync();
    if (lane == 0) { sh.fv[warp] = x.v; sh.uo[warp] = x.o; }
    g.sync();
    if (warp == 0) {
        ValOwner y = lane < nw ? ValOwner{sh.fv[lane], sh.uo[lane]} : x;
        y = warp_pick<kMax>(y);
        if (lane == 0) { sh.fv[0] = y.v; sh.uo[0] = y.o; }
    }
    g.sync();
    return ValOwner{sh.fv[0], sh.uo[0]};
}
template <bool kMax> __device__ __forceinline__ ValOwner block_pick(ValOwner x, BlockScratch& sh) {
    return shape_pick<kMax>(x, sh, BlockShape{});
}

// Two (value, owner) reductions in the barriers of one (kMaxA / kMaxB: maximum or minimum).
template <bool kMaxA, bool kMaxB, class Shape>
__device__ __forceinline__ void shape_pick2(ValOwner& a, ValOwner& b, BlockScratch& sh, const Shape& g) {
    const uint32_t lane = threadIdx.x & 31u, warp = g.tid() >> 5, nw = (g.count() + 31u) >> 5;
    a = warp_pick<kMaxA>(a);
    b = warp_pick<kMaxB>(b);
    if (nw == 1u) { g.sync(); return; }
    g.sync();
    if (lane == 0) { sh.fv[warp] = a.v; sh.uo[warp] = a.o; sh.fv2[warp] = b.v; sh.uo2[warp] = b.o; }
    g.sync();
    if (warp == 0) {
        ValOwner x = lane < nw ? ValOwner{sh.fv[lane], sh.uo[lane]} : a;
        ValOwner y = lane < nw ? ValOwner{sh.fv2[lane], sh.uo2[lane]} : b;
        x = warp_pick<kMaxA>(x);
        y = warp_pick<kMaxB>(y);
        if (lane == 0) { sh.fv[0] = x.v; sh.uo[0] = x.o; sh.fv2[0] = y.v; sh.uo2[0] = y.o; }
    }
    g.sync();
    a = ValOwner{sh.fv[0], sh.uo[0]};
    b = ValOwner{sh.fv2[0], sh.uo2[0]};
}
template <bool kMaxA, bool kMaxB>
__device__ __forceinline__ void block_pick2(ValOwner& a, ValOwner& b, BlockScratch& sh) {
    shape_pick2<kMaxA, kMaxB>(a, b, sh, BlockShape{});
}

template <class Shape> __device__ __forceinline__ uint32_t shape_reduce_u(uint32_t x, bool isMax, BlockScratch& sh, const Shape& g) {
    const uint32_t lane = threadIdx.x & 31u, warp = g.tid() >> 5, nw = (g.count() + 31u) >> 5;
    x = isMax ? warp_max(x) : warp_sum(x);
    if (nw == 1u) { g.sync(); return x; }
    g.sync();
    if (lane == 0) sh.u[warp] = x;
    g.sync();
    if (warp == 0) {
        uint32_t y = lane < nw ? sh.u[lane] : 0u;
        y = isMax ? warp_max(y) : warp_sum(y);
        if (lane == 0) sh.u[32] = y;
    }
    g.sync();
    return sh.u[32];
}
__device__ __forceinline__ uint32_t block_sum(uint32_t x, BlockScratch& sh) { return shape_reduce_u(x, false, sh, BlockShape{}); }
__device__ __forceinline__ uint32_t block_max(uint32_t x, BlockScratch& sh) { return shape_reduce_u(x, true, sh, BlockShape{}); }

template <class Shape> __device__ __forceinline__ float shape_fmax(float x, BlockScratch& sh, const Shape& g) {
    const uint32_t lane = threadIdx.x & 31u, warp = g.tid() >> 5, nw = (g.count() + 31u) >> 5;
    x = warp_fmax(x);
    if (nw == 1u) { g.sync(); return x; }
    g.sync();
    if (lane == 0) sh.fv[warp] = x;
    g.sync();
    if (warp == 0) {
        float y = lane < nw ? sh.fv[lane] : x;
        y = warp_fmax(y);
        if (lane == 0) sh.fv[0] = y;
    }
    g.sync();
    return sh.fv[0];
}
__device__ __forceinline__ float block_fmax(float x, BlockScratch& sh) { return shape_fmax(x, sh, BlockShape{}); }

// Exclusive scan of one value per thread over the shape; *total receives the shape's total.
template <class Shape>
__device__ __forceinline__ uint32_t shape_excl_scan(uint32_t x, uint32_t* total, BlockScratch& sh, const Shape& g) {
    const uint32_t lane = threadIdx.x & 31u, warp = g.tid() >> 5, nw = (g.count() + 31u) >> 5;
    uint32_t incl = warp_incl_scan(x);
    if (nw == 1u) {
        *total = __shfl_sync(0xffffffffu, incl, 31);
        g.sync();
        return incl - x;
    }
    g.sync();
    if (lane == 31u || g.tid() == g.count() - 1) sh.u[warp] = incl;
    g.sync();
    if (warp == 0) {
        uint32_t y = lane < nw ? sh.u[lane] : 0u;
        uint32_t s = warp_incl_scan(y);
        if (lane < nw) sh.u[lane] = s - y;
        if (lane == nw - 1) sh.u[32] = s;
    }
    g.sync();
    *total = sh.u[32];
    return sh.u[warp] + incl - x;
}
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t x, uint32_t* total, BlockScratch& sh) {
    return shape_excl_scan(x, total, sh, BlockShape{});
}

// Exclusive scan of `count` values in place over the shape (values in memory visible to the whole shape).
template <class Shape> __device__ __forceinline__ void shape_scan_inplace(uint32_t* values, uint32_t count, BlockScratch& sh, const Shape& g) {
    const uint32_t T = g.count(), r = g.tid();
    uint32_t per = (count + T - 1) / T;
    uint32_t first = min(r * per, count), last = min(first + per, count);
    uint32_t local = 0;
    if (T == 32u) __syncwarp();
    for (uint32_t i = first; i < last; ++i) local += values[i];
    uint32_t total;
    uint32_t running = shape_excl_scan(local, &total, sh, g);
    for (uint32_t i = first; i < last; ++i) { uint32_t own = values[i]; values[i] = running; running += own; }
    g.sync();
}

// ----------------------------------------------------------------------------------------------------------------
// CTA team: one thread block owns the world.
// ----------------------------------------------------------------------------------------------------------------
struct CtaTeam {
    BlockScratch* sh;
    __device__ uint32_t rank() const { return threadIdx.x; }
    __device__ uint32_t size() const { return blockDim.x; }
    __device__ bool leader() const { return threadIdx.x == 0; }
    __device__ bool sync() const { __syncthreads(); return true; }
    // the thread that writes the team's shared-memory records, and the barrier after it
    __device__ bool shared_leader() const { return threadIdx.x == 0; }
    __device__ void shared_sync() const { __syncthreads(); }
    __device__ bool ok() const { return true; }
    template <bool kMax> __device__ ValOwner pick(ValOwner x) const { return block_pick<kMax>(x, *sh); }
    template <bool kMaxA, bool kMaxB> __device__ void pick2(ValOwner& a, ValOwner& b) const {
        block_pick2<kMaxA, kMaxB>(a, b, *sh);
    }
    __device__ uint32_t sum(uint32_t x) const { return block_sum(x, *sh); }
    __device__ uint32_t umax(uint32_t x) const { return block_max(x, *sh); }
    __device__ float fmax(float x) const { return block_fmax(x, *sh); }
    template <uint32_t kMaxMask> __device__ void reduce4(uint32_t (&v)[4]) const { block_reduce4<kMaxMask>(v, *sh); }
    // Exclusive scan of `count` values in place (values live in memory visible to the whole team).
    __device__ void scan_inplace(uint32_t* values, uint32_t count) const {
        shape_scan_inplace(values, count, *sh, BlockShape{});
    }
};

// ----------------------------------------------------------------------------------------------------------------
// Group team: a group of consecutive warps of a block owns a world; the block's groups step different worlds at the
// same time, each synchronised by its own named barrier (bar.sync id, width), so a block keeps several small and
// medium worlds in flight instead of one. A one-warp group synchronises with __syncwarp and reduces with shuffles.
// ----------------------------------------------------------------------------------------------------------------
struct GroupTeam {
    BlockScratch* sh;  // the group's own scratch
    GroupShape g;
    __device__ uint32_t rank() const { return g.tid(); }
    __device__ uint32_t size() const { return g.width; }
    __device__ bool leader() const { return g.tid() == 0u; }
    __device__ bool sync() const { g.sync(); return true; }
    __device__ bool shared_leader() const { return g.tid() == 0u; }
    __device__ void shared_sync() const { g.sync(); }
    __device__ bool ok() const { return true; }
    template <bool kMax> __device__ ValOwner pick(ValOwner x) const { return shape_pick<kMax>(x, *sh, g); }
    template <bool kMaxA, bool kMaxB> __device__ void pick2(ValOwner& a, ValOwner& b) const {
        shape_pick2<kMaxA, kMaxB>(a, b, *sh, g);
    }
    __device__ uint32_t sum(uint32_t x) const { return shape_reduce_u(x, false, *sh, g); }
    __device__ uint32_t umax(uint32_t x) const { return shape_reduce_u(x, true, *sh, g); }
    __device__ float fmax(float x) const { return shape_fmax(x, *sh, g); }
    template <uint32_t kMaxMask> __device__ void reduce4(uint32_t (&v)[4]) const { shape_reduce4<kMaxMask>(v, *sh, g); }
    __device__ void scan_inplace(uint32_t* values, uint32_t count) const { shape_scan_inplace(values, count, *sh, g); }
};

// GPU-scope memory operations of the grid barrier.
__device__ __forceinline__ unsigned int ld_relaxed(const unsigned int* p) {
    unsigned int v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned int atom_add_release(unsigned int* p, unsigned int v) {
    unsigned int old;
    asm volatile("atom.add.release.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}
__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

// ----------------------------------------------------------------------------------------------------------------
// Grid team: every block of a cooperative launch works on one world. Partials go through global memory with
// alternating parity so a reduction never overwrites partials another block may still read; each parity has four
// regions of gridDim.x entries (pv: 4 x 2 x grid floats, po: 4 x 2 x grid words), so up to four values reduce
// behind one grid barrier.
// ----------------------------------------------------------------------------------------------------------------
struct GridTeam {
    BlockScratch* sh;
    unsigned int* bar;       // [0] arrivals since the launch (zeroed before every launch)
    uint32_t* err;
    float* pv;               // 2 parities x 4 regions x gridDim.x partial values
    uint32_t* po;            // 2 parities x 4 regions x gridDim.x partial owners / counts
    uint32_t* parity;        // per-thread copy lives in registers; this is unused storage
    mutable uint32_t par;
    mutable bool failed;

    __device__ uint32_t rank() const { return blockIdx.x * blockDim.x + threadIdx.x; }
    __device__ uint32_t size() const { return gridDim.x * blockDim.x; }
    __device__ bool leader() const { return blockIdx.x == 0 && threadIdx.x == 0; }
    // every block keeps its own copy of the team's shared-memory records
    __device__ bool shared_leader() const { return threadIdx.x == 0; }
    __device__ void shared_sync() const { __syncthreads(); }
    __device__ bool ok() const { return !failed; }

    // Bounded grid barrier on a counter that only grows within a launch: the barrier a block enters with the counter
    // at `old` ends when the counter reaches the next multiple of the grid size. Arrival is a release add (the block's
    // writes, ordered before it by the block barrier, are released); the waiters poll relaxed and then acquire with one
    // fence. Returns false when any block gave up waiting (the error word is polled every 64 spins).
    __device__ bool sync() const {
        __syncthreads();
        if (threadIdx.x == 0) {
            const unsigned int old = atom_add_release(bar, 1u);
            const unsigned int target = (old / gridDim.x + 1u) * gridDim.x;
            unsigned long long spins = 0;
            while ((int)(ld_relaxed(bar) - target) < 0) {
                if ((++spins & 63u) == 0u && ld_relaxed(err) != 0u) break;
                if (spins > kBarrierSpinLimit) { atomicOr(err, 1u); break; }
                __nanosleep(32);
            }
            fence_acq_rel_gpu();
            sh->bcastU[7] = ld_relaxed(err);
        }
        __syncthreads();
        failed = sh->bcastU[7] != 0u;
        return !failed;
    }

    template <bool kMax> __device__ ValOwner pick(ValOwner x) const {
        x = block_pick<kMax>(x, *sh);
        uint32_t base = par * 4u * gridDim.x;
        if (threadIdx.x == 0) { pv[base + blockIdx.x] = x.v; po[base + blockIdx.x] = x.o; }
        par ^= 1u;
        sync();
        if (threadIdx.x < 32) {
            ValOwner y{kMax ? -__int_as_float(0x7f800000) : __int_as_float(0x7f800000), 0xffffffffu};
            for (uint32_t b = threadIdx.x; b < gridDim.x; b += 32) {
                ValOwner z{__ldcg(pv + base + b), __ldcg(po + base + b)};
                y = kMax ? pick_max(y, z) : pick_min(y, z);
            }
            y = warp_pick<kMax>(y);
            if (threadIdx.x == 0) { sh->bcastF[0] = y.v; sh->bcastU[0] = y.o; }
        }
        __syncthreads();
        return ValOwner{sh->bcastF[0], sh->bcastU[0]};
    }
    template <bool kMaxA, bool kMaxB> __device__ void pick2(ValOwner& a, ValOwner& b) const {
        block_pick2<kMaxA, kMaxB>(a, b, *sh);
        const uint32_t base = par * 4u * gridDim.x, G = gridDim.x;
        if (threadIdx.x == 0) {
            pv[base + blockIdx.x] = a.v; po[base + blockIdx.x] = a.o;
            pv[base + G + blockIdx.x] = b.v; po[base + G + blockIdx.x] = b.o;
        }
        par ^= 1u;
        sync();
        if (threadIdx.x < 32) {
            const float inf = __int_as_float(0x7f800000);
            ValOwner x{kMaxA ? -inf : inf, 0xffffffffu}, y{kMaxB ? -inf : inf, 0xffffffffu};
            for (uint32_t blk = threadIdx.x; blk < G; blk += 32) {
                ValOwner z{__ldcg(pv + base + blk), __ldcg(po + base + blk)};
                ValOwner w{__ldcg(pv + base + G + blk), __ldcg(po + base + G + blk)};
                x = kMaxA ? pick_max(x, z) : pick_min(x, z);
                y = kMaxB ? pick_max(y, w) : pick_min(y, w);
            }
            x = warp_pick<kMaxA>(x);
            y = warp_pick<kMaxB>(y);
            if (threadIdx.x == 0) { sh->bcastF[0] = x.v; sh->bcastU[0] = x.o; sh->bcastF[2] = y.v; sh->bcastU[3] = y.o; }
        }
        __syncthreads();
        a = ValOwner{sh->bcastF[0], sh->bcastU[0]};
        b = ValOwner{sh->bcastF[2], sh->bcastU[3]};
    }
    __device__ uint32_t reduce_u(uint32_t x, bool isMax) const {
        x = isMax ? block_max(x, *sh) : block_sum(x, *sh);
        uint32_t base = par * 4u * gridDim.x;
        if (threadIdx.x == 0) po[base + blockIdx.x] = x;
        par ^= 1u;
        sync();
        if (threadIdx.x < 32) {
            uint32_t y = 0;
            for (uint32_t b = threadIdx.x; b < gridDim.x; b += 32) {
                uint32_t z = __ldcg(po + base + b);
                y = isMax ? max(y, z) : y + z;
            }
            y = isMax ? warp_max(y) : warp_sum(y);
            if (threadIdx.x == 0) sh->bcastU[1] = y;
        }
        __syncthreads();
        return sh->bcastU[1];
    }
    __device__ uint32_t sum(uint32_t x) const { return reduce_u(x, false); }
    __device__ uint32_t umax(uint32_t x) const { return reduce_u(x, true); }
    // Four sums / maxima behind one grid barrier (kMaxMask bit c set: maximum for component c).
    template <uint32_t kMaxMask> __device__ void reduce4(uint32_t (&v)[4]) const {
        block_reduce4<kMaxMask>(v, *sh);
        const uint32_t base = par * 4u * gridDim.x, G = gridDim.x;
        if (threadIdx.x == 0) {
#pragma unroll
            for (int c = 0; c < 4; ++c) po[base + c * G + blockIdx.x] = v[c];
        }
        par ^= 1u;
        sync();
        if (threadIdx.x < 32) {
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const bool isMax = ((kMaxMask >> c) & 1u) != 0u;
                uint32_t y = 0;
                for (uint32_t blk = threadIdx.x; blk < G; blk += 32) {
                    uint32_t z = __ldcg(po + base + c * G + blk);
                    y = isMax ? max(y, z) : y + z;
                }
                y = isMax ? warp_max(y) : warp_sum(y);
                if (threadIdx.x == 0) sh->u4[c][32] = y;
            }
        }
        __syncthreads();
#pragma unroll
        for (int c = 0; c < 4; ++c) v[c] = sh->u4[c][32];
    }
    __device__ float fmax(float x) const {
        x = block_fmax(x, *sh);
        uint32_t base = par * 4u * gridDim.x;
        if (threadIdx.x == 0) pv[base + blockIdx.x] = x;
        par ^= 1u;
        sync();
        if (threadIdx.x < 32) {
            float y = -__int_as_float(0x7f800000);
            for (uint32_t b = threadIdx.x; b < gridDim.x; b += 32) y = fmaxf(y, __ldcg(pv + base + b));
            y = warp_fmax(y);
            if (threadIdx.x == 0) sh->bcastF[1] = y;
        }
        __syncthreads();
        return sh->bcastF[1];
    }
    // Exclusive scan of `count` values in global memory: each block scans a contiguous chunk.
    __device__ void scan_inplace(uint32_t* values, uint32_t count) const {
        uint32_t per = (count + gridDim.x - 1) / gridDim.x;
        uint32_t first = min(blockIdx.x * per, count), last = min(first + per, count);
        uint32_t tper = (last - first + blockDim.x - 1) / blockDim.x;
        uint32_t tf = min(first + threadIdx.x * tper, last), tl = min(tf + tper, last);
        uint32_t local = 0;
        for (uint32_t i = tf; i < tl; ++i) local += __ldcg(values + i);
        uint32_t total;
        uint32_t running = block_excl_scan(local, &total, *sh);
        uint32_t base = par * 4u * gridDim.x;
        if (threadIdx.x == 0) po[base + blockIdx.x] = total;
        par ^= 1u;
        sync();
        if (threadIdx.x < 32) {  // the totals of the blocks before this one, summed by one warp
            uint32_t off = 0;
            for (uint32_t b = threadIdx.x; b < blockIdx.x; b += 32) off += __ldcg(po + base + b);
            off = warp_sum(off);
            if (threadIdx.x == 0) sh->bcastU[2] = off;
        }
        __syncthreads();
        running += sh->bcastU[2];
        for (uint32_t i = tf; i < tl; ++i) { uint32_t own = __ldcg(values + i); values[i] = running; running += own; }
        sync();
    }
};

}  // namespace bp
