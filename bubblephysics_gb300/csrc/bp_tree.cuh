// bp_tree.cuh - LBVH over the rigid leaves of one world (its one-sided segments and its bodies), rebuilt by the
// world's team at the start of every step, after the kinematic advance.
//
// The reference finds rigid candidates by brute force: every bubble tests every segment (nativeFinishBubbleRow,
// NativeGeometryKernels:279-290) and every body tests every bubble (nativeEmitBodyCandidates,
// NativeGeometryKernels:350-415). This tree replaces those O(N * S) and O(N * B) loops with O(N log L) traversals and
// keeps the candidate SETS exact: a traversal only prunes a node whose box fails a test that every accepted leaf
// would pass, and the leaf itself still runs the reference predicate.
//
// Build (all team-wide, deterministic):
//   1. centres of the leaf boxes, their bounding box (orderable-bit max reductions), scale = 32767 / extent;
//   2. key = (morton30(q(cx), q(cy)) << 32) | leaf, q = trunc(clamp((c - lo) * scale, 0, 32767)), x in the even bits;
//   3. stable LSD radix sort of the keys on the Morton bits (4-bit digits, per-worker counters, team scans);
//   4. Karras (2012) hierarchy over the sorted keys: internal node i covers a key range, split at the highest
//      differing bit; leaf children carry their leaf index;
//   5. bottom-up refit: each leaf walks to the root, the second child to arrive at a node writes the union upward.
// Child boxes are stored in the parent; a body leaf's box is its swept box widened by its hull radius beyond the
// bounding radius, so the inside-body test of the contact assertion can use the same tree.
//
// Conservative node tests need no slack: a node box is the exact min / max of its leaves' boxes and correctly
// rounded float arithmetic is monotone, so fl(node.lo - r) <= fl(leaf.lo - r) and the node test holds whenever the
// leaf test does.
#pragma once

#include "bp_device.cuh"
#include "bp_team.cuh"

namespace bp {

constexpr uint32_t kTreeStack = 64;      // tree depth <= 64: every level adds a bit of common key prefix
constexpr uint32_t kTreeNoParent = 0xffffffffu;

// Bit order of finite floats as unsigned integers (max of the encoding = max of the floats).
__device__ __forceinline__ uint32_t float_order(float f) {
    uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float float_unorder(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// Bits 0..14 of v moved to the even bit positions 0..28.
__device__ __forceinline__ uint32_t spread_bits15(uint32_t v) {
    v &= 0x7fffu;
    v = (v | (v << 8)) & 0x00ff00ffu;
    v = (v | (v << 4)) & 0x0f0f0f0fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}

__device__ __forceinline__ uint32_t quantize15(float c, float lo, float scale) {
    return (uint32_t)fminf(fmaxf((c - lo) * scale, 0.0f), 32767.0f);
}

// Box of leaf `leaf` (segments first, then bodies): the segment's [min(a,b), max(a,b)] or the body's swept box.
__device__ __forceinline__ float4 leaf_box(const DState& S, const DWorld& W, uint32_t leaf) {
    return leaf < W.s ? S.segBox[W.soff + leaf].box : S.bodyBox[W.bodyOff + leaf - W.s].box;
}
// The same box with a body widened by its hull radius beyond the bounding radius (the inside-body prefilter box).
__device__ __forceinline__ float4 leaf_box_wide(const DState& S, const DWorld& W, uint32_t leaf) {
    if (leaf < W.s) return S.segBox[W.soff + leaf].box;
    const RigidBox rb = S.bodyBox[W.bodyOff + leaf - W.s];
    const float e = __uint_as_float(rb.pad);
    return make_float4(rb.box.x - e, rb.box.y - e, rb.box.z + e, rb.box.w + e);
}

__device__ __forceinline__ float4 box_union(float4 a, float4 b) {
    return make_float4(fminf(a.x, b.x), fminf(a.y, b.y), fmaxf(a.z, b.z), fmaxf(a.w, b.w));
}

// Stable LSD radix sort of `count` keys on bits 32..63, 4 bits per pass (8 passes: the result ends in `keys`).
// Worker w owns the contiguous chunk [w * chunk, (w + 1) * chunk); counters are digit-major so one exclusive team
// scan gives every worker the first slot of each digit, and a worker scattering its chunk in order keeps the sort
// stable.
template <class Team>
__device__ void tree_sort(unsigned long long* keys, unsigned long long* alt, uint32_t* counts, uint32_t count,
                          const Team& team) {
    const uint32_t T = team.size(), r = team.rank();
    const uint32_t chunk = (count + T - 1u) / T;
    const uint32_t workers = (count + chunk - 1u) / chunk;
    const uint32_t first = min(r * chunk, count), last = min(first + chunk, count);
    for (uint32_t pass = 0; pass < 8u; ++pass) {
        const uint32_t shift = 32u + 4u * pass;
        if (r < workers) {
            uint32_t c[16];
#pragma unroll
            for (uint32_t d = 0; d < 16u; ++d) c[d] = 0u;
            for (uint32_t e = first; e < last; ++e) {
                const uint32_t digit = (uint32_t)(keys[e] >> shift) & 15u;
#pragma unroll
                for (uint32_t d = 0; d < 16u; ++d) c[d] += digit == d ? 1u : 0u;
            }
#pragma unroll
            for (uint32_t d = 0; d < 16u; ++d) counts[d * workers + r] = c[d];
        }
        team.sync();
        team.scan_inplace(counts, 16u * workers);
        if (r < workers) {
            uint32_t o[16];
#pragma unroll
            for (uint32_t d = 0; d < 16u; ++d) o[d] = counts[d * workers + r];
            for (uint32_t e = first; e < last; ++e) {
                const unsigned long long key = keys[e];
                const uint32_t digit = (uint32_t)(key >> shift) & 15u;
                uint32_t slot = 0;
#pragma unroll
                for (uint32_t d = 0; d < 16u; ++d)
                    if (digit == d) slot = o[d]++;
                alt[slot] = key;
            }
        }
        team.sync();
        unsigned long long* t = keys;
        keys = alt;
        alt = t;
    }
}

// Stable LSD radix sort of `count` keys on bits 32..63 by one block of 16 warps (8-bit digits, 4 passes: the result
// ends in `keys`). Warp w owns a contiguous chunk of the keys and walks it 32 keys at a time, in order. Each pass
// builds the warp's digit histogram (shared memory), runs one block scan in digit-major, warp-minor order, and
// scatters: lanes with the same digit take consecutive slots in lane order (__match_any_sync), so the sort is stable.
// The histograms live in the launch's dynamic shared memory (kRadixHistBytes), which only launches that build a tree
// ask for: static shared memory would take L1 from every launch of the kernel.
extern __shared__ __align__(16) uint32_t g_radix_hist[];
__device__ inline void block_radix_sort(unsigned long long* keys, unsigned long long* alt, uint32_t count,
                                        const CtaTeam& block) {
    uint32_t* hist = g_radix_hist;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t per = (count + kRadixWarps - 1u) / kRadixWarps;
    const uint32_t first = min(warp * per, count), last = min(first + per, count);
    const uint32_t below = (1u << lane) - 1u;
    for (uint32_t pass = 0; pass < 4u; ++pass) {
        const uint32_t shift = 32u + 8u * pass;
        for (uint32_t d = lane; d < kRadixDigits; d += 32u) hist[d * kRadixWarps + warp] = 0u;
        __syncwarp();
        // each loop loads the next batch's key while it processes the current one
        unsigned long long ahead = first + lane < last ? keys[first + lane] : 0ull;
        for (uint32_t base = first; base < last; base += 32u) {  // uniform over the warp
            const uint32_t e = base + lane;
            const bool in = e < last;
            const unsigned long long key = ahead;
            ahead = e + 32u < last ? keys[e + 32u] : 0ull;
            const uint32_t digit = (uint32_t)(key >> shift) & 0xffu;
            const uint32_t peers = __match_any_sync(0xffffffffu, in ? digit : kRadixDigits + lane);
            if (in && (peers & below) == 0u) hist[digit * kRadixWarps + warp] += __popc(peers);
            __syncwarp();
        }
        __syncthreads();
        block.scan_inplace(hist, kRadixDigits * kRadixWarps);  // ends with a block barrier
        ahead = first + lane < last ? keys[first + lane] : 0ull;
        for (uint32_t base = first; base < last; base += 32u) {
            const uint32_t e = base + lane;
            const bool in = e < last;
            const unsigned long long key = ahead;
            ahead = e + 32u < last ? keys[e + 32u] : 0ull;
            const uint32_t digit = (uint32_t)(key >> shift) & 0xffu;
            const uint32_t peers = __match_any_sync(0xffffffffu, in ? digit : kRadixDigits + lane);
            if (in) alt[hist[digit * kRadixWarps + warp] + __popc(peers & below)] = key;
            __syncwarp();
            if (in && (peers & below) == 0u) hist[digit * kRadixWarps + warp] += __popc(peers);
            __syncwarp();
        }
        __syncthreads();
        unsigned long long* t = keys;
        keys = alt;
        alt = t;
    }
}

// Sort of a world's leaf keys by its team. The whole-GPU team sorts inside its first block (block barriers instead of
// the grid barriers of team-wide passes: a few thousand keys sort faster than the grid can synchronise), with the
// 8-bit sort above when the block has 16 warps and the launch gave it the histogram memory, and the other blocks wait
// at one grid barrier.
template <class Team>
__device__ __forceinline__ void sort_leaf_keys(unsigned long long* keys, unsigned long long* alt, uint32_t* counts,
                                               uint32_t count, const Team& team) {
    tree_sort(keys, alt, counts, count, team);
}
__device__ __forceinline__ void sort_leaf_keys(unsigned long long* keys, unsigned long long* alt, uint32_t* counts,
                                               uint32_t count, const GridTeam& team) {
    if (blockIdx.x == 0) {
        CtaTeam block{team.sh};
        uint32_t dynamic;
        asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dynamic));
        if (blockDim.x == 32u * kRadixWarps && dynamic >= kRadixHistBytes) block_radix_sort(keys, alt, count, block);
        else tree_sort(keys, alt, counts, count, block);
    }
    team.sync();
}

// Length of the common prefix of sorted keys i and j (-1 outside [0, count)); keys are unique (leaf index bits).
__device__ __forceinline__ int tree_delta(const unsigned long long* keys, int count, int i, int j) {
    if (j < 0 || j >= count) return -1;
    return __clzll(keys[i] ^ keys[j]);
}

// Per-part cycle counters of the tree build for profiling builds (-DBP_PHASE_TIMING; phase ids 19-23).
#ifdef BP_PHASE_TIMING
#define BP_TREE_MARK(id)                                                                                 \
    do {                                                                                                 \
        if (team.leader() && S.phaseCycles) {                                                            \
            const long long now_ = clock64();                                                            \
            S.phaseCycles[(uint64_t)wi * kPhaseCount + (id)] += (unsigned long long)(now_ - treeMark);   \
            treeMark = now_;                                                                             \
        }                                                                                                \
    } while (0)
#else
#define BP_TREE_MARK(id) do { } while (0)
#endif

// Builds the world's tree; false (uniform over the team) when the world has no leaves or a leaf box is not finite,
// in which case the step uses the brute-force loops.
template <class Team>
__device__ bool build_rigid_tree(const DState& S, const DWorld& W, uint32_t wi, const Team& team) {
    const uint32_t L = W.s + W.nb, base = W.treeOff, T = team.size(), r = team.rank();
    team.sync();  // the boxes of this step are written
#ifdef BP_PHASE_TIMING
    long long treeMark = clock64();
#endif
    uint32_t v[4] = {0u, 0u, 0u, 0u};
    for (uint32_t p = r; p < L; p += T) {
        const float4 b = leaf_box(S, W, p);
        if (!isfinite(b.x) || !isfinite(b.y) || !isfinite(b.z) || !isfinite(b.w)) { v[0] = 0xffffffffu; continue; }
        const float cx = (b.x + b.z) * 0.5f, cy = (b.y + b.w) * 0.5f;
        v[0] = max(v[0], float_order(cx));
        v[1] = max(v[1], float_order(cy));
        v[2] = max(v[2], ~float_order(cx));
        v[3] = max(v[3], ~float_order(cy));
    }
    team.template reduce4<0xfu>(v);
    BP_TREE_MARK(19);
    const bool ok = L > 0u && v[0] != 0xffffffffu;
    if (team.leader()) S.tValid[wi] = ok ? 1u : 0u;
    if (!ok) return false;
    const float lox = float_unorder(~v[2]), loy = float_unorder(~v[3]);
    const float ex = float_unorder(v[0]) - lox, ey = float_unorder(v[1]) - loy;
    const float sx = ex > 0.0f ? 32767.0f / ex : 0.0f, sy = ey > 0.0f ? 32767.0f / ey : 0.0f;
    unsigned long long* keys = S.tKeys + base;
    for (uint32_t p = r; p < L; p += T) {
        const float4 b = leaf_box(S, W, p);
        const float cx = (b.x + b.z) * 0.5f, cy = (b.y + b.w) * 0.5f;
        const uint32_t code = spread_bits15(quantize15(cx, lox, sx)) | (spread_bits15(quantize15(cy, loy, sy)) << 1);
        keys[p] = ((unsigned long long)code << 32) | p;
    }
    team.sync();
    BP_TREE_MARK(20);
    sort_leaf_keys(keys, S.tKeysAlt + base, S.tCounts + 16ull * base, L, team);
    BP_TREE_MARK(21);
    if (L == 1u) return true;
    // hierarchy (Karras 2012, "Maximizing parallelism in the construction of BVHs, octrees and k-d trees")
    TreeNode* nodes = S.tNodes + base;
    const int count = (int)L;
    for (uint32_t node = r; node + 1u < L; node += T) {
        const int i = (int)node;
        const int d = tree_delta(keys, count, i, i + 1) > tree_delta(keys, count, i, i - 1) ? 1 : -1;
        const int dmin = tree_delta(keys, count, i, i - d);
        int lmax = 2;
        while (tree_delta(keys, count, i, i + lmax * d) > dmin) lmax <<= 1;
        int l = 0;
        for (int t = lmax >> 1; t >= 1; t >>= 1)
            if (tree_delta(keys, count, i, i + (l + t) * d) > dmin) l += t;
        const int j = i + l * d;
        const int dnode = tree_delta(keys, count, i, j);
        int s = 0, t = l;
        do {
            t = (t + 1) >> 1;
            if (tree_delta(keys, count, i, i + (s + t) * d) > dnode) s += t;
        } while (t > 1);
        const int split = i + s * d + min(d, 0);
        const int lo = min(i, j), hi = max(i, j);
        uint32_t child[2];
        if (lo == split) {
            child[0] = kTreeLeaf | (uint32_t)(keys[split] & 0xffffffffull);
            S.tLeafParent[base + split] = node << 1;
        } else {
            child[0] = (uint32_t)split;
            nodes[split].parent = node << 1;
        }
        if (hi == split + 1) {
            child[1] = kTreeLeaf | (uint32_t)(keys[split + 1] & 0xffffffffull);
            S.tLeafParent[base + split + 1] = (node << 1) | 1u;
        } else {
            child[1] = (uint32_t)(split + 1);
            nodes[split + 1].parent = (node << 1) | 1u;
        }
        nodes[node].child[0] = child[0];
        nodes[node].child[1] = child[1];
        if (node == 0u) nodes[0].parent = kTreeNoParent;
        S.tVisit[base + node] = 0u;
    }
    team.sync();
    BP_TREE_MARK(22);
    // bottom-up refit: the second child to reach a node carries the union to the parent
    for (uint32_t q = r; q < L; q += T) {
        float4 box = leaf_box_wide(S, W, (uint32_t)(keys[q] & 0xffffffffull));
        uint32_t up = S.tLeafParent[base + q];
        for (uint32_t depth = 0; depth < L; ++depth) {  // a path to the root has fewer than L nodes
            const uint32_t node = up >> 1, side = up & 1u;
            nodes[node].box[side] = box;
            // one acquire-release add: it releases this child's box, and the second arriver acquires the sibling's
            unsigned int arrived;
            asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], 1;" : "=r"(arrived) : "l"(S.tVisit + base + node) : "memory");
            if (arrived == 0u) break;
            box = box_union(box, __ldcg(&nodes[node].box[side ^ 1u]));
            up = __ldcg(&nodes[node].parent);
            if (up == kTreeNoParent) break;
        }
    }
    team.sync();
    BP_TREE_MARK(23);
    return true;
}

// Visits every leaf whose box passes `test` along the whole path from the root (leaf(index), index in segments-then-
// bodies numbering). `test` must hold for a box whenever it holds for a box inside it (the leaf functor re-checks).
template <class Test, class Leaf>
__device__ __forceinline__ void tree_query(const DState& S, const DWorld& W, Test&& test, Leaf&& leaf) {
    const uint32_t L = W.s + W.nb;
    if (L == 0u) return;
    if (L == 1u) { leaf(0u); return; }
    const TreeNode* nodes = S.tNodes + W.treeOff;
    uint32_t stack[kTreeStack];
    uint32_t sp = 0, node = 0;
    for (uint32_t visits = 0; visits < L; ++visits) {  // each of the L - 1 internal nodes is entered at most once
        const float4 b0 = nodes[node].box[0], b1 = nodes[node].box[1];
        const uint32_t c0 = nodes[node].child[0], c1 = nodes[node].child[1];
        bool h0 = test(b0), h1 = test(b1);
        if (h0 && (c0 & kTreeLeaf)) { leaf(c0 & ~kTreeLeaf); h0 = false; }
        if (h1 && (c1 & kTreeLeaf)) { leaf(c1 & ~kTreeLeaf); h1 = false; }
        if (h0 && h1) {
            if (sp < kTreeStack) stack[sp++] = c1;
            node = c0;
        } else if (h0) {
            node = c0;
        } else if (h1) {
            node = c1;
        } else {
            if (sp == 0u) break;
            node = stack[--sp];
        }
    }
}

}  // namespace bp
