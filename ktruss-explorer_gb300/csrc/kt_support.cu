// Edge support (triangle count per edge) on the degree-oriented CSR.
//
// Replaces count_triangles_kernel of the reference (kernel_ddc.cu:11-54): there one thread
// merges the two out-lists of its edge and issues three atomics per triangle.  Two counts here,
// chosen by the schedule's support_group:
//
// support_group 4, 8, 16, 32 - edge-centric: each oriented edge (u,v), u < v in rank order, is
// handled by a group of G lanes.  Only the part of N+(u) above v can hold a common neighbour, and
// it starts right after the edge itself in u's row, so the intersection is
// S = o_col[j+1 .. o_ptr[u+1])  with  L = N+(v).  Lanes stride over the shorter list and
// binary-search the longer one; for a triangle (u,v,w) found at positions x (in u's row) and y
// (in v's row), the edges (u,w) = x and (v,w) = y gain one support each, and (u,v) gains the
// group's match count once.  Bound: uncoalesced probes (about nine per search) through L1/L2.
//
// support_group 0 - vertex-centric with a shared-memory hash: every triangle u < v < w is found
// from its middle vertex v.  The row N+(v) (at most a few thousand entries under degree
// orientation) is hashed once into shared memory, key w -> position in the row; then the tails
// S_uv = o_col[j+1 .. o_ptr[u+1]) of v's in-edges j = (u,v) (the lower part of v's symmetric row)
// are streamed, coalesced, and each entry is one hash probe instead of a binary search.  A hit
// at tail position x credits edge (u,w) = x with a global atomic, edge (v,w) with a shared-memory
// counter at its row position (added to the support array once per row), and edge (u,v) with a
// shared-memory counter per in-edge (added once per in-edge).  Lanes of a warp share the tails of
// 32 in-edges at a time through a warp scan of the tail lengths, so short tails waste no lanes.
// Scheduling by degree: a plan kernel sends vertices with short rows and few in-edges to single
// warps (a warp-private table), all others as ranges of at most kHeavyIn in-edges to whole blocks
// (a block table); rows longer than the block table are searched in HBM instead of hashed.

#include <algorithm>

#include "kt_device.cuh"
#include "kt_engine.h"

namespace kt {

namespace {

constexpr int kThreads = 256;

template <int G>
__device__ __forceinline__ void support_body(const uint32_t* __restrict__ o_ptr, const uint32_t* __restrict__ o_col,
                                             const uint32_t* __restrict__ e_src, uint32_t m,
                                             uint32_t* __restrict__ sup) {
    const uint32_t lane = lane_id();
    const uint32_t glane = lane & (G - 1);
    const uint32_t gmask = (G == 32) ? kFullMask : (((1u << G) - 1) << (lane & ~(uint32_t)(G - 1)));
    const uint64_t gid = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
    const uint64_t ngroups = ((uint64_t)gridDim.x * blockDim.x) / G;
    for (uint64_t j64 = gid; j64 < m; j64 += ngroups) {
        const uint32_t j = (uint32_t)j64;
        const uint32_t u = e_src[j], v = o_col[j];
        const uint32_t a0 = j + 1, a1 = o_ptr[u + 1];
        const uint32_t b0 = o_ptr[v], b1 = o_ptr[v + 1];
        const uint32_t na = a1 - a0, nb = b1 - b0;
        uint32_t cnt = 0;
        if (na && nb) {
            // iterate the shorter list, search the longer
            const bool iter_a = na <= nb;
            const uint32_t i0 = iter_a ? a0 : b0, ni = iter_a ? na : nb;
            const uint32_t s0 = iter_a ? b0 : a0, ns = iter_a ? nb : na;
            for (uint32_t t = glane; t < ni; t += G) {
                const uint32_t x = i0 + t;
                const uint32_t w = o_col[x];
                const uint32_t idx = lower_bound_u32(o_col + s0, ns, w);
                if (idx < ns && o_col[s0 + idx] == w) {
                    ++cnt;
                    atomicAdd(&sup[x], 1u);
                    atomicAdd(&sup[s0 + idx], 1u);
                }
            }
        }
        __syncwarp(gmask);
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) cnt += __shfl_xor_sync(gmask, cnt, o);
        if (glane == 0 && cnt) atomicAdd(&sup[j], cnt);
    }
}

template <int G>
__global__ void __launch_bounds__(kThreads) k_support(const uint32_t* __restrict__ o_ptr,
                                                      const uint32_t* __restrict__ o_col,
                                                      const uint32_t* __restrict__ e_src, uint32_t m,
                                                      uint32_t* __restrict__ sup) {
    support_body<G>(o_ptr, o_col, e_src, m, sup);
}

// The same count with the lane group read from the control block, where the learned selector's
// inference kernel wrote its choice: the schedule is chosen on the device, with no host read.
__global__ void __launch_bounds__(kThreads) k_support_chosen(const uint32_t* __restrict__ o_ptr,
                                                             const uint32_t* __restrict__ o_col,
                                                             const uint32_t* __restrict__ e_src, uint32_t m,
                                                             const uint32_t* __restrict__ sched,
                                                             uint32_t* __restrict__ sup) {
    switch (sched[0]) {
        case 4: support_body<4>(o_ptr, o_col, e_src, m, sup); break;
        case 16: support_body<16>(o_ptr, o_col, e_src, m, sup); break;
        case 32: support_body<32>(o_ptr, o_col, e_src, m, sup); break;
        default: support_body<8>(o_ptr, o_col, e_src, m, sup); break;
    }
}

// ---- vertex-centric hashed count (support_group 0) --------------------------------------------

constexpr int kHashThreads = 512;                 // 16 warps
constexpr int kHashWarps = kHashThreads / 32;
constexpr uint32_t kWarpSlots = 256;              // warp table: rows of at most 128 entries
constexpr uint32_t kLightOut = kWarpSlots / 2;
constexpr uint32_t kLightIn = 256;                // ... and at most this many in-edges
constexpr uint32_t kBlockSlots = 4096;            // block table: rows of at most 2048 entries
constexpr uint32_t kBlockOut = kBlockSlots / 2;
constexpr uint32_t kHeavyIn = 1024;               // in-edges per block work item
constexpr uint32_t kEmpty = 0xffffffffu;
// control words of the plan (free during the support count)
constexpr uint32_t kHLight = 21, kHHeavy = 22, kHLightCur = 23, kHHeavyCur = 24;

struct HashSmem {
    uint32_t wkey[kHashWarps][kWarpSlots];
    uint16_t wval[kHashWarps][kWarpSlots];
    uint32_t wcnt[kHashWarps][kLightOut];     // per row position of the warp's vertex
    uint32_t jcnt[kHashWarps][32];            // per in-edge of the current batch
    uint32_t bkey[kBlockSlots];
    uint16_t bval[kBlockSlots];
    uint32_t bcnt[kBlockOut];
    uint32_t item;                            // the block's current heavy item
};

__device__ __forceinline__ uint32_t hash_slot(uint32_t w, uint32_t mask) { return (w * 0x9E3779B1u) >> 8 & mask; }

// Plan: every vertex with in-edges and an out-row becomes a light vertex (one warp) or a list of
// heavy items {v, first in-edge, end in-edge} (one block each).
__global__ void k_support_plan(const uint32_t* __restrict__ s_ptr, const uint32_t* __restrict__ s_split,
                               const uint32_t* __restrict__ o_ptr, uint32_t n, uint32_t* __restrict__ light,
                               uint4* __restrict__ heavy, uint32_t* __restrict__ ctrl) {
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t indeg = 0, outdeg = 0;
    if (v < n) {
        indeg = s_split[v] - s_ptr[v];
        outdeg = o_ptr[v + 1] - o_ptr[v];
    }
    const bool work = indeg && outdeg;
    const bool is_light = work && outdeg <= kLightOut && indeg <= kLightIn;
    const uint32_t lm = __ballot_sync(kFullMask, is_light);
    uint32_t lb = 0;
    if (lm && lane_id() == 0) lb = atomicAdd(ctrl + kHLight, __popc(lm));
    lb = __shfl_sync(kFullMask, lb, 0);
    if (is_light) light[lb + __popc(lm & lanemask_lt())] = v;
    const uint32_t items = work && !is_light ? (indeg + kHeavyIn - 1) / kHeavyIn : 0u;
    if (items) {
        const uint32_t h0 = atomicAdd(ctrl + kHHeavy, items);
        const uint32_t base = s_ptr[v];
        for (uint32_t i = 0; i < items; ++i) {
            const uint32_t a = base + i * kHeavyIn;
            heavy[h0 + i] = make_uint4(v, a, min(a + kHeavyIn, base + indeg), 0u);
        }
    }
}

// The tails of in-edges [a, b) (symmetric-row positions of v's lower neighbours), 32 in-edges at a
// time per warp, starting at `first` and striding by `step` batches of 32.  `lookup(w)` returns the
// row position of w in N+(v) or kEmpty; `credit_vw(pos)` records a triangle on edge (v,w).
template <class Lookup, class Credit>
__device__ __forceinline__ void stream_tails(const uint32_t* __restrict__ o_ptr, const uint32_t* __restrict__ o_col,
                                             const uint32_t* __restrict__ s_col,
                                             const uint32_t* __restrict__ s_eid, uint32_t* __restrict__ sup,
                                             uint32_t a, uint32_t b, uint32_t first, uint32_t step,
                                             uint32_t* jcnt, Lookup lookup, Credit credit_vw) {
    const uint32_t lane = lane_id();
    for (uint32_t base = a + first; base < b; base += step) {
        const uint32_t p = base + lane;
        uint32_t t0 = 0, len = 0, j = 0;
        if (p < b) {
            j = s_eid[p];
            const uint32_t u = s_col[p];
            t0 = j + 1;
            len = o_ptr[u + 1] - t0;
        }
        jcnt[lane] = 0;
        uint32_t incl = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(kFullMask, incl, o);
            if (lane >= (uint32_t)o) incl += t;
        }
        const uint32_t total = __shfl_sync(kFullMask, incl, 31);
        __syncwarp();
        for (uint32_t t = lane; t - lane < total; t += 32) {
            // in-edge of flattened item t: the number of inclusive prefixes <= t
            uint32_t i = 0;
#pragma unroll
            for (uint32_t s2 = 16; s2 > 0; s2 >>= 1) {
                const uint32_t pv = __shfl_sync(kFullMask, incl, i + s2 - 1);
                if (pv <= t) i += s2;
            }
            const uint32_t inc_i = __shfl_sync(kFullMask, incl, i & 31);
            const uint32_t len_i = __shfl_sync(kFullMask, len, i & 31);
            const uint32_t t0_i = __shfl_sync(kFullMask, t0, i & 31);
            if (t < total) {
                const uint32_t x = t0_i + (t - (inc_i - len_i));
                const uint32_t pos = lookup(__ldg(o_col + x));
                if (pos != kEmpty) {
                    atomicAdd(&sup[x], 1u);
                    credit_vw(pos);
                    atomicAdd(&jcnt[i], 1u);
                }
            }
        }
        __syncwarp();
        const uint32_t c = jcnt[lane];
        if (p < b && c) atomicAdd(&sup[j], c);
        __syncwarp();
    }
}

__global__ void __launch_bounds__(kHashThreads) k_support_hash(const uint32_t* __restrict__ o_ptr,
                                                               const uint32_t* __restrict__ o_col,
                                                               const uint32_t* __restrict__ o_fence,
                                                               const uint32_t* __restrict__ s_col,
                                                               const uint32_t* __restrict__ s_eid,
                                                               const uint32_t* __restrict__ s_ptr,
                                                               const uint32_t* __restrict__ s_split,
                                                               const uint32_t* __restrict__ light,
                                                               const uint4* __restrict__ heavy,
                                                               uint32_t* __restrict__ sup, uint32_t* __restrict__ ctrl) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    HashSmem& S = *reinterpret_cast<HashSmem*>(smem_raw);
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    const uint32_t n_heavy = ld_acquire(ctrl + kHHeavy), n_light = ld_acquire(ctrl + kHLight);

    // heavy items: one block per item, the block table holds N+(v)
    for (;;) {
        if (threadIdx.x == 0) S.item = atomicAdd(ctrl + kHHeavyCur, 1u);
        __syncthreads();
        const uint32_t it = S.item;
        if (it >= n_heavy) break;
        const uint4 d = heavy[it];
        const uint32_t v = d.x, r0 = o_ptr[v], outdeg = o_ptr[v + 1] - r0;
        const bool hashed = outdeg <= kBlockOut;
        uint32_t bits = 1;
        while ((1u << bits) < 2 * outdeg) ++bits;
        const uint32_t mask = (1u << bits) - 1;
        if (hashed) {
            for (uint32_t i = threadIdx.x; i <= mask; i += blockDim.x) S.bkey[i] = kEmpty;
            for (uint32_t i = threadIdx.x; i < outdeg; i += blockDim.x) S.bcnt[i] = 0;
            __syncthreads();
            for (uint32_t i = threadIdx.x; i < outdeg; i += blockDim.x) {
                const uint32_t w = o_col[r0 + i];
                uint32_t h = hash_slot(w, mask);
                while (atomicCAS(&S.bkey[h], kEmpty, w) != kEmpty) h = (h + 1) & mask;
                S.bval[h] = (uint16_t)i;
            }
            __syncthreads();
            stream_tails(o_ptr, o_col, s_col, s_eid, sup, d.y, d.z, 32 * warp, 32 * kHashWarps, S.jcnt[warp],
                         [&](uint32_t w) {
                             uint32_t h = hash_slot(w, mask);
                             for (;;) {
                                 const uint32_t k = S.bkey[h];
                                 if (k == w) return (uint32_t)S.bval[h];
                                 if (k == kEmpty) return kEmpty;
                                 h = (h + 1) & mask;
                             }
                         },
                         [&](uint32_t pos) { atomicAdd(&S.bcnt[pos], 1u); });
            __syncthreads();
            for (uint32_t i = threadIdx.x; i < outdeg; i += blockDim.x)
                if (S.bcnt[i]) atomicAdd(&sup[r0 + i], S.bcnt[i]);
        } else {
            // a row too long for the table: binary search in HBM (through its fences), credits direct
            stream_tails(o_ptr, o_col, s_col, s_eid, sup, d.y, d.z, 32 * warp, 32 * kHashWarps, S.jcnt[warp],
                         [&](uint32_t w) {
                             const uint32_t y = fenced_lower_bound(o_col, o_fence, r0, r0 + outdeg, w);
                             return y < r0 + outdeg && __ldg(o_col + y) == w ? y - r0 : kEmpty;
                         },
                         [&](uint32_t pos) { atomicAdd(&sup[r0 + pos], 1u); });
        }
        __syncthreads();
    }

    // light vertices: one warp each, the warp's own table holds N+(v); batches of 32 vertices
    uint32_t* wkey = S.wkey[warp];
    uint16_t* wval = S.wval[warp];
    uint32_t* wcnt = S.wcnt[warp];
    for (;;) {
        uint32_t b0 = 0;
        if (lane == 0) b0 = atomicAdd(ctrl + kHLightCur, 32u);
        b0 = __shfl_sync(kFullMask, b0, 0);
        if (b0 >= n_light) break;
        const uint32_t b1 = min(b0 + 32u, n_light);
        for (uint32_t li = b0; li < b1; ++li) {
            const uint32_t v = light[li], r0 = o_ptr[v], outdeg = o_ptr[v + 1] - r0;
            uint32_t bits = 1;
            while ((1u << bits) < 2 * outdeg) ++bits;
            const uint32_t mask = (1u << bits) - 1;
            for (uint32_t i = lane; i <= mask; i += 32) wkey[i] = kEmpty;
            for (uint32_t i = lane; i < outdeg; i += 32) wcnt[i] = 0;
            __syncwarp();
            for (uint32_t i = lane; i < outdeg; i += 32) {
                const uint32_t w = o_col[r0 + i];
                uint32_t h = hash_slot(w, mask);
                while (atomicCAS(&wkey[h], kEmpty, w) != kEmpty) h = (h + 1) & mask;
                wval[h] = (uint16_t)i;
            }
            __syncwarp();
            stream_tails(o_ptr, o_col, s_col, s_eid, sup, s_ptr[v], s_split[v], 0u, 32u, S.jcnt[warp],
                         [&](uint32_t w) {
                             uint32_t h = hash_slot(w, mask);
                             for (;;) {
                                 const uint32_t k = wkey[h];
                                 if (k == w) return (uint32_t)wval[h];
                                 if (k == kEmpty) return kEmpty;
                                 h = (h + 1) & mask;
                             }
                         },
                         [&](uint32_t pos) { atomicAdd(&wcnt[pos], 1u); });
            __syncwarp();
            for (uint32_t i = lane; i < outdeg; i += 32)
                if (wcnt[i]) atomicAdd(&sup[r0 + i], wcnt[i]);
            __syncwarp();
        }
    }
}

int count_support_hash(kt_engine* e) {
    int rc;
    if ((rc = check_cuda(cudaMemsetAsync(e->ctrl + kHLight, 0, 4 * sizeof(uint32_t), e->stream), "clear plan")))
        return rc;
    k_support_plan<<<(e->n + kThreads - 1) / kThreads, kThreads, 0, e->stream>>>(e->s_ptr, e->s_split, e->o_ptr, e->n,
                                                                                  e->q0, e->chunks0, e->ctrl);
    count_launch(e);
    if ((rc = check_launch(e, "k_support_plan"))) return rc;
    const int smem = (int)sizeof(HashSmem);
    if ((rc = check_cuda(cudaFuncSetAttribute(k_support_hash, cudaFuncAttributeMaxDynamicSharedMemorySize, smem),
                         "shared memory of k_support_hash")))
        return rc;
    int per_sm = 0;
    if ((rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_support_hash, kHashThreads, smem),
                         "occupancy of k_support_hash")))
        return rc;
    if (per_sm < 1) return fail(KT_ERR_CUDA, "k_support_hash cannot be resident");
    k_support_hash<<<e->num_sms * per_sm, kHashThreads, smem, e->stream>>>(e->o_ptr, e->o_col, e->o_fence, e->s_col,
                                                                           e->s_eid, e->s_ptr, e->s_split, e->q0,
                                                                           e->chunks0, e->sup, e->ctrl);
    count_launch(e);
    return check_launch(e, "k_support_hash");
}

}  // namespace

int count_support(kt_engine* e) {
    if (e->m == 0) return KT_OK;
    int rc = check_cuda(cudaMemsetAsync(e->sup, 0, sizeof(uint32_t) * e->m, e->stream), "clear support");
    if (rc) return rc;
    if (e->sched_on_device) {
        // any group the selector may choose (4, 8 or 16 lanes per edge) fits this grid
        const uint64_t blocks = std::min<uint64_t>(((uint64_t)e->m * 16 + kThreads - 1) / kThreads,
                                                   (uint64_t)e->num_sms * 16);
        k_support_chosen<<<(uint32_t)blocks, kThreads, 0, e->stream>>>(e->o_ptr, e->o_col, e->e_src, e->m,
                                                                       e->ctrl + kPSched, e->sup);
        count_launch(e);
        return check_launch(e, "k_support_chosen");
    }
    const uint32_t G = e->sched.support_group;
    if (G == 0) return count_support_hash(e);
    uint64_t blocks = ((uint64_t)e->m * G + kThreads - 1) / kThreads;
    const uint64_t max_blocks = (uint64_t)e->num_sms * 16;
    if (blocks > max_blocks) blocks = max_blocks;
    switch (G) {
        case 4: k_support<4><<<(uint32_t)blocks, kThreads, 0, e->stream>>>(e->o_ptr, e->o_col, e->e_src, e->m, e->sup); break;
        case 16: k_support<16><<<(uint32_t)blocks, kThreads, 0, e->stream>>>(e->o_ptr, e->o_col, e->e_src, e->m, e->sup); break;
        case 32: k_support<32><<<(uint32_t)blocks, kThreads, 0, e->stream>>>(e->o_ptr, e->o_col, e->e_src, e->m, e->sup); break;
        default: k_support<8><<<(uint32_t)blocks, kThreads, 0, e->stream>>>(e->o_ptr, e->o_col, e->e_src, e->m, e->sup); break;
    }
    count_launch(e);
    return check_launch(e, "k_support");
}

}  // namespace kt
