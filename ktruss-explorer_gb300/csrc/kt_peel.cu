// Peeling: the full truss decomposition and the single-k truss, as one persistent kernel.
//
// Replaces the reference's host-driven count/prune loop (kernel_ddc.cu:116-214, the same shape
// in all eight variant files) and its affected-edge recount (kernel_ddc.cu:79-114): support is
// counted once, then kept exact by atomic decrements, and the whole loop over levels and rounds
// runs on the device in one cooperative launch (grid barriers between phases, no host round
// trips).
//
// Level k removes, in synchronous rounds, the alive edges with support < k-2; each removed edge
// gets truss number k-1.  A round's frontier is exactly the set of edges that one count-and-prune
// pass of the reference deletes at that point, so the edge sets agree with the reference pass by
// pass.  When an edge e = (x,y) is removed in round r, every triangle (x,y,w) whose other two
// edges are still alive or removed in round r is destroyed once: the removed edge with the
// smallest id among the triangle's round-r edges decrements each surviving edge by one.  A
// decrement that takes an edge from k-2 to k-3 pushes it onto the next round's frontier, so
// frontiers are built without scans.  A new level starts from one coalesced pass over the
// support array that also finds the minimum support, so empty levels are skipped (k jumps to
// min+3).
//
// One round is one phase followed by one grid barrier.  When an edge is queued (its support
// fell below the threshold, or it is in a level's first frontier) it is stamped with the next
// round number and the walk of its shorter row is split into chunks of up to W entries (the
// schedule's chunk width, 8, 16 or 32); in the round every warp takes chunks, so a long row is
// spread over many warps and no warp walks more than its share.  Per neighbour w of the shorter
// row's vertex x, the edge (y,w) is found by a binary search in an oriented row: in the row's
// fences (every 32nd column, an array that stays in L2), then in one block of at most 32 entries,
// so a search misses L2 once or twice however long the row.  A round whose
// frontier holds at least the schedule's recount share of the alive edges instead removes the
// frontier at once and recounts the survivors' support (the reference's full recount).  A removed
// edge's support is set to kDead, so a level's scan of the alive list reads one array; that scan
// also collects the frontier of level k_last+1, and only when that level turns out to be empty
// does a second pass collect the frontier of the next non-empty level.
// Symmetric rows are compacted in place at a level start once enough edges have been removed
// since the last compaction, so the walks see few removed entries.
//
// Every grid barrier wait is bounded: by the engine's base limit (kt_engine_set_wait_limit, 10 s by
// default) plus a share proportional to the work the wait can legitimately cover - per row entry
// slot of the chunks queued for the round that the barrier closes, per edge for the level phases (scans, compaction,
// recount) - so a long legitimate round on a large graph is not cut short.  On expiry the kernel
// reports KT_ERR_TIMEOUT through the control block and returns.

#include <algorithm>
#include <cstdlib>
#include <vector>

#include "kt_device.cuh"
#include "kt_engine.h"

namespace kt {

namespace {

constexpr int kThreads = 256;          // helper kernels
#ifndef KT_PEEL_THREADS
#define KT_PEEL_THREADS 1024
#endif
constexpr int kPeelThreads = KT_PEEL_THREADS;  // persistent kernel, one block per SM ...
#ifndef KT_PEEL_WIDE_THREADS
#define KT_PEEL_WIDE_THREADS 1024
#endif
#ifndef KT_PEEL_WIDE_BLOCKS
#define KT_PEEL_WIDE_BLOCKS 2
#endif
constexpr int kWideThreads = KT_PEEL_WIDE_THREADS;  // ... or kWideBlocks blocks of kWideThreads per SM
constexpr int kWideBlocks = KT_PEEL_WIDE_BLOCKS;
static_assert(kWideBlocks >= 2, "the wide build has more than one block per SM");
template <int kBlocksPerSm>
__host__ __device__ constexpr int peel_threads() {
    return kBlocksPerSm == 1 ? kPeelThreads : kWideThreads;
}

inline uint32_t grid_for(uint64_t n, int threads = kThreads) {
    uint64_t b = (n + threads - 1) / threads;
    return (uint32_t)(b == 0 ? 1 : b);
}

struct PeelParams {
    const uint32_t* __restrict__ o_ptr;
    const uint32_t* __restrict__ o_col;
    const uint32_t* __restrict__ o_fence;  // o_fence[f] = o_col[32 f]
    const uint32_t* __restrict__ e_src;
    const uint32_t* __restrict__ s_ptr;
    uint32_t* s_len;
    uint32_t* s_col;
    uint32_t* s_eid;
    uint32_t* sup;
    uint32_t* rnd;
    uint32_t* tr;
    uint4* ch[2];      // work chunks of the round's frontier, by round parity
    uint32_t cap_chunks;
    uint32_t* big[2];  // frontier edges walked by whole blocks (chunk buffer full), by parity
    uint32_t* ctrl;
    uint32_t* round_size;
    uint32_t* round_level;
    uint32_t* round_ns;  // device time of each round (first block's view, barrier to barrier)
    uint32_t* level_k;     // per level: k, alive edges at its start, device time of its start
    uint32_t* level_alive; //   (scan and frontier collection), first frontier size
    uint32_t* level_ns;
    uint32_t* level_front;
    uint32_t cap_rounds;
    uint32_t cap_levels;
    uint32_t n, m, big_row, tiny_row;
    uint32_t cw_shift;  // log2 of the chunk width (row entries per work chunk): 3, 4 or 5
    uint32_t compact_num;  // rows are compacted once alive edges < compact_num/100 of the count
                           // at the last compaction (0: never)
    uint32_t recount_num;  // a round whose frontier holds >= recount_num % of the alive edges
                           // recounts the survivors' support instead of decrementing (0: never)
    uint32_t single_k;  // 0: full decomposition; >= 3: the k of a single-k truss
    const uint32_t* d_sched;  // non-null: chunk width, compaction and recount from these control
                              // words (the selector's on-device choice) instead of the three above
    uint64_t wait_base_ns;      // wait limit of every grid barrier: base ...
    uint64_t wait_ns_per_unit;  // ... plus this per unit of work the wait covers
};

constexpr uint32_t kDead = 0xffffffffu;  // support of a removed edge

// The launch's chunk width (log2), compaction and recount percentages, set once per block at the
// start of k_peel from its parameters or from the device-side schedule choice.
__shared__ uint32_t s_sched[3];
// Row entries this block queued for walks over the whole launch (a statistic, added to the control
// block once when the block finishes, so the pushes pay a shared-memory atomic, not a global one).
__shared__ unsigned long long s_walk;
// Edges this block queued since its last barrier and their ring slot (every push between two
// barriers targets the same round), added to the control block once per block at the barrier.
__shared__ uint32_t s_edges, s_edge_slot;
// A level scan's alive count, minimum support and smallest alive edge id over the block's warps.
__shared__ uint32_t s_lv_alive, s_lv_min, s_lv_min_id;
__device__ __forceinline__ uint32_t cw_shift() { return s_sched[0]; }
__device__ __forceinline__ uint32_t compact_num() { return s_sched[1]; }
__device__ __forceinline__ uint32_t recount_num() { return s_sched[2]; }

constexpr uint32_t kFirstChunk = 0x80000000u;
constexpr uint32_t kNullChunk = 0xffffffffu;

// Queues edge e for round rr if `take`: stamps it, and splits the walk of its shorter row into
// chunks of up to W = 1 << cw_shift entries (8, 16 or 32), each walked by W lanes, described by
// {edge, other endpoint y, row position, entry count | kFirstChunk on the edge's first chunk}.
// Rows are only compacted at level starts, so the row measured here is the row walked.  An edge
// queued with support 0 (`walk` false) has no triangle left whose other edges are alive or in
// its round, so nothing to decrement: it gets one empty chunk, which only marks it removed.
// Called by all 32 lanes of a warp together: chunk slots are claimed with one atomic per warp.
// If the chunk buffer is full, the claimed slots are nulled and the edges go to the
// block-walked queue instead.
__device__ __forceinline__ void push_edges(const PeelParams& P, uint32_t e, bool take, uint32_t rr, bool walk) {
    const uint32_t mt = __ballot_sync(kFullMask, take);
    if (!mt) return;
    uint32_t nch = 0, y = 0, base = 0, len = 0;
    if (take) {
        P.rnd[e] = rr;
        if (walk) {
            const uint32_t u = P.e_src[e], v = P.o_col[e];
            const uint32_t lu = P.s_len[u], lv = P.s_len[v];
            const bool ux = lu <= lv;
            y = ux ? v : u;
            base = P.s_ptr[ux ? u : v];
            len = ux ? lu : lv;
        }
        nch = len ? (len + (1u << cw_shift()) - 1) >> cw_shift() : 1;
    }
    const uint32_t lane = lane_id(), slot = rr & 3;
    uint32_t incl = nch;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(kFullMask, incl, o);
        if (lane >= (uint32_t)o) incl += t;
    }
    const uint32_t total = __shfl_sync(kFullMask, incl, 31);
    const uint32_t walked = __reduce_add_sync(kFullMask, len);
    unsigned long long cb = 0;
    if (lane == 0) {
        cb = atomicAdd(reinterpret_cast<unsigned long long*>(P.ctrl + kPChunks) + slot, (unsigned long long)total);
        atomicAdd(&s_edges, __popc(mt));
        s_edge_slot = slot;
        atomicAdd(&s_walk, (unsigned long long)walked);
    }
    cb = __shfl_sync(kFullMask, cb, 0);
    uint4* ch = P.ch[rr & 1];
    if (cb + total <= P.cap_chunks) {
        if (take) {
            const uint32_t c0 = (uint32_t)cb + incl - nch;
            for (uint32_t c = 0; c < nch; ++c) {
                const uint32_t off = c << cw_shift();
                const uint32_t cnt = len > off ? min(1u << cw_shift(), len - off) : 0u;
                ch[c0 + c] = make_uint4(e, y, base + off, cnt | (c == 0 ? kFirstChunk : 0u));
            }
        }
    } else {
        const uint64_t stop = cb + total < P.cap_chunks ? cb + total : P.cap_chunks;
        for (uint64_t i = cb + lane; i < stop; i += 32) ch[i] = make_uint4(kNullChunk, 0, 0, 0);
        uint32_t bb = 0;
        if (lane == 0) bb = atomicAdd(P.ctrl + kPBigCount + slot, __popc(mt));
        bb = __shfl_sync(kFullMask, bb, 0);
        if (take) P.big[rr & 1][bb + __popc(mt & lanemask_lt())] = e;
    }
}

// Grid barrier of the peel: first adds the edges this block queued since its last barrier to
// their round's count (one atomic per block instead of one per pushing warp).  The arrival's
// release orders that add before any block reads the count after the barrier.
__device__ __forceinline__ bool peel_barrier(uint32_t* ctrl, uint32_t nblocks, uint64_t wait_ns) {
    __syncthreads();
    if (threadIdx.x == 0 && s_edges) {
        atomicAdd(ctrl + kPEdges + s_edge_slot, s_edges);
        s_edges = 0;
    }
    return grid_barrier(ctrl, nblocks, wait_ns);
}

// Entries of a removed edge e's shorter row (vertex x): called by all 32 lanes of a warp
// together (each lane may serve a different edge); the lane at position `pos` of its group
// handles row positions base + t0 + pos + j*step (j < NB) that are below base + len (the kernel
// uses NB = 1: wider batches measured slower, their registers spill).  For a neighbour w of x,
// edge (x,w) is s_eid at the entry and edge (y,w) is found by a binary search in an oriented row
// (w in N+(y) if w > y, else y in N+(w)), first in its fences, then in one 32-entry block.  Edge
// states during round r:
// rnd 0 = alive, r+1 = alive but queued for the next round, r = removed in this round,
// 1..r-1 = removed earlier.  A triangle is skipped if one of its edges was removed earlier or if
// a smaller-id edge of this round owns it; otherwise each surviving edge loses one support, and
// an edge whose support falls from k-2 to k-3 is queued for round r+1.
template <int NB>
__device__ __forceinline__ void peel_entries(const PeelParams& P, uint32_t e, uint32_t y, uint32_t base, uint32_t len,
                                             uint32_t t0, uint32_t pos, uint32_t step, uint32_t r, uint32_t km2) {
    uint32_t a[NB], lo[NB], n[NB], end[NB], tgt[NB];
    bool act[NB];
#pragma unroll
    for (int j = 0; j < NB; ++j) {
        const uint32_t t = t0 + pos + (uint32_t)j * step;
        act[j] = t < len;
        uint32_t w = y;
        if (act[j]) {
            w = P.s_col[base + t];
            a[j] = P.s_eid[base + t];
        }
        act[j] = act[j] && w != y;
        if (act[j]) {
            const uint32_t row = w > y ? y : w;
            tgt[j] = w > y ? w : y;
            lo[j] = P.o_ptr[row];
            end[j] = P.o_ptr[row + 1];
            n[j] = end[j] - lo[j];
        }
    }
    uint32_t ra[NB];
#pragma unroll
    for (int j = 0; j < NB; ++j) {
        if (act[j]) {
            ra[j] = P.rnd[a[j]];
            // (x,w) removed earlier: the triangle is gone; (x,w) removed in this round with a
            // smaller id: that edge (or a smaller one) owns the triangle.  Either way no search.
            if ((ra[j] != 0 && ra[j] < r) || (ra[j] == r && a[j] < e)) act[j] = false;
        }
        if (!act[j]) n[j] = 0;
    }
    // lower bounds, through the fences: a row longer than 32 entries is searched in o_fence (a 32x
    // smaller array that stays in L2) and then in one block of at most 32 entries, so a search
    // reads one or two lines of o_col instead of one per halving (R-MAT 24: peel 7.6 s -> 5.4 s)
#pragma unroll
    for (int j = 0; j < NB; ++j)
        if (n[j] > 0) lo[j] = fenced_lower_bound(P.o_col, P.o_fence, lo[j], end[j], tgt[j]);
#pragma unroll
    for (int j = 0; j < NB; ++j) {
        // lo is the lower bound: the edge exists only if it is inside the row and matches
        if (act[j]) act[j] = lo[j] < end[j] && __ldg(P.o_col + lo[j]) == tgt[j];
        bool qa = false, qb = false;
        uint32_t b = 0;
        if (act[j]) {
            b = lo[j];
            const uint32_t rb = P.rnd[b];
            if ((rb == 0 || rb >= r) && !((ra[j] == r && a[j] < e) || (rb == r && b < e))) {
                if (ra[j] != r) qa = atomicSub(&P.sup[a[j]], 1u) == km2;
                if (rb != r) qb = atomicSub(&P.sup[b], 1u) == km2;
            }
        }
        // a decrement queues an edge with support k-3, which is 0 only at level 3
        push_edges(P, a[j], qa, r + 1, km2 != 1);
        push_edges(P, b, qb, r + 1, km2 != 1);
    }
}

// Support of every alive edge (rnd == 0) counted again from scratch over the triangles whose
// three edges are alive, for a round that removes most of the alive edges: walking the rows of
// all removed edges would cost far more than counting what survives.  Supports of alive edges
// must be zero on entry.  Groups of 8 lanes per oriented edge (u,v): the part of N+(u) above v
// (it follows the edge in u's row) is intersected with N+(v), the shorter list walked and the
// longer binary-searched, as in the support count; the oriented rows still hold removed edges,
// which are skipped by their round stamps.
__device__ void recount_support(const PeelParams& P, uint32_t start, uint64_t tid, uint64_t nthreads) {
    constexpr uint32_t G = 8;
    const uint32_t lane = lane_id(), glane = lane & (G - 1);
    const uint32_t gmask = 0xffu << (lane & ~(G - 1));
    for (uint64_t j64 = start + tid / G; j64 < P.m; j64 += nthreads / G) {
        const uint32_t j = (uint32_t)j64;
        if (P.rnd[j] != 0) continue;  // the same for the whole group
        const uint32_t u = P.e_src[j], v = P.o_col[j];
        const uint32_t a0 = j + 1, a1 = P.o_ptr[u + 1];
        const uint32_t b0 = P.o_ptr[v], b1 = P.o_ptr[v + 1];
        const uint32_t na = a1 - a0, nb = b1 - b0;
        uint32_t cnt = 0;
        if (na && nb) {
            const bool iter_a = na <= nb;
            const uint32_t i0 = iter_a ? a0 : b0, ni = iter_a ? na : nb;
            const uint32_t s0 = iter_a ? b0 : a0, ns = iter_a ? nb : na;
            for (uint32_t t = glane; t < ni; t += G) {
                const uint32_t x = i0 + t;
                if (P.rnd[x] != 0) continue;
                const uint32_t w = __ldg(P.o_col + x);
                const uint32_t y = fenced_lower_bound(P.o_col, P.o_fence, s0, s0 + ns, w);
                if (y < s0 + ns && __ldg(P.o_col + y) == w && P.rnd[y] == 0) {
                    ++cnt;
                    atomicAdd(&P.sup[x], 1u);
                    atomicAdd(&P.sup[y], 1u);
                }
            }
        }
        __syncwarp(gmask);
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) cnt += __shfl_xor_sync(gmask, cnt, o);
        if (glane == 0 && cnt) atomicAdd(&P.sup[j], cnt);
    }
}

// Edge e's row walk context: the other endpoint y, the start and length of the shorter row.
__device__ __forceinline__ void slot_context(const PeelParams& P, uint32_t e, uint32_t* y, uint32_t* base,
                                             uint32_t* len) {
    const uint32_t u = P.e_src[e], v = P.o_col[e];
    const uint32_t lu = P.s_len[u], lv = P.s_len[v];
    const bool ux = lu <= lv;
    *y = ux ? v : u;
    *base = P.s_ptr[ux ? u : v];
    *len = ux ? lu : lv;
}

// In-place ordered compaction of the symmetric rows: threads take the tiny rows [0, tiny_row)
// (at most 8 entries, read four at a time), warps the short rows [tiny_row, big_row), blocks the
// long rows [big_row, n).  Entries of edges removed in rounds <= r_done are dropped.  Each step
// reads before any write of the step, and writes never pass the read position.
__device__ void compact_rows(const PeelParams& P, uint32_t r_done, uint32_t* warp_cnt) {
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    const uint32_t gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t big = P.big_row < P.n ? P.big_row : P.n;
    const uint32_t tiny = P.tiny_row < big ? P.tiny_row : big;
    for (uint32_t row = blockIdx.x * blockDim.x + threadIdx.x; row < tiny; row += gridDim.x * blockDim.x) {
        const uint32_t base = P.s_ptr[row], len = P.s_len[row];
        uint32_t w = 0;
        for (uint32_t i0 = 0; i0 < len; i0 += 4) {
            uint32_t c[4], id[4];
            bool keep[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                keep[q] = i0 + q < len;
                if (keep[q]) {
                    c[q] = P.s_col[base + i0 + q];
                    id[q] = P.s_eid[base + i0 + q];
                }
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if (keep[q]) {
                    const uint32_t rr = P.rnd[id[q]];
                    keep[q] = rr == 0 || rr > r_done;
                }
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if (keep[q]) {
                    P.s_col[base + w] = c[q];
                    P.s_eid[base + w] = id[q];
                    ++w;
                }
            }
        }
        P.s_len[row] = w;
    }
    for (uint32_t row = tiny + gwarp; row < big; row += nwarps) {
        const uint32_t base = P.s_ptr[row], len = P.s_len[row];
        uint32_t w = 0;
        for (uint32_t i0 = 0; i0 < len; i0 += 32) {
            const uint32_t i = i0 + lane;
            uint32_t c = 0, eid = 0;
            bool keep = false;
            if (i < len) {
                c = P.s_col[base + i];
                eid = P.s_eid[base + i];
                const uint32_t rr = P.rnd[eid];
                keep = rr == 0 || rr > r_done;
            }
            const uint32_t ballot = __ballot_sync(kFullMask, keep);
            __syncwarp();
            if (keep) {
                const uint32_t pos = base + w + __popc(ballot & lanemask_lt());
                P.s_col[pos] = c;
                P.s_eid[pos] = eid;
            }
            w += __popc(ballot);
        }
        if (lane == 0) P.s_len[row] = w;
    }
    __syncthreads();
    for (uint32_t row = big + blockIdx.x; row < P.n; row += gridDim.x) {
        const uint32_t base = P.s_ptr[row], len = P.s_len[row];
        uint32_t w = 0;
        for (uint32_t i0 = 0; i0 < len; i0 += blockDim.x) {
            const uint32_t i = i0 + threadIdx.x;
            uint32_t c = 0, eid = 0;
            bool keep = false;
            if (i < len) {
                c = P.s_col[base + i];
                eid = P.s_eid[base + i];
                const uint32_t rr = P.rnd[eid];
                keep = rr == 0 || rr > r_done;
            }
            const uint32_t ballot = __ballot_sync(kFullMask, keep);
            if (lane == 0) warp_cnt[warp] = __popc(ballot);
            __syncthreads();
            uint32_t before = 0, total = 0;
            for (uint32_t x = 0; x < (blockDim.x >> 5); ++x) {
                const uint32_t c2 = warp_cnt[x];
                before += x < warp ? c2 : 0;
                total += c2;
            }
            if (keep) {
                const uint32_t pos = base + w + before + __popc(ballot & lanemask_lt());
                P.s_col[pos] = c;
                P.s_eid[pos] = eid;
            }
            w += total;
            __syncthreads();
        }
        if (threadIdx.x == 0) P.s_len[row] = w;
    }
}

// Collects a level's first frontier: alive edges with support <= thr, queued for round rr
// (removed edges hold kDead and never qualify).
__device__ __forceinline__ void collect(const PeelParams& P, uint32_t thr, uint32_t rr, uint32_t start, uint64_t tid,
                                        uint64_t nthreads) {
    for (uint64_t j0 = start + tid - lane_id(); j0 < P.m; j0 += nthreads) {
        const uint64_t j = j0 + lane_id();
        const uint32_t sj = j < P.m ? P.sup[j] : kDead;
        push_edges(P, (uint32_t)j, sj <= thr, rr, sj != 0);
    }
}

// Two builds of the kernel: one block per SM (64 registers a thread) for graphs whose oriented
// CSR fits in L2, and two blocks per SM (32 registers, twice the warps to hide DRAM latency) for
// larger graphs, whose walks wait on DRAM.  Measured on GB300, peel with one / two blocks per SM:
// R-MAT 20 (CSR in L2) 65.5 / 67.4 ms, R-MAT 21 (just over L2) 135.0 / 131.4 ms, R-MAT 24 (CSR
// 2 GB) 6.27 / 4.78 s.
template <int kBlocksPerSm>
__global__ void __launch_bounds__(peel_threads<kBlocksPerSm>(), kBlocksPerSm) k_peel(PeelParams P) {
    __shared__ uint32_t warp_cnt[peel_threads<kBlocksPerSm>() / 32];
    uint32_t* ctrl = P.ctrl;
    if (threadIdx.x == 0) {
        if (P.d_sched) {
            const uint32_t w = P.d_sched[1];
            s_sched[0] = w == 8 ? 3u : w == 16 ? 4u : 5u;
            s_sched[1] = P.d_sched[2];
            s_sched[2] = P.d_sched[3];
        } else {
            s_sched[0] = P.cw_shift;
            s_sched[1] = P.compact_num;
            s_sched[2] = P.recount_num;
        }
        s_walk = 0;
        s_edges = 0;
        s_lv_alive = 0;
        s_lv_min = s_lv_min_id = kDead;
    }
    __syncthreads();
    unsigned long long* chunk_ctr = reinterpret_cast<unsigned long long*>(ctrl + kPChunks);
    const uint32_t nblocks = gridDim.x;
    const uint32_t lane = lane_id();
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;  // grids of at most 2^20 threads
    const uint32_t nthreads = gridDim.x * blockDim.x;
    const uint32_t gwarp = tid >> 5;
    const uint32_t nwarps = nthreads >> 5;
    const bool leader = blockIdx.x == 0 && threadIdx.x == 0;

    // phase clock (block 0, thread 0): time from the previous barrier to the end of this one,
    // kept in shared memory so that it costs the other threads no registers
    __shared__ unsigned long long phase_ns[9];  // [6] = time of the last phase boundary,
                                                // [7] = start of the level, [8] = start of the round
    if (leader) {
        for (int i = 0; i < 6; ++i) phase_ns[i] = 0;
        phase_ns[6] = global_ns();
    }
    uint32_t compactions = 0;
#define KT_PHASE(kind)                                   \
    if (leader) {                                        \
        const unsigned long long now_ = global_ns();     \
        phase_ns[kind] += now_ - phase_ns[6];            \
        phase_ns[6] = now_;                              \
    }

    // wait limits: level phases (scans, compaction, recount) cover work proportional to the edges;
    // a round's closing barrier covers the round's queued chunks, each of at most 1 << cw_shift row
    // entries (read at its start; the count includes chunks that overflowed to the block queue)
    const uint64_t phase_wait = P.wait_base_ns + P.wait_ns_per_unit * 2ull * P.m;
    for (uint64_t j = tid; j < P.m; j += nthreads) {
        P.rnd[j] = 0;
        P.tr[j] = 0;
    }
    if (!peel_barrier(ctrl, nblocks, phase_wait)) return;
    KT_PHASE(0)

    // r: stamp of the last round run.  A level's first round skips one stamp: the blocks still
    // reading the previous level's exit test look at ring slot (r+1) & 3, so the new level's
    // first frontier goes to slot (r+2) & 3.  `rounds` counts the rounds actually run.
    uint32_t r = 0, rounds = 0, level = 0, k = 3, k_last = 2;
    uint32_t live = P.m, live_at_compaction = P.m;  // alive edges now and at the last compaction
#define KT_MAX_STAMP (2ull * P.m + 8)
    for (;;) {
        const uint32_t ls = level & 3;
        if (leader) phase_ns[7] = global_ns();
        r += 1;                     // skipped stamp
        const uint32_t rr = r + 1;  // stamp of this level's first round
        if (level > P.m + 1 || rr > KT_MAX_STAMP) {
            if (leader) atomicOr(ctrl + kCtrlError, kErrRunaway);
            return;
        }
        if (leader) {
            chunk_ctr[(rr + 1) & 3] = 0;
            ctrl[kPBigCount + ((rr + 1) & 3)] = ctrl[kPEdges + ((rr + 1) & 3)] = 0;
        }
        // compact the rows once the alive edges have dropped enough since the last compaction
        if ((uint64_t)live * 100 < (uint64_t)live_at_compaction * compact_num()) {
            compact_rows(P, r, warp_cnt);
            if (!peel_barrier(ctrl, nblocks, phase_wait)) return;
            KT_PHASE(3)
            ++compactions;
            live_at_compaction = live;
        }
        uint32_t lvl_start = 0;  // no edge below this id is alive at this level
        if (P.single_k == 0) {
            // one pass over the alive list: compact it, minimum support, and the frontier of
            // level k_last+1 (the usual next level); a second pass only if that level is empty
            const uint32_t kg = k_last + 1;
            if (leader) {
                const uint32_t z = (level + 2) & 3;
                ctrl[kPLAlive + z] = 0;
                ctrl[kPLMin + z] = 0xffffffffu;
                ctrl[kPLMinId + z] = 0xffffffffu;
            }
            // stream the support array (16-byte loads, four edges per lane; removed edges hold
            // kDead) from the smallest edge id alive at the previous level's scan: edges below it
            // are all removed, and low ids (rows of low-degree vertices) go first
            const uint32_t start = level ? ld_acquire(ctrl + kPLMinId + ((level + 3) & 3)) & ~3u : 0u;
            uint32_t n_alive = 0, mn = kDead, min_id = kDead;
            const uint4* sup4 = reinterpret_cast<const uint4*>(P.sup);
            const uint64_t m4 = ((uint64_t)P.m + 3) / 4;
            constexpr int kScanUnroll = 2;  // 16-byte loads in flight per lane
            for (uint64_t i0 = (start >> 2) + tid - lane; i0 < m4; i0 += nthreads * kScanUnroll) {
                uint4 q4[kScanUnroll];
#pragma unroll
                for (int u = 0; u < kScanUnroll; ++u) {
                    const uint64_t i = i0 + (uint64_t)u * nthreads + lane;
                    q4[u] = i < m4 ? sup4[i] : make_uint4(kDead, kDead, kDead, kDead);
                }
#pragma unroll
                for (int u = 0; u < kScanUnroll; ++u) {
                    const uint64_t i = i0 + (uint64_t)u * nthreads + lane;
                    const uint32_t sv[4] = {q4[u].x, q4[u].y, q4[u].z, q4[u].w};
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        const uint64_t j = 4 * i + c;
                        const uint32_t sj = j < P.m ? sv[c] : kDead;
                        if (sj != kDead) {
                            ++n_alive;
                            mn = sj < mn ? sj : mn;
                            min_id = (uint32_t)j < min_id ? (uint32_t)j : min_id;
                        }
                        push_edges(P, (uint32_t)j, sj != kDead && sj <= kg - 3, rr, sj != 0);
                    }
                }
            }
            n_alive = __reduce_add_sync(kFullMask, n_alive);
            mn = __reduce_min_sync(kFullMask, mn);
            min_id = __reduce_min_sync(kFullMask, min_id);
            if (lane == 0 && n_alive) {
                atomicAdd(&s_lv_alive, n_alive);
                atomicMin(&s_lv_min, mn);
                atomicMin(&s_lv_min_id, min_id);
            }
            __syncthreads();
            if (threadIdx.x == 0 && s_lv_alive) {
                atomicAdd(ctrl + kPLAlive + ls, s_lv_alive);
                atomicMin(ctrl + kPLMin + ls, s_lv_min);
                atomicMin(ctrl + kPLMinId + ls, s_lv_min_id);
                s_lv_alive = 0;
                s_lv_min = s_lv_min_id = kDead;
            }
            if (!peel_barrier(ctrl, nblocks, phase_wait)) return;
            KT_PHASE(1)
            if (ld_acquire(ctrl + kPLAlive + ls) == 0) break;
            k = ld_acquire(ctrl + kPLMin + ls) + 3;
            lvl_start = ld_acquire(ctrl + kPLMinId + ls);
            if (k != kg) {
                collect(P, k - 3, rr, lvl_start, tid, nthreads);
                if (!peel_barrier(ctrl, nblocks, phase_wait)) return;
                KT_PHASE(2)
            }
        } else {
            k = P.single_k;
            collect(P, k - 3, rr, 0u, tid, nthreads);
            if (!peel_barrier(ctrl, nblocks, phase_wait)) return;
            KT_PHASE(2)
        }
        const uint32_t km2 = k - 2;
        uint32_t E = ld_acquire(ctrl + kPEdges + (rr & 3)), B = ld_acquire(ctrl + kPBigCount + (rr & 3));
        if (leader && level < P.cap_levels) {
            P.level_k[level] = k;
            P.level_alive[level] = P.single_k ? P.m : ld_acquire(ctrl + kPLAlive + ls);
            P.level_ns[level] = (uint32_t)(global_ns() - phase_ns[7]);
            P.level_front[level] = E;
        }
        uint32_t C = (uint32_t)min(ld_acquire_u64(chunk_ctr + (rr & 3)), (unsigned long long)P.cap_chunks);
        while (E) {
            ++r;
            ++rounds;
            if (r > KT_MAX_STAMP) {
                if (leader) atomicOr(ctrl + kCtrlError, kErrRunaway);
                return;
            }
            if (leader) {
                const uint32_t z = (r + 2) & 3;
                chunk_ctr[z] = 0;
                ctrl[kPBigCount + z] = 0;
                ctrl[kPEdges + z] = 0;
                if (rounds < P.cap_rounds) {
                    P.round_size[rounds] = E;
                    P.round_level[rounds] = k;
                }
            }
            const bool recount = recount_num() != 0 && (uint64_t)E * 100 >= (uint64_t)recount_num() * live;
            if (leader) phase_ns[8] = phase_ns[6];
            // limit of the barrier that closes the round: base + the round's queued chunk entries
            const uint64_t round_wait =
                threadIdx.x == 0 ? (recount ? phase_wait
                                            : P.wait_base_ns + P.wait_ns_per_unit *
                                                                   (ld_acquire_u64(chunk_ctr + (r & 3)) << cw_shift()))
                                 : 0;
            if (recount) {
                // the whole frontier is removed at once (truss number k-1), the support of every
                // surviving edge is counted again, and the next frontier comes from a scan
                for (uint64_t j = lvl_start + tid; j < P.m; j += nthreads) {
                    const uint32_t st = P.rnd[j];
                    if (st == r) {
                        P.tr[j] = k - 1;
                        P.sup[j] = kDead;
                    } else if (st == 0) {
                        P.sup[j] = 0;
                    }
                }
                if (!peel_barrier(ctrl, nblocks, phase_wait)) return;
                KT_PHASE(4)
                recount_support(P, lvl_start, tid, nthreads);
                if (!peel_barrier(ctrl, nblocks, phase_wait)) return;
                KT_PHASE(4)
                collect(P, k - 3, r + 1, lvl_start, tid, nthreads);
            } else {
            // chunks: a warp takes 32 / W chunks at a time, W lanes per chunk of up to W row
            // entries
            {
                const uint4* ch = P.ch[r & 1];
                const uint32_t per_warp = 32u >> cw_shift(), pos = lane & ((1u << cw_shift()) - 1);
                const uint32_t mine = lane >> cw_shift();
                for (uint32_t c0 = gwarp * per_warp; c0 < C; c0 += nwarps * per_warp) {
                    const uint32_t c = c0 + mine;
                    const uint4 d = c < C ? ch[c] : make_uint4(kNullChunk, 0, 0, 0);
                    const bool real = d.x != kNullChunk;
                    if (real && (d.w & kFirstChunk) && pos == 0) {
                        P.tr[d.x] = k - 1;
                        P.sup[d.x] = kDead;
                    }
                    peel_entries<1>(P, real ? d.x : 0u, d.y, d.z, real ? d.w & ~kFirstChunk : 0u, 0, pos, 32, r, km2);
                }
            }
            // edges that did not fit the chunk buffer: one warp per edge when there are at least
            // as many edges as warps; else one block per edge, or several blocks per edge
            if (B >= nwarps) {
                const uint32_t* bq = P.big[r & 1];
                for (uint32_t i = gwarp; i < B; i += nwarps) {
                    const uint32_t e = bq[i];
                    uint32_t y, base, len;
                    slot_context(P, e, &y, &base, &len);
                    if (lane == 0) {
                        P.tr[e] = k - 1;
                        P.sup[e] = kDead;
                    }
                    for (uint32_t t0 = 0; t0 < len; t0 += 32) peel_entries<1>(P, e, y, base, len, t0, lane, 32, r, km2);
                }
            } else if (B) {
                const uint32_t* bq = P.big[r & 1];
                const uint32_t parts = B >= nblocks ? 1u : nblocks / B;
                const uint32_t units = B >= nblocks ? B : B * parts;
                for (uint32_t u = blockIdx.x; u < units; u += nblocks) {
                    const uint32_t i = u % B, part = u / B;
                    const uint32_t e = bq[i];
                    uint32_t y, base, len;
                    slot_context(P, e, &y, &base, &len);
                    if (part == 0 && threadIdx.x == 0) {
                        P.tr[e] = k - 1;
                        P.sup[e] = kDead;
                    }
                    const uint32_t wofs = threadIdx.x & ~31u;
                    for (uint32_t t0 = part * blockDim.x + wofs; t0 < len; t0 += parts * blockDim.x)
                        peel_entries<1>(P, e, y, base, len, t0, lane, parts * blockDim.x, r, km2);
                }
            }
            }
            if (!peel_barrier(ctrl, nblocks, round_wait)) return;
            if (leader && rounds < P.cap_rounds) P.round_ns[rounds] = (uint32_t)(global_ns() - phase_ns[8]);
            KT_PHASE(recount ? 4 : 5)
            live -= E;
            E = ld_acquire(ctrl + kPEdges + ((r + 1) & 3));
            B = ld_acquire(ctrl + kPBigCount + ((r + 1) & 3));
            C = (uint32_t)min(ld_acquire_u64(chunk_ctr + ((r + 1) & 3)), (unsigned long long)P.cap_chunks);
        }
        ++level;
        k_last = k;
        if (P.single_k != 0) break;
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_walk) atomicAdd(reinterpret_cast<unsigned long long*>(ctrl + kPWalk), s_walk);
    if (leader) {
        ctrl[kPKmax] = P.single_k ? 0 : k_last - 1;
        ctrl[kPRounds] = rounds;
        ctrl[kPLevels] = level;
        ctrl[kPCompactions] = compactions;
        for (int i = 0; i < 6; ++i) {
            ctrl[kPPhaseNs + 2 * i] = (uint32_t)phase_ns[i];
            ctrl[kPPhaseNs + 2 * i + 1] = (uint32_t)(phase_ns[i] >> 32);
        }
    }
#undef KT_PHASE
#undef KT_MAX_STAMP
}

// A barrier that cannot complete (it expects one block more than the grid has): every wait
// runs out after timeout_ns and the kernel returns with kErrTimeout set.
__global__ void k_barrier_probe(uint32_t* ctrl, uint64_t timeout_ns) {
    grid_barrier(ctrl, gridDim.x + 1, timeout_ns);
}

__global__ void k_init_peel_ctrl(uint32_t* ctrl) {
    const uint32_t i = threadIdx.x;
    if (i >= kPBarCount && i < kPSched)
        ctrl[i] = (i >= kPLMin && i < kPLMin + 4) || (i >= kPLMinId && i < kPLMinId + 4) ? 0xffffffffu : 0u;
}

__global__ void k_sum_support(const uint32_t* __restrict__ sup, uint32_t m, unsigned long long* __restrict__ total) {
    uint64_t s = 0;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < m; j += gridDim.x * blockDim.x) s += sup[j];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(kFullMask, s, o);
    if (lane_id() == 0 && s) atomicAdd(total, (unsigned long long)s);
}

__global__ void k_emit_truss(const uint32_t* __restrict__ entry_eid, uint64_t entries, const uint32_t* __restrict__ tr,
                             uint32_t* __restrict__ out) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < entries) out[i] = tr[entry_eid[i]];
}

__global__ void k_emit_keep(const uint32_t* __restrict__ entry_eid, uint64_t entries, const uint32_t* __restrict__ rnd,
                            uint8_t* __restrict__ out) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < entries) out[i] = rnd[entry_eid[i]] == 0 ? 1 : 0;
}

__global__ void k_copy_u32(uint32_t* dst, const uint32_t* src) { *dst = *src; }

// Graph of vertex s: the last g with offsets[g] <= s (num_graphs when s is past the last range,
// 0xffffffff when it is below the first).
__device__ __forceinline__ uint32_t graph_of(const uint32_t* __restrict__ offsets, uint32_t num_graphs, uint32_t s) {
    uint32_t lo = 0, len = num_graphs + 1;
    while (len > 0) {
        const uint32_t half = len >> 1;
        if (offsets[lo + half] <= s) {
            lo += half + 1;
            len -= half + 1;
        } else {
            len = half;
        }
    }
    return lo - 1;
}

// Per-graph k_max of a batch: entry i belongs to the graph whose vertex range holds its source;
// an entry whose endpoints lie in different graphs sets kErrCrossGraph.  Each warp walks its own
// contiguous span of entries 32 at a time and keeps, per lane, the maximum of the graph it is in;
// it adds that maximum to the graph's word with one atomic when the span leaves the graph (and at
// its end).  Batches list their graphs one after another, so the atomics are about one per warp
// and graph boundary - with one per 32 entries, every warp of the grid hit the same few graphs'
// words at once and waited for each other (batch4096: 10.7 ms).  A step that straddles a graph
// boundary or finds entries out of order falls back to a search per lane and combines lanes of
// the same graph before their atomic.
__global__ void k_graph_kmax(const uint32_t* __restrict__ src, const uint32_t* __restrict__ dst, uint64_t entries,
                             const uint32_t* __restrict__ offsets, uint32_t num_graphs,
                             const uint32_t* __restrict__ truss, uint32_t* __restrict__ kmax,
                             uint32_t* __restrict__ ctrl) {
    const uint32_t lane = lane_id();
    const uint64_t gwarp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint64_t span = ((entries + nwarps - 1) / nwarps + 31) & ~31ull;
    const uint64_t begin = gwarp * span;
    const uint64_t end = begin + span < entries ? begin + span : entries;
    uint32_t gc = 0xffffffffu, lo = 1u, hi = 0u;  // the warp's current graph and its vertex range
    uint32_t mx = 0, err = 0;                     // this lane's maximum in graph gc
    for (uint64_t i0 = begin; i0 < end; i0 += 32) {
        const uint64_t i = i0 + lane;
        const bool active = i < end;
        const uint32_t s = active ? src[i] : 0u, d = active ? dst[i] : 0u;
        const uint32_t t = active ? truss[i] : 0u;
        const bool in_gc = !active || (s >= lo && s < hi && d >= lo && d < hi);
        if (__all_sync(kFullMask, in_gc)) {
            mx = t > mx ? t : mx;
            continue;
        }
        // the step leaves graph gc: flush it, then place every entry of the step on its own
        const uint32_t best = __reduce_max_sync(kFullMask, mx);
        if (lane == 0 && gc != 0xffffffffu && best) atomicMax(&kmax[gc], best);
        mx = 0;
        uint32_t g = 0xffffffffu;
        if (active) {
            g = graph_of(offsets, num_graphs, s);
            if (g >= num_graphs || d < offsets[g] || d >= offsets[g + 1]) {
                err = kErrCrossGraph;
                g = 0xffffffffu;
            }
        }
        // the graph of the step's last active lane becomes the current one; the others are
        // combined per graph and added now
        const uint32_t last = 31 - __clz(__ballot_sync(kFullMask, active));
        const uint32_t gl = __shfl_sync(kFullMask, g, last);
        const bool keep = g == gl && g != 0xffffffffu;
        if (keep) mx = t;
        const uint32_t key = keep ? 0xffffffffu : g;
        const uint32_t peers = __match_any_sync(kFullMask, key);
        const uint32_t m2 = __reduce_max_sync(peers, key != 0xffffffffu ? t : 0u);
        if (key != 0xffffffffu && lane == (uint32_t)(__ffs(peers) - 1)) atomicMax(&kmax[key], m2);
        gc = gl;
        if (gc != 0xffffffffu) {
            lo = offsets[gc];
            hi = offsets[gc + 1];
        } else {
            lo = 1u;
            hi = 0u;
        }
    }
    const uint32_t best = __reduce_max_sync(kFullMask, mx);
    if (lane == 0 && gc != 0xffffffffu && best) atomicMax(&kmax[gc], best);
    err = __reduce_or_sync(kFullMask, err);
    if (err && lane == 0) atomicOr(&ctrl[kCtrlError], err);
}

__global__ void k_fill_edges(uint32_t m, uint32_t value, uint32_t* __restrict__ rnd) {
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < m) rnd[j] = value;
}

int launch_peel(kt_engine* e, uint32_t single_k) {
    int rc;
    k_init_peel_ctrl<<<1, kCtrlWords, 0, e->stream>>>(e->ctrl);
    count_launch(e);
    if ((rc = check_launch(e, "k_init_peel_ctrl"))) return rc;
    int l2 = 0;
    if ((rc = check_cuda(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, e->device), "L2 size"))) return rc;
    // automatic choice: two blocks per SM when the oriented CSR outgrows L2 - but not for a batch,
    // whose many small graphs keep their walks local (batch4096: peel 303 ms with one block per
    // SM, 342 ms with two)
    const bool wide = e->sched.peel_blocks == 2 ||
                      (e->sched.peel_blocks == 0 && !e->batch_call && 4 * ((uint64_t)e->m + e->n + 1) > (uint64_t)l2);
    const void* kernel = wide ? (const void*)k_peel<kWideBlocks> : (const void*)k_peel<1>;
    const int threads = wide ? kWideThreads : kPeelThreads;
    int per_sm = 0;
    if ((rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0),
                         "occupancy of k_peel")))
        return rc;
    if (per_sm < 1) return fail(KT_ERR_CUDA, "k_peel cannot be resident (occupancy 0)");
    PeelParams P;
    P.o_ptr = e->o_ptr;
    P.o_col = e->o_col;
    P.o_fence = e->o_fence;
    P.e_src = e->e_src;
    P.s_ptr = e->s_ptr;
    P.s_len = e->s_len;
    P.s_col = e->s_col;
    P.s_eid = e->s_eid;
    P.sup = e->sup;
    P.rnd = e->rnd;
    P.tr = e->tr;
    P.ch[0] = e->chunks0;
    P.ch[1] = e->chunks1;
    P.cap_chunks = e->cap_chunks;
    P.big[0] = e->q0;
    P.big[1] = e->q1;
    P.ctrl = e->ctrl;
    P.round_size = e->round_size;
    P.round_level = e->round_level;
    P.round_ns = e->round_ns;
    P.level_k = e->level_k;
    P.level_alive = e->level_alive;
    P.level_ns = e->level_ns;
    P.level_front = e->level_front;
    P.cap_rounds = e->cap_rounds;
    P.cap_levels = e->cap_levels;
    P.n = e->n;
    P.m = e->m;
    P.big_row = e->big_row;
    P.tiny_row = e->tiny_row < e->big_row ? e->tiny_row : e->big_row;
    P.cw_shift = e->sched.chunk_width == 8 ? 3u : e->sched.chunk_width == 16 ? 4u : 5u;
    P.compact_num = e->sched.compact_percent;
    P.recount_num = e->sched.recount_percent;
    P.single_k = single_k;
    P.d_sched = e->sched_on_device ? e->ctrl + kPSched : nullptr;
    P.wait_base_ns = e->wait_base_ns;
    P.wait_ns_per_unit = e->wait_ns_per_unit;
    void* args[] = {&P};
    const bool timed = e->ev_peel0 && e->ev_peel1 && !e->trusted;
    if (timed && (rc = check_cuda(cudaEventRecord(e->ev_peel0, e->stream), "record event"))) return rc;
    const int blocks_per_sm = wide ? std::min(per_sm, kWideBlocks) : 1;
    rc = check_cuda(cudaLaunchCooperativeKernel(kernel, dim3((unsigned)(e->num_sms * blocks_per_sm)),
                                                dim3((unsigned)threads),
                                                args, 0, e->stream),
                    "cooperative launch of k_peel");
    count_launch(e);
    if (rc || !timed) return rc;
    e->peel_timed = true;
    return check_cuda(cudaEventRecord(e->ev_peel1, e->stream), "record event");
}

int triangles(kt_engine* e) {
    unsigned long long* tot = reinterpret_cast<unsigned long long*>(e->ctrl + kCtrlTriLo);
    int rc = check_cuda(cudaMemsetAsync(tot, 0, sizeof(unsigned long long), e->stream), "clear triangle counter");
    if (rc) return rc;
    if (e->m) {
        k_sum_support<<<(uint32_t)e->num_sms * 4, kThreads, 0, e->stream>>>(e->sup, e->m, tot);
        count_launch(e);
        if ((rc = check_launch(e, "k_sum_support"))) return rc;
    }
    return KT_OK;
}

}  // namespace

int peel_decompose(kt_engine* e) {
    int rc;
    e->peel_timed = false;
    e->peel_mode = 0;
    e->stats_ready = false;
    if ((rc = triangles(e))) return rc;
    if (e->m == 0) return KT_OK;
    return launch_peel(e, 0);
}

int peel_single_k(kt_engine* e, uint32_t k) {
    int rc;
    e->peel_timed = false;
    e->peel_mode = 1;
    e->stats_ready = false;
    if (k >= 3 && (rc = triangles(e))) return rc;
    if (e->m == 0) return KT_OK;
    if (k < 3) {
        // k = 2 keeps every edge; k < 2 removes every edge (k-2 wraps as unsigned, as in
        // mark_deleted_edges_kernel, kernel_ddc.cu:64)
        e->peel_mode = 2;
        k_fill_edges<<<grid_for(e->m), kThreads, 0, e->stream>>>(e->m, k < 2 ? 1u : 0u, e->rnd);
        count_launch(e);
        return check_launch(e, "k_fill_edges");
    }
    return launch_peel(e, k);
}

int emit_truss_per_entry(kt_engine* e, uint32_t* d_out, uint32_t* d_k_max) {
    int rc;
    if (e->entries) {
        k_emit_truss<<<grid_for(e->entries), kThreads, 0, e->stream>>>(e->entry_eid, e->entries, e->tr, d_out);
        count_launch(e);
        if ((rc = check_launch(e, "k_emit_truss"))) return rc;
    }
    if (d_k_max) {
        if (e->m) {
            k_copy_u32<<<1, 1, 0, e->stream>>>(d_k_max, e->ctrl + kPKmax);
        } else {
            if ((rc = check_cuda(cudaMemsetAsync(d_k_max, 0, sizeof(uint32_t), e->stream), "clear k_max"))) return rc;
        }
        count_launch(e);
        if ((rc = check_launch(e, "k_copy_u32"))) return rc;
    }
    return KT_OK;
}

int emit_graph_kmax(kt_engine* e, const uint32_t* d_src, const uint32_t* d_dst, const uint32_t* d_offsets,
                    uint32_t num_graphs, const uint32_t* d_truss, uint32_t* d_kmax) {
    int rc = check_cuda(cudaMemsetAsync(d_kmax, 0, sizeof(uint32_t) * num_graphs, e->stream), "clear k_max");
    if (rc || !e->entries) return rc;
    // a grid of eight blocks a SM; each warp takes a contiguous span of the entries
    const uint64_t blocks = std::min<uint64_t>(grid_for(e->entries), (uint64_t)e->num_sms * 8);
    k_graph_kmax<<<(uint32_t)blocks, kThreads, 0, e->stream>>>(d_src, d_dst, e->entries, d_offsets, num_graphs,
                                                                d_truss, d_kmax, e->ctrl);
    count_launch(e);
    return check_launch(e, "k_graph_kmax");
}

int emit_keep(kt_engine* e, uint8_t* d_keep) {
    if (!e->entries) return KT_OK;
    k_emit_keep<<<grid_for(e->entries), kThreads, 0, e->stream>>>(e->entry_eid, e->entries, e->rnd, d_keep);
    count_launch(e);
    return check_launch(e, "k_emit_keep");
}

// Reads the control block and the round log after the stream has drained; fills the peel
// statistics, including the pass statistics of the reference's chained schedule: level 3 is
// one pass over all m edges; each level k >= 4 up to k_max+1 takes one pass per removing round
// plus a final pass, each seeing the edges alive at its start; levels that remove nothing take
// one pass each.
int finish_stats(kt_engine* e) {
    if (e->stats_ready) return KT_OK;
    if (e->replay_timing) {  // the stream has drained: the replay's events are complete
        e->replay_timing = false;
        int rc = check_cuda(cudaEventElapsedTime(&e->stats.last_ms, e->ev_start, e->ev_stop), "elapsed time");
        if (rc) return rc;
    }
    if (e->m == 0 || e->peel_mode == 2 || e->peel_mode == 3) {
        e->stats.compactions = 0;
        e->stats.walk_entries = 0;
        e->stats.peel_kernel_ms = 0;
        for (int i = 0; i < 6; ++i) e->stats.peel_phase_ms[i] = 0;
        e->stats.k_max = 0;
        e->stats.num_rounds = e->stats.num_levels = e->stats.plain_passes = 0;
        if (e->m && e->peel_mode == 3) e->stats.num_rounds = e->variant_passes;  // count-and-delete passes
        e->stats.plain_alive_sum = 0;
        e->stats.triangles = 0;
        e->stats_ready = true;
        return KT_OK;
    }
    int rc = check_cuda(cudaMemcpy(e->h_ctrl, e->ctrl, sizeof(uint32_t) * kCtrlWords, cudaMemcpyDeviceToHost),
                        "read control block");
    if (rc) return rc;
    const uint32_t err = e->h_ctrl[kCtrlError];
    if (err & kErrTimeout) return fail(KT_ERR_TIMEOUT, "a grid barrier wait of the peel kernel expired");
    if (err & kErrRunaway) return fail(KT_ERR_INTERNAL, "the peel kernel exceeded its round or level bound");
    if (err & kErrCrossGraph) return fail(KT_ERR_INVALID_ARG, "a batch entry joins vertices of two different graphs");
    const uint64_t m = e->m;
    e->stats.triangles = ((uint64_t)e->h_ctrl[kCtrlTriHi] << 32 | e->h_ctrl[kCtrlTriLo]) / 3;
    e->stats.k_max = m ? (e->peel_mode == 0 ? e->h_ctrl[kPKmax] : 0) : 0;
    e->stats.num_rounds = m ? e->h_ctrl[kPRounds] : 0;
    e->stats.num_levels = m ? e->h_ctrl[kPLevels] : 0;
    e->stats.compactions = e->h_ctrl[kPCompactions];
    e->stats.walk_entries = (uint64_t)e->h_ctrl[kPWalk + 1] << 32 | e->h_ctrl[kPWalk];
    if (e->sched_on_device) {  // the schedule the selector chose on the device for this call
        e->sched.support_group = e->h_ctrl[kPSched];
        e->sched.chunk_width = e->h_ctrl[kPSched + 1];
        e->sched.compact_percent = e->h_ctrl[kPSched + 2];
        e->sched.recount_percent = e->h_ctrl[kPSched + 3];
    }
    e->stats.peel_kernel_ms = 0;
    if (e->peel_timed &&
        (rc = check_cuda(cudaEventElapsedTime(&e->stats.peel_kernel_ms, e->ev_peel0, e->ev_peel1), "elapsed time")))
        return rc;
    for (int i = 0; i < 6; ++i)
        e->stats.peel_phase_ms[i] =
            (float)(((uint64_t)e->h_ctrl[kPPhaseNs + 2 * i + 1] << 32 | e->h_ctrl[kPPhaseNs + 2 * i]) * 1e-6);
    e->stats.plain_passes = 0;
    e->stats.plain_alive_sum = 0;
    const uint32_t R = e->stats.num_rounds;
    if (e->peel_mode == 0 && m && R < e->cap_rounds) {
        std::vector<uint32_t> size(R + 1), lvl(R + 1);
        if (R && ((rc = check_cuda(cudaMemcpy(size.data(), e->round_size, sizeof(uint32_t) * (R + 1),
                                              cudaMemcpyDeviceToHost), "read round log")) ||
                  (rc = check_cuda(cudaMemcpy(lvl.data(), e->round_level, sizeof(uint32_t) * (R + 1),
                                              cudaMemcpyDeviceToHost), "read round log"))))
            return rc;
        uint64_t alive = m, passes = 1, alive_sum = m;
        uint32_t next_k = 3;
        for (uint32_t r = 1; r <= R;) {
            const uint32_t k = lvl[r];
            if (k < next_k || k > e->stats.k_max + 1) return fail(KT_ERR_INTERNAL, "inconsistent round log");
            for (uint32_t kk = next_k > 4 ? next_k : 4; kk < k; ++kk) { passes++; alive_sum += alive; }
            while (r <= R && lvl[r] == k) {
                if (k >= 4) { passes++; alive_sum += alive; }
                alive -= size[r];
                ++r;
            }
            if (k >= 4) { passes++; alive_sum += alive; }
            next_k = k + 1;
        }
        e->stats.plain_passes = (uint32_t)passes;
        e->stats.plain_alive_sum = alive_sum;
    }
    e->stats_ready = true;
    return KT_OK;
}

int barrier_timeout_probe(kt_engine* e, uint64_t timeout_ns) {
    int rc = check_cuda(cudaMemsetAsync(e->ctrl, 0, sizeof(uint32_t) * kCtrlWords, e->stream), "clear control block");
    if (rc) return rc;
    uint32_t* ctrl = e->ctrl;
    void* args[] = {&ctrl, &timeout_ns};
    if ((rc = check_cuda(cudaLaunchCooperativeKernel((const void*)k_barrier_probe, dim3(2), dim3(32), args, 0, e->stream),
                         "cooperative launch of k_barrier_probe")))
        return rc;
    count_launch(e);
    if ((rc = check_cuda(cudaStreamSynchronize(e->stream), "synchronize"))) return rc;
    if ((rc = check_cuda(cudaMemcpy(e->h_ctrl, e->ctrl, sizeof(uint32_t) * kCtrlWords, cudaMemcpyDeviceToHost),
                         "read control block")))
        return rc;
    if (e->h_ctrl[kCtrlError] & kErrTimeout) return fail(KT_ERR_TIMEOUT, "barrier probe: wait expired as intended");
    return KT_OK;
}

}  // namespace kt
