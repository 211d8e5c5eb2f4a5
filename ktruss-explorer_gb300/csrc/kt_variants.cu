// The reference's single-k variants that are not the engine's own peel (config.h:51-161 switches):
//
//   -d undirected (kernel_duc.cu:11-54 and its CPU twin kernel_huc.cu): every pass counts, for
//   each alive edge (u,v), the alive common neighbours of u and v in the symmetric rows - capped
//   at k-2, the count stops as soon as k-2 are found - and deletes the edges below k-2; passes
//   repeat until one deletes nothing (after the first pass at k = 3).  With -r affected, a pass
//   recounts only the edges with an endpoint that lost an edge in the previous pass (the other
//   edges' triangles are unchanged; kernel_duc.cu:79-93 marks the same vertices).  Here a group
//   of G lanes intersects the two rows (the shorter walked, the longer binary-searched), the
//   group's count is summed after every step and the walk stops at the cap; the reference runs
//   one thread per directed entry, merging both full lists.
//
//   -f tiled-coocsr (kernel_ddt.cu:11-63, the 2-D grid of kernel_ddt.cu:141-154): the columns are
//   cut into T tiles of ceil(n/T) vertices; a table holds, for every vertex and column tile, the
//   first position of that tile in the vertex's oriented row (the tiled COO/CSR index over the
//   oriented column array).  A pass clears the supports and counts them again over the alive
//   edges: work item (edge (u,v), slot y) walks the column tiles x = tile(v) + y, + Y, ... (Y =
//   num_parallel_tiles, the reference's -y) and merges the x-tiles of N+(u) and N+(v); a triangle
//   credits its three edges.  Edges below k-2 are then deleted, until a pass deletes nothing.
//   Every pass recounts all alive edges (with -r affected too: the tiled schedule has no affected
//   marking).  Threads per block: the reference's -b.
//
// The pass loop is driven from the host like the reference's (one 4-byte read per pass); edge
// states live in the engine's round stamps (0 = alive, else the pass that deleted the edge), so
// the keep mask is emitted as for the peel.

#include <algorithm>

#include "kt_device.cuh"
#include "kt_engine.h"

namespace kt {

namespace {

constexpr int kThreads = 256;

inline uint32_t grid_for(uint64_t n, int threads = kThreads) {
    uint64_t b = (n + threads - 1) / threads;
    return (uint32_t)(b == 0 ? 1 : b);
}

// Capped count of the alive common neighbours of every alive oriented edge j = (u, v) that must
// be recounted this pass (all of them, or those with a touched endpoint).
template <int G>
__global__ void __launch_bounds__(kThreads) k_capped_count(const uint32_t* __restrict__ s_ptr,
                                                           const uint32_t* __restrict__ s_col,
                                                           const uint32_t* __restrict__ s_eid,
                                                           const uint32_t* __restrict__ o_col,
                                                           const uint32_t* __restrict__ e_src,
                                                           const uint32_t* __restrict__ rnd,
                                                           const uint8_t* __restrict__ touched, uint32_t all,
                                                           uint32_t m, uint32_t cap, uint32_t* __restrict__ cnt) {
    const uint32_t lane = lane_id(), glane = lane & (G - 1);
    const uint32_t gmask = (G == 32) ? kFullMask : (((1u << G) - 1) << (lane & ~(uint32_t)(G - 1)));
    const uint64_t gid = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
    const uint64_t ngroups = ((uint64_t)gridDim.x * blockDim.x) / G;
    for (uint64_t j64 = gid; j64 < m; j64 += ngroups) {
        const uint32_t j = (uint32_t)j64;
        if (rnd[j]) continue;  // the same for the whole group
        const uint32_t u = e_src[j], v = o_col[j];
        if (!all && !touched[u] && !touched[v]) continue;
        const uint32_t a0 = s_ptr[u], na = s_ptr[u + 1] - a0;
        const uint32_t b0 = s_ptr[v], nb = s_ptr[v + 1] - b0;
        uint32_t c = 0;
        // kernel_duc.cu:27: both lists must hold at least k-2 entries
        if (na >= cap && nb >= cap) {
            const bool iter_a = na <= nb;
            const uint32_t i0 = iter_a ? a0 : b0, ni = iter_a ? na : nb;
            const uint32_t s0 = iter_a ? b0 : a0, ns = iter_a ? nb : na;
            for (uint32_t t0 = 0; t0 < ni && c < cap; t0 += G) {
                const uint32_t t = t0 + glane;
                uint32_t hit = 0;
                if (t < ni && rnd[s_eid[i0 + t]] == 0) {
                    const uint32_t w = s_col[i0 + t];
                    const uint32_t y = lower_bound_u32(s_col + s0, ns, w);
                    hit = y < ns && s_col[s0 + y] == w && rnd[s_eid[s0 + y]] == 0;
                }
#pragma unroll
                for (int o = G / 2; o > 0; o >>= 1) hit += __shfl_xor_sync(gmask, hit, o);
                c += hit;
            }
        }
        if (glane == 0) cnt[j] = c < cap ? c : cap;
    }
}

// Deletes the alive edges whose count is below the cap; marks their endpoints for the next pass.
__global__ void k_capped_prune(const uint32_t* __restrict__ o_col, const uint32_t* __restrict__ e_src,
                               const uint32_t* __restrict__ cnt, uint32_t m, uint32_t cap, uint32_t pass,
                               uint32_t* __restrict__ rnd, uint8_t* __restrict__ touched_next,
                               uint32_t* __restrict__ changed) {
    const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool del = false;
    if (j < m && rnd[j] == 0 && cnt[j] < cap) {
        del = true;
        rnd[j] = pass;
        touched_next[e_src[j]] = 1;
        touched_next[o_col[j]] = 1;
    }
    if (__any_sync(kFullMask, del) && lane_id() == 0) *changed = 1;
}

// tile_off[u * T + x] = first position of u's oriented row with a column in tile x (or the row end).
__global__ void k_tile_offsets(const uint32_t* __restrict__ o_ptr, const uint32_t* __restrict__ o_col, uint32_t n,
                               uint32_t T, uint32_t ts, uint32_t* __restrict__ tile_off) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (uint64_t)n * T) return;
    const uint32_t u = (uint32_t)(i / T), x = (uint32_t)(i % T);
    const uint32_t lo = o_ptr[u], hi = o_ptr[u + 1];
    const uint64_t first = (uint64_t)x * ts;
    tile_off[i] = first >= 0xffffffffull ? hi : lo + lower_bound_u32(o_col + lo, hi - lo, (uint32_t)first);
}

// One pass of the tiled count: item (edge j, slot y) merges the column tiles x = tile(v) + y,
// tile(v) + y + Y, ... of N+(u) and N+(v), skipping removed edges; supports of alive edges are
// zero on entry.
__global__ void k_tiled_count(const uint32_t* __restrict__ o_ptr, const uint32_t* __restrict__ o_col,
                              const uint32_t* __restrict__ e_src, const uint32_t* __restrict__ tile_off,
                              const uint32_t* __restrict__ rnd, uint32_t m, uint32_t T, uint32_t ts, uint32_t Y,
                              uint32_t* __restrict__ sup) {
    const uint64_t items = (uint64_t)m * Y;
    for (uint64_t it = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; it < items;
         it += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t j = (uint32_t)(it / Y), y = (uint32_t)(it % Y);
        if (rnd[j]) continue;
        const uint32_t u = e_src[j], v = o_col[j];
        uint32_t c = 0;
        for (uint32_t x = v / ts + y; x < T; x += Y) {
            uint32_t a = tile_off[(uint64_t)u * T + x];
            const uint32_t ae = x + 1 < T ? tile_off[(uint64_t)u * T + x + 1] : o_ptr[u + 1];
            uint32_t b = tile_off[(uint64_t)v * T + x];
            const uint32_t be = x + 1 < T ? tile_off[(uint64_t)v * T + x + 1] : o_ptr[v + 1];
            while (a < ae && b < be) {
                if (rnd[a]) { ++a; continue; }
                if (rnd[b]) { ++b; continue; }
                const uint32_t wa = o_col[a], wb = o_col[b];
                if (wa < wb) {
                    ++a;
                } else if (wa > wb) {
                    ++b;
                } else {
                    ++c;
                    atomicAdd(&sup[a], 1u);
                    atomicAdd(&sup[b], 1u);
                    ++a;
                    ++b;
                }
            }
        }
        if (c) atomicAdd(&sup[j], c);
    }
}

__global__ void k_clear_alive_support(const uint32_t* __restrict__ rnd, uint32_t m, uint32_t* __restrict__ sup) {
    const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j < m && rnd[j] == 0) sup[j] = 0;
}

}  // namespace

int ktruss_tiled(kt_engine* e, uint32_t k, bool recount_all, bool capped) {
    (void)recount_all;  // every tiled pass recounts all alive edges
    (void)capped;       // the undirected cap changes no result; the tiled count finds every triangle
    int rc;
    const uint32_t m = e->m, n = e->n;
    e->peel_mode = 3;
    e->stats_ready = false;
    e->variant_passes = 0;
    if (m == 0) return KT_OK;
    if ((rc = check_cuda(cudaMemsetAsync(e->rnd, 0, sizeof(uint32_t) * m, e->stream), "clear stamps"))) return rc;
    if (k < 3) {
        if (k < 2 && (rc = check_cuda(cudaMemsetAsync(e->rnd, 1, sizeof(uint32_t) * m, e->stream), "delete all")))
            return rc;
        return KT_OK;
    }
    const uint32_t T = e->variant.num_tiles, Y = e->variant.num_parallel_tiles;
    const uint32_t threads = e->variant.block_size;
    const uint32_t ts = (uint32_t)(((uint64_t)n + T - 1) / T);
    const uint64_t words = (uint64_t)n * T;
    if (words > e->tile_off_words) {
        if ((rc = check_cuda(cudaStreamSynchronize(e->stream), "synchronize"))) return rc;
        if (e->tile_off) cudaFree(e->tile_off);
        e->tile_off = nullptr;
        e->tile_off_words = 0;
        if ((rc = check_cuda(cudaMalloc(&e->tile_off, sizeof(uint32_t) * (words ? words : 1)), "allocate tile table")))
            return rc;
        e->tile_off_words = words;
    }
    k_tile_offsets<<<grid_for(words), kThreads, 0, e->stream>>>(e->o_ptr, e->o_col, n, T, ts, e->tile_off);
    count_launch(e);
    if ((rc = check_launch(e, "k_tile_offsets"))) return rc;
    uint32_t* changed = e->ctrl + kCtrlVariantChanged;
    uint32_t* h_changed = e->h_ctrl + kCtrlVariantChanged;
    const uint32_t cap = k - 2;
    const uint64_t items = (uint64_t)m * Y;
    const uint64_t blocks = std::min<uint64_t>((items + threads - 1) / threads, (uint64_t)e->num_sms * 32);
    uint8_t* touched_next = reinterpret_cast<uint8_t*>(e->key_b);  // written by the prune, unused here
    for (uint32_t pass = 1;; ++pass) {
        k_clear_alive_support<<<grid_for(m), kThreads, 0, e->stream>>>(e->rnd, m, e->sup);
        count_launch(e);
        if ((rc = check_launch(e, "k_clear_alive_support"))) return rc;
        k_tiled_count<<<(uint32_t)blocks, threads, 0, e->stream>>>(e->o_ptr, e->o_col, e->e_src, e->tile_off, e->rnd, m,
                                                                   T, ts, Y, e->sup);
        count_launch(e);
        if ((rc = check_launch(e, "k_tiled_count"))) return rc;
        if ((rc = check_cuda(cudaMemsetAsync(changed, 0, sizeof(uint32_t), e->stream), "clear changed"))) return rc;
        k_capped_prune<<<grid_for(m), kThreads, 0, e->stream>>>(e->o_col, e->e_src, e->sup, m, cap, pass, e->rnd,
                                                                  touched_next, changed);
        count_launch(e);
        if ((rc = check_launch(e, "k_capped_prune"))) return rc;
        e->variant_passes = pass;
        if ((rc = check_cuda(cudaMemcpyAsync(h_changed, changed, sizeof(uint32_t), cudaMemcpyDeviceToHost, e->stream),
                             "read changed")) ||
            (rc = check_cuda(cudaStreamSynchronize(e->stream), "synchronize")))
            return rc;
        if (!*h_changed || k == 3) break;  // kernel_ddt.cu: k = 3 needs one pass
        if (pass >= m + 1) return fail(KT_ERR_INTERNAL, "tiled k-truss: pass bound exceeded");
    }
    return KT_OK;
}

int ktruss_undirected(kt_engine* e, uint32_t k, bool recount_all, uint32_t group) {
    int rc;
    const uint32_t m = e->m, n = e->n;
    e->peel_mode = 3;
    e->stats_ready = false;
    e->variant_passes = 0;
    if (m == 0) return KT_OK;
    if ((rc = check_cuda(cudaMemsetAsync(e->rnd, 0, sizeof(uint32_t) * m, e->stream), "clear stamps"))) return rc;
    if (k < 3) {
        // k = 2 keeps every edge; k < 2 deletes every edge (the unsigned k-2 of kernel_duc.cu:64)
        if (k < 2 && (rc = check_cuda(cudaMemsetAsync(e->rnd, 1, sizeof(uint32_t) * m, e->stream), "delete all")))
            return rc;
        return KT_OK;
    }
    // scratch after the build: the sort buffers are free; touched flags of this and the next pass
    uint8_t* touched[2] = {reinterpret_cast<uint8_t*>(e->key_b), reinterpret_cast<uint8_t*>(e->key_b) + n};
    uint32_t* changed = e->ctrl + kCtrlVariantChanged;
    uint32_t* h_changed = e->h_ctrl + kCtrlVariantChanged;
    const uint32_t cap = k - 2;
    const uint64_t blocks = std::min<uint64_t>(((uint64_t)m * group + kThreads - 1) / kThreads, (uint64_t)e->num_sms * 16);
    if ((rc = check_cuda(cudaMemsetAsync(touched[0], 0, 2 * (size_t)n, e->stream), "clear touched"))) return rc;
    for (uint32_t pass = 1;; ++pass) {
        uint8_t* cur = touched[(pass - 1) & 1];
        uint8_t* next = touched[pass & 1];
        const uint32_t all = recount_all || pass == 1;
        switch (group) {
            case 4: k_capped_count<4><<<(uint32_t)blocks, kThreads, 0, e->stream>>>(e->s_ptr, e->s_col, e->s_eid, e->o_col, e->e_src, e->rnd, cur, all, m, cap, e->sup); break;
            case 16: k_capped_count<16><<<(uint32_t)blocks, kThreads, 0, e->stream>>>(e->s_ptr, e->s_col, e->s_eid, e->o_col, e->e_src, e->rnd, cur, all, m, cap, e->sup); break;
            case 32: k_capped_count<32><<<(uint32_t)blocks, kThreads, 0, e->stream>>>(e->s_ptr, e->s_col, e->s_eid, e->o_col, e->e_src, e->rnd, cur, all, m, cap, e->sup); break;
            default: k_capped_count<8><<<(uint32_t)blocks, kThreads, 0, e->stream>>>(e->s_ptr, e->s_col, e->s_eid, e->o_col, e->e_src, e->rnd, cur, all, m, cap, e->sup); break;
        }
        count_launch(e);
        if ((rc = check_launch(e, "k_capped_count"))) return rc;
        if ((rc = check_cuda(cudaMemsetAsync(next, 0, n, e->stream), "clear touched")) ||
            (rc = check_cuda(cudaMemsetAsync(changed, 0, sizeof(uint32_t), e->stream), "clear changed")))
            return rc;
        k_capped_prune<<<grid_for(m), kThreads, 0, e->stream>>>(e->o_col, e->e_src, e->sup, m, cap, pass, e->rnd,
                                                                  next, changed);
        count_launch(e);
        if ((rc = check_launch(e, "k_capped_prune"))) return rc;
        e->variant_passes = pass;
        if ((rc = check_cuda(cudaMemcpyAsync(h_changed, changed, sizeof(uint32_t), cudaMemcpyDeviceToHost, e->stream),
                             "read changed")) ||
            (rc = check_cuda(cudaStreamSynchronize(e->stream), "synchronize")))
            return rc;
        if (!*h_changed || k == 3) break;  // kernel_duc.cu: k = 3 needs one pass
        if (pass >= m + 1) return fail(KT_ERR_INTERNAL, "undirected k-truss: pass bound exceeded");
    }
    return KT_OK;
}

}  // namespace kt
