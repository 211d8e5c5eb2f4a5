// Peeling: the full truss decomposition and the single-k truss.
//
// Replaces the reference's host-driven count/prune loop (kernel_ddc.cu:116-214, the same
// shape in all eight variant files) and its affected-edge recount (kernel_ddc.cu:79-114):
// support is counted once, then kept exact by atomic decrements.
//
// Level k removes, in synchronous rounds, the alive edges with support < k-2; each removed
// edge gets truss number k-1.  A round's frontier is exactly the set of edges that one
// count-and-prune pass of the reference deletes at that point, so the edge sets agree with
// the reference pass by pass.  When an edge e = (x,y) is removed in round r, every triangle
// (x,y,w) whose other two edges are still alive or removed in round r is destroyed once:
// the removed edge with the smallest id among the triangle's round-r edges decrements each
// surviving edge by one.  A decrement that takes an edge from k-2 to k-3 pushes it onto the
// next round's frontier, so frontiers are built without scans.  A new level starts from a
// scan of the compacted alive-edge list that also finds the minimum support, so empty levels
// are skipped (k jumps to min+3).
//
// Per-round kernels: k_mark (stamp the frontier, record each slot's work), an exclusive scan
// of the work, k_process (find triangles, decrement, push).  Symmetric rows are compacted in
// place once the alive edges have halved since the last compaction, so rows hold few removed
// entries.

#include <vector>

#include "kt_device.cuh"
#include "kt_engine.h"

namespace kt {

namespace {

constexpr int kThreads = 256;

inline uint32_t grid_for(uint64_t n, int threads = kThreads) {
    uint64_t b = (n + threads - 1) / threads;
    return (uint32_t)(b == 0 ? 1 : b);
}

__global__ void k_init_edges(uint32_t m, uint32_t* __restrict__ rnd, uint32_t* __restrict__ tr,
                             uint32_t* __restrict__ alive) {
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < m) {
        rnd[j] = 0;
        tr[j] = 0;
        alive[j] = j;
    }
}

// Warp-ballot stream compaction of the alive list, with the minimum support of the survivors
// (atomicMin into ctrl[kCtrlMin]) and the survivor count (ctrl[kCtrlCount0]).
__global__ void k_level_scan(const uint32_t* __restrict__ alive_in, uint32_t count,
                             const uint32_t* __restrict__ rnd, const uint32_t* __restrict__ sup,
                             uint32_t* __restrict__ alive_out, uint32_t* __restrict__ ctrl) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t e = 0, s = 0xffffffffu;
    bool keep = false;
    if (i < count) {
        e = alive_in[i];
        keep = rnd[e] == 0;
        if (keep) s = sup[e];
    }
    const uint32_t ballot = __ballot_sync(kFullMask, keep);
    uint32_t base = 0;
    if (lane_id() == 0 && ballot) base = atomicAdd(&ctrl[kCtrlCount0], __popc(ballot));
    base = __shfl_sync(kFullMask, base, 0);
    if (keep) alive_out[base + __popc(ballot & lanemask_lt())] = e;
    s = __reduce_min_sync(kFullMask, s);
    if (lane_id() == 0 && s != 0xffffffffu) atomicMin(&ctrl[kCtrlMin], s);
}

// Frontier of a new level: alive edges with support <= thr (= k-3).
__global__ void k_collect(const uint32_t* __restrict__ alive, uint32_t count, const uint32_t* __restrict__ sup,
                          uint32_t thr, uint32_t* __restrict__ q, uint32_t* __restrict__ ctrl) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t e = 0;
    bool take = false;
    if (i < count) {
        e = alive[i];
        take = sup[e] <= thr;
    }
    const uint32_t ballot = __ballot_sync(kFullMask, take);
    uint32_t base = 0;
    if (lane_id() == 0 && ballot) base = atomicAdd(&ctrl[kCtrlCount1], __popc(ballot));
    base = __shfl_sync(kFullMask, base, 0);
    if (take) q[base + __popc(ballot & lanemask_lt())] = e;
}

// Stamps the frontier edges with the round and their truss number, and records for each
// frontier slot the shorter symmetric row (x), the other endpoint (y), x's row start and the
// row length as the slot's work.  work[count] = 0 so that its exclusive scan ends in the total.
__global__ void k_mark(const uint32_t* __restrict__ q, uint32_t count, uint32_t r, uint32_t truss,
                       uint32_t* __restrict__ rnd, uint32_t* __restrict__ tr, const uint32_t* __restrict__ e_src,
                       const uint32_t* __restrict__ o_col, const uint32_t* __restrict__ s_ptr,
                       const uint32_t* __restrict__ s_len, uint32_t* __restrict__ fx, uint32_t* __restrict__ fy,
                       uint32_t* __restrict__ fbase, uint64_t* __restrict__ work) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) {
        const uint32_t e = q[i];
        rnd[e] = r;
        tr[e] = truss;
        const uint32_t u = e_src[e], v = o_col[e];
        const uint32_t lu = s_len[u], lv = s_len[v];
        const bool ux = lu <= lv;
        const uint32_t x = ux ? u : v;
        fx[i] = x;
        fy[i] = ux ? v : u;
        fbase[i] = s_ptr[x];
        work[i] = ux ? lu : lv;
    } else if (i == count) {
        work[count] = 0;
    }
}

__global__ void k_mark_all(const uint32_t* __restrict__ q, uint32_t count, uint32_t r, uint32_t truss,
                           uint32_t* __restrict__ rnd, uint32_t* __restrict__ tr) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) {
        rnd[q[i]] = r;
        tr[q[i]] = truss;
    }
}

// Index i with offs[i] <= t < offs[i+1] in the non-decreasing offs[0, n).
__device__ __forceinline__ uint32_t find_slot(const uint64_t* __restrict__ offs, uint32_t n, uint64_t t) {
    uint32_t lo = 0, len = n;
    while (len > 0) {  // upper bound of t
        uint32_t half = len >> 1;
        if (offs[lo + half] <= t) {
            lo += half + 1;
            len -= half + 1;
        } else {
            len = half;
        }
    }
    return lo - 1;
}

constexpr int kItems = 4;  // work units per lane per warp tile

// One peel round over the flattened work of the frontier: unit t belongs to the slot i with
// offs[i] <= t < offs[i+1] and names entry t - offs[i] of that slot's shorter row.  Each warp
// takes tiles of 32*kItems consecutive units, so long rows are spread over many warps and short
// rows share a warp.  For a neighbour w of x (unit entry), edge (x,w) is identified by its id;
// edge (y,w) by a binary search in an oriented row (w in N+(y) if w > y, else y in N+(w)).  The
// triangle is skipped if either edge was removed in an earlier round or if a smaller-id edge of
// this round owns it; otherwise each still-alive edge loses one support, and an edge whose
// support falls from k-2 to k-3 joins the next frontier.
__global__ void __launch_bounds__(kThreads) k_process(const uint32_t* __restrict__ q, uint32_t count,
                                                      const uint64_t* __restrict__ offs,
                                                      const uint32_t* __restrict__ fx,
                                                      const uint32_t* __restrict__ fy,
                                                      const uint32_t* __restrict__ fbase, uint32_t r, uint32_t k,
                                                      const uint32_t* __restrict__ o_ptr,
                                                      const uint32_t* __restrict__ o_col,
                                                      const uint32_t* __restrict__ s_col,
                                                      const uint32_t* __restrict__ s_eid,
                                                      const uint32_t* __restrict__ rnd, uint32_t* __restrict__ sup,
                                                      uint32_t* __restrict__ qnext, uint32_t* __restrict__ ctrl) {
    const uint64_t W = offs[count];
    const uint32_t lane = lane_id();
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint32_t km2 = k - 2;
    for (uint64_t tile = warp * (32 * kItems); tile < W; tile += nwarps * (32 * kItems)) {
        uint64_t t = tile + lane;
        if (t >= W) continue;
        uint32_t i = find_slot(offs, count + 1, t);
#pragma unroll
        for (int s = 0; s < kItems; ++s, t += 32) {
            if (t >= W) break;
            while (offs[i + 1] <= t) ++i;
            const uint32_t e = q[i], y = fy[i];
            const uint32_t p = fbase[i] + (uint32_t)(t - offs[i]);
            const uint32_t w = s_col[p];
            if (w == y) continue;
            const uint32_t a = s_eid[p];
            const uint32_t ra = rnd[a];
            if (ra != 0 && ra != r) continue;
            uint32_t lo, n, target;
            if (w > y) { lo = o_ptr[y]; n = o_ptr[y + 1] - lo; target = w; }
            else { lo = o_ptr[w]; n = o_ptr[w + 1] - lo; target = y; }
            const uint32_t idx = lower_bound_u32(o_col + lo, n, target);
            if (idx >= n || o_col[lo + idx] != target) continue;
            const uint32_t b = lo + idx;
            const uint32_t rb = rnd[b];
            if (rb != 0 && rb != r) continue;
            if ((ra == r && a < e) || (rb == r && b < e)) continue;
            if (ra == 0) {
                uint32_t old = atomicSub(&sup[a], 1u);
                if (old == km2) qnext[atomicAdd(&ctrl[kCtrlCount1], 1u)] = a;
            }
            if (rb == 0) {
                uint32_t old = atomicSub(&sup[b], 1u);
                if (old == km2) qnext[atomicAdd(&ctrl[kCtrlCount1], 1u)] = b;
            }
        }
    }
}

// In-place ordered compaction of symmetric rows [r0, r1): entries whose edge was removed are
// dropped, the survivors keep their order at the front of the row.  One warp per row: each
// 32-entry step reads before any lane writes, and writes never pass the read position.
__global__ void k_compact_rows_warp(const uint32_t* __restrict__ s_ptr, uint32_t* __restrict__ s_len,
                                    uint32_t* __restrict__ s_col, uint32_t* __restrict__ s_eid,
                                    const uint32_t* __restrict__ rnd, uint32_t r0, uint32_t r1) {
    const uint32_t lane = lane_id();
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t row = r0 + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5); row < r1; row += nwarps) {
        const uint32_t base = s_ptr[row], len = s_len[row];
        uint32_t w = 0;
        for (uint32_t i0 = 0; i0 < len; i0 += 32) {
            const uint32_t i = i0 + lane;
            uint32_t c = 0, eid = 0;
            bool keep = false;
            if (i < len) {
                c = s_col[base + i];
                eid = s_eid[base + i];
                keep = rnd[eid] == 0;
            }
            const uint32_t ballot = __ballot_sync(kFullMask, keep);
            __syncwarp();  // every lane's reads of this step precede any lane's writes
            if (keep) {
                const uint32_t pos = base + w + __popc(ballot & lanemask_lt());
                s_col[pos] = c;
                s_eid[pos] = eid;
            }
            w += __popc(ballot);
        }
        if (lane == 0) s_len[row] = w;
    }
}

// The same for long rows, one block per row.
__global__ void __launch_bounds__(kThreads) k_compact_rows_block(const uint32_t* __restrict__ s_ptr,
                                                                 uint32_t* __restrict__ s_len,
                                                                 uint32_t* __restrict__ s_col,
                                                                 uint32_t* __restrict__ s_eid,
                                                                 const uint32_t* __restrict__ rnd, uint32_t r0,
                                                                 uint32_t r1) {
    __shared__ uint32_t warp_cnt[kThreads / 32];
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    for (uint32_t row = r0 + blockIdx.x; row < r1; row += gridDim.x) {
        const uint32_t base = s_ptr[row], len = s_len[row];
        uint32_t w = 0;
        for (uint32_t i0 = 0; i0 < len; i0 += kThreads) {
            const uint32_t i = i0 + threadIdx.x;
            uint32_t c = 0, eid = 0;
            bool keep = false;
            if (i < len) {
                c = s_col[base + i];
                eid = s_eid[base + i];
                keep = rnd[eid] == 0;
            }
            const uint32_t ballot = __ballot_sync(kFullMask, keep);
            if (lane == 0) warp_cnt[warp] = __popc(ballot);
            __syncthreads();  // every thread has read its entry; counts are visible
            uint32_t before = 0, total = 0;
            for (uint32_t x = 0; x < kThreads / 32; ++x) {
                before += x < warp ? warp_cnt[x] : 0;
                total += warp_cnt[x];
            }
            if (keep) {
                const uint32_t pos = base + w + before + __popc(ballot & lanemask_lt());
                s_col[pos] = c;
                s_eid[pos] = eid;
            }
            w += total;
            __syncthreads();  // writes of this step done before the next step's reads
        }
        if (threadIdx.x == 0) s_len[row] = w;
    }
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

__global__ void k_store_u32(uint32_t* p, uint32_t v) { *p = v; }

int read_ctrl(kt_engine* e) {
    int rc = check_cuda(cudaMemcpyAsync(e->h_ctrl, e->ctrl, sizeof(uint32_t) * kCtrlWords, cudaMemcpyDeviceToHost,
                                        e->stream), "read control block");
    if (rc) return rc;
    return check_cuda(cudaStreamSynchronize(e->stream), "peel synchronize");
}

int set_ctrl(kt_engine* e, uint32_t word, uint32_t value) {
    k_store_u32<<<1, 1, 0, e->stream>>>(e->ctrl + word, value);
    count_launch(e);
    return check_launch(e, "k_store_u32");
}

// Drops removed edges from every symmetric row.
int compact_rows(kt_engine* e) {
    int rc;
    const uint32_t big = e->big_row < e->n ? e->big_row : e->n;
    if (big > 0) {
        uint64_t blocks = ((uint64_t)big * 32 + kThreads - 1) / kThreads;
        uint64_t cap = (uint64_t)e->num_sms * 8;
        k_compact_rows_warp<<<(uint32_t)(blocks < cap ? blocks : cap), kThreads, 0, e->stream>>>(
            e->s_ptr, e->s_len, e->s_col, e->s_eid, e->rnd, 0, big);
        count_launch(e);
        if ((rc = check_launch(e, "k_compact_rows_warp"))) return rc;
    }
    if (big < e->n) {
        uint32_t rows = e->n - big;
        uint32_t blocks = rows < (uint32_t)e->num_sms * 4 ? rows : (uint32_t)e->num_sms * 4;
        k_compact_rows_block<<<blocks, kThreads, 0, e->stream>>>(e->s_ptr, e->s_len, e->s_col, e->s_eid, e->rnd, big,
                                                                 e->n);
        count_launch(e);
        if ((rc = check_launch(e, "k_compact_rows_block"))) return rc;
    }
    return KT_OK;
}

// Runs rounds at level k from the frontier in q0 (count F) until no edge falls below k-2.
// Appends each round's frontier size to `sizes`.  Rows are compacted between rounds once the
// alive edges have halved since the last compaction.
int run_rounds(kt_engine* e, uint32_t k, uint32_t F, uint32_t* r, std::vector<uint32_t>& sizes, uint64_t* alive,
               uint64_t* alive_at_compaction) {
    int rc;
    const uint32_t process_blocks = (uint32_t)e->num_sms * 8;
    while (F) {
        if (*alive * 2 < *alive_at_compaction) {
            if ((rc = compact_rows(e))) return rc;
            *alive_at_compaction = *alive;
        }
        ++*r;
        sizes.push_back(F);
        k_mark<<<grid_for((uint64_t)F + 1), kThreads, 0, e->stream>>>(e->q0, F, *r, k - 1, e->rnd, e->tr, e->e_src,
                                                                      e->o_col, e->s_ptr, e->s_len, e->fx, e->fy,
                                                                      e->fbase, e->work);
        count_launch(e);
        if ((rc = check_launch(e, "k_mark"))) return rc;
        if ((rc = exclusive_scan_u64(e, e->work, e->work, (uint64_t)F + 1))) return rc;
        if ((rc = set_ctrl(e, kCtrlCount1, 0))) return rc;
        k_process<<<process_blocks, kThreads, 0, e->stream>>>(e->q0, F, e->work, e->fx, e->fy, e->fbase, *r, k,
                                                              e->o_ptr, e->o_col, e->s_col, e->s_eid, e->rnd, e->sup,
                                                              e->q1, e->ctrl);
        count_launch(e);
        if ((rc = check_launch(e, "k_process"))) return rc;
        if ((rc = read_ctrl(e))) return rc;
        *alive -= F;
        F = e->h_ctrl[kCtrlCount1];
        std::swap(e->q0, e->q1);
    }
    return KT_OK;
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
    const uint32_t m = e->m;
    int rc;
    e->stats.k_max = 0;
    e->stats.num_levels = 0;
    e->stats.num_rounds = 0;
    e->stats.plain_passes = 0;
    e->stats.plain_alive_sum = 0;
    if ((rc = triangles(e))) return rc;
    if (m == 0) return KT_OK;
    k_init_edges<<<grid_for(m), kThreads, 0, e->stream>>>(m, e->rnd, e->tr, e->alive0);
    count_launch(e);
    if ((rc = check_launch(e, "k_init_edges"))) return rc;
    if ((rc = read_ctrl(e))) return rc;
    e->stats.triangles = ((uint64_t)e->h_ctrl[kCtrlTriHi] << 32 | e->h_ctrl[kCtrlTriLo]) / 3;

    // pass statistics of the reference chain (level 3 is one pass over all m edges, each
    // level k >= 4 up to k_max+1 one pass per removing round plus a final one)
    uint64_t alive = m, passes = 1, alive_sum = m;
    uint64_t live = m, live_at_compaction = m;
    uint32_t count = m, r = 0, k = 3, k_last = 2;
    std::vector<uint32_t> sizes;
    for (;;) {
        if ((rc = set_ctrl(e, kCtrlCount0, 0))) return rc;
        if ((rc = set_ctrl(e, kCtrlMin, 0xffffffffu))) return rc;
        k_level_scan<<<grid_for(count), kThreads, 0, e->stream>>>(e->alive0, count, e->rnd, e->sup, e->alive1, e->ctrl);
        count_launch(e);
        if ((rc = check_launch(e, "k_level_scan"))) return rc;
        if ((rc = read_ctrl(e))) return rc;
        count = e->h_ctrl[kCtrlCount0];
        std::swap(e->alive0, e->alive1);
        if (count == 0) break;
        const uint32_t mn = e->h_ctrl[kCtrlMin];
        const uint32_t next_k = mn + 3;
        for (uint32_t kk = k > 3 ? k : 4; kk < next_k; ++kk) { passes++; alive_sum += alive; }
        k = next_k;
        if ((rc = set_ctrl(e, kCtrlCount1, 0))) return rc;
        k_collect<<<grid_for(count), kThreads, 0, e->stream>>>(e->alive0, count, e->sup, k - 3, e->q0, e->ctrl);
        count_launch(e);
        if ((rc = check_launch(e, "k_collect"))) return rc;
        if ((rc = read_ctrl(e))) return rc;
        const uint32_t F = e->h_ctrl[kCtrlCount1];
        sizes.clear();
        if ((rc = run_rounds(e, k, F, &r, sizes, &live, &live_at_compaction))) return rc;
        for (uint32_t s : sizes) {
            if (k >= 4) { passes++; alive_sum += alive; }
            alive -= s;
        }
        if (k >= 4) { passes++; alive_sum += alive; }
        e->stats.num_levels++;
        k_last = k;
        ++k;
    }
    e->stats.k_max = k_last - 1;
    e->stats.num_rounds = r;
    e->stats.plain_passes = (uint32_t)passes;
    e->stats.plain_alive_sum = alive_sum;
    return KT_OK;
}

int peel_single_k(kt_engine* e, uint32_t k) {
    const uint32_t m = e->m;
    int rc;
    e->stats.num_rounds = 0;
    e->stats.triangles = 0;
    if (k >= 3 && (rc = triangles(e))) return rc;
    if (m == 0) return KT_OK;
    k_init_edges<<<grid_for(m), kThreads, 0, e->stream>>>(m, e->rnd, e->tr, e->alive0);
    count_launch(e);
    if ((rc = check_launch(e, "k_init_edges"))) return rc;
    if (k < 3) {
        // k = 2 keeps every edge; k < 2 removes every edge (k-2 wraps as unsigned, as in
        // mark_deleted_edges_kernel, kernel_ddc.cu:64)
        if (k < 2) {
            k_mark_all<<<grid_for(m), kThreads, 0, e->stream>>>(e->alive0, m, 1, 1, e->rnd, e->tr);
            count_launch(e);
            if ((rc = check_launch(e, "k_mark_all"))) return rc;
        }
        return KT_OK;
    }
    if ((rc = set_ctrl(e, kCtrlCount1, 0))) return rc;
    k_collect<<<grid_for(m), kThreads, 0, e->stream>>>(e->alive0, m, e->sup, k - 3, e->q0, e->ctrl);
    count_launch(e);
    if ((rc = check_launch(e, "k_collect"))) return rc;
    if ((rc = read_ctrl(e))) return rc;
    e->stats.triangles = ((uint64_t)e->h_ctrl[kCtrlTriHi] << 32 | e->h_ctrl[kCtrlTriLo]) / 3;
    uint32_t r = 0;
    uint64_t live = m, live_at_compaction = m;
    std::vector<uint32_t> sizes;
    if ((rc = run_rounds(e, k, e->h_ctrl[kCtrlCount1], &r, sizes, &live, &live_at_compaction))) return rc;
    e->stats.num_rounds = r;
    return KT_OK;
}

int emit_truss_per_entry(kt_engine* e, uint32_t* d_out, uint32_t* d_k_max) {
    int rc;
    if (e->entries) {
        k_emit_truss<<<grid_for(e->entries), kThreads, 0, e->stream>>>(e->entry_eid, e->entries, e->tr, d_out);
        count_launch(e);
        if ((rc = check_launch(e, "k_emit_truss"))) return rc;
    }
    if (d_k_max) {
        k_store_u32<<<1, 1, 0, e->stream>>>(d_k_max, e->stats.k_max);
        count_launch(e);
        if ((rc = check_launch(e, "k_store_u32"))) return rc;
    }
    return KT_OK;
}

int emit_keep(kt_engine* e, uint8_t* d_keep) {
    if (!e->entries) return KT_OK;
    k_emit_keep<<<grid_for(e->entries), kThreads, 0, e->stream>>>(e->entry_eid, e->entries, e->rnd, d_keep);
    count_launch(e);
    return check_launch(e, "k_emit_keep");
}

}  // namespace kt
