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
// Per-round kernels: k_mark (stamp the frontier), k_process (find triangles, decrement).

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

__global__ void k_mark(const uint32_t* __restrict__ q, uint32_t count, uint32_t r, uint32_t truss,
                       uint32_t* __restrict__ rnd, uint32_t* __restrict__ tr) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) {
        uint32_t e = q[i];
        rnd[e] = r;
        tr[e] = truss;
    }
}

// One peel round: a group of G lanes per frontier edge e = (u,v).  The group walks the
// shorter symmetric row (endpoint x, other endpoint y); for each neighbour w it checks edge
// (x,w) by its id, finds edge (y,w) by a binary search in an oriented row (w in N+(y) if
// w > y, else y in N+(w)), applies the ownership rule and decrements survivors.
template <int G>
__global__ void __launch_bounds__(kThreads) k_process(const uint32_t* __restrict__ q, uint32_t count, uint32_t r,
                                                      uint32_t k, const uint32_t* __restrict__ e_src,
                                                      const uint32_t* __restrict__ o_ptr,
                                                      const uint32_t* __restrict__ o_col,
                                                      const uint32_t* __restrict__ s_ptr,
                                                      const uint32_t* __restrict__ s_len,
                                                      const uint32_t* __restrict__ s_col,
                                                      const uint32_t* __restrict__ s_eid,
                                                      const uint32_t* __restrict__ rnd, uint32_t* __restrict__ sup,
                                                      uint32_t* __restrict__ qnext, uint32_t* __restrict__ ctrl) {
    const uint32_t glane = lane_id() & (G - 1);
    const uint64_t gid = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
    const uint64_t ngroups = ((uint64_t)gridDim.x * blockDim.x) / G;
    const uint32_t km2 = k - 2;
    for (uint64_t i = gid; i < count; i += ngroups) {
        const uint32_t e = q[i];
        const uint32_t u = e_src[e], v = o_col[e];
        const uint32_t lu = s_len[u], lv = s_len[v];
        const uint32_t x = lu <= lv ? u : v, y = lu <= lv ? v : u;
        const uint32_t base = s_ptr[x], len = lu <= lv ? lu : lv;
        for (uint32_t t = glane; t < len; t += G) {
            const uint32_t w = s_col[base + t];
            if (w == y) continue;
            const uint32_t a = s_eid[base + t];
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

__global__ void k_sum_support(const uint32_t* __restrict__ sup, uint32_t m, unsigned long long* __restrict__ total) {
    uint64_t s = 0;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < m; j += gridDim.x * blockDim.x) s += sup[j];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(kFullMask, s, o);
    if (lane_id() == 0 && s) atomicAdd(total, (unsigned long long)s);
}

__global__ void k_emit_truss(const uint32_t* __restrict__ sorted_entry, const uint32_t* __restrict__ s_eid,
                             uint64_t entries, const uint32_t* __restrict__ tr, uint32_t* __restrict__ out) {
    uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < entries) out[sorted_entry[p]] = tr[s_eid[p]];
}

__global__ void k_emit_keep(const uint32_t* __restrict__ sorted_entry, const uint32_t* __restrict__ s_eid,
                            uint64_t entries, const uint32_t* __restrict__ rnd, uint8_t* __restrict__ out) {
    uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < entries) out[sorted_entry[p]] = rnd[s_eid[p]] == 0 ? 1 : 0;
}

__global__ void k_store_u32(uint32_t* p, uint32_t v) { *p = v; }

constexpr int G = 8;

uint32_t process_blocks(kt_engine* e, uint32_t count) {
    uint64_t blocks = ((uint64_t)count * G + kThreads - 1) / kThreads;
    uint64_t cap = (uint64_t)e->num_sms * 16;
    if (blocks > cap) blocks = cap;
    return (uint32_t)(blocks ? blocks : 1);
}

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

// Runs rounds at level k from the frontier in q0 (count F) until no edge falls below k-2.
// Appends each round's frontier size to e->stats bookkeeping via the sizes vector.
int run_rounds(kt_engine* e, uint32_t k, uint32_t F, uint32_t* r, std::vector<uint32_t>& sizes) {
    int rc;
    while (F) {
        ++*r;
        sizes.push_back(F);
        k_mark<<<grid_for(F), kThreads, 0, e->stream>>>(e->q0, F, *r, k - 1, e->rnd, e->tr);
        count_launch(e);
        if ((rc = check_launch(e, "k_mark"))) return rc;
        if ((rc = set_ctrl(e, kCtrlCount1, 0))) return rc;
        k_process<G><<<process_blocks(e, F), kThreads, 0, e->stream>>>(e->q0, F, *r, k, e->e_src, e->o_ptr, e->o_col,
                                                                       e->s_ptr, e->s_len, e->s_col, e->s_eid, e->rnd,
                                                                       e->sup, e->q1, e->ctrl);
        count_launch(e);
        if ((rc = check_launch(e, "k_process"))) return rc;
        if ((rc = read_ctrl(e))) return rc;
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
        if ((rc = run_rounds(e, k, F, &r, sizes))) return rc;
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
    if ((rc = triangles(e))) return rc;
    if (m == 0) return KT_OK;
    k_init_edges<<<grid_for(m), kThreads, 0, e->stream>>>(m, e->rnd, e->tr, e->alive0);
    count_launch(e);
    if ((rc = check_launch(e, "k_init_edges"))) return rc;
    if (k < 3) {
        // k = 2 keeps every edge; k < 2 removes every edge (k-2 wraps as unsigned, as in
        // mark_deleted_edges_kernel, kernel_ddc.cu:64)
        if (k < 2) {
            k_mark<<<grid_for(m), kThreads, 0, e->stream>>>(e->alive0, m, 1, 1, e->rnd, e->tr);
            count_launch(e);
            if ((rc = check_launch(e, "k_mark"))) return rc;
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
    std::vector<uint32_t> sizes;
    if ((rc = run_rounds(e, k, e->h_ctrl[kCtrlCount1], &r, sizes))) return rc;
    e->stats.num_rounds = r;
    return KT_OK;
}

int emit_truss_per_entry(kt_engine* e, uint32_t* d_out, uint32_t* d_k_max) {
    int rc;
    if (e->entries) {
        k_emit_truss<<<grid_for(e->entries), kThreads, 0, e->stream>>>(e->sorted_entry, e->s_eid, e->entries, e->tr,
                                                                       d_out);
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
    k_emit_keep<<<grid_for(e->entries), kThreads, 0, e->stream>>>(e->sorted_entry, e->s_eid, e->entries, e->rnd,
                                                                  d_keep);
    count_launch(e);
    return check_launch(e, "k_emit_keep");
}

}  // namespace kt
