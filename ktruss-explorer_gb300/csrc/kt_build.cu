// Device-side graph build: the GB300 replacement for the reference's relabel and COO->CSR
// conversion (sortByDegree graph.cu:152-185, undirected2directedCOO graph.cu:194-237,
// coo2coocsrOnDevice graph.cu:435-478).  The reference sorts vertices on the CPU and sorts
// every adjacency list on the CPU between two PCIe copies; here everything stays in HBM:
//
//   1. degree histogram of the input entries (with id, self-loop checks);
//   2. vertex rank = position in ascending (degree, id) order (radix sort of n keys);
//   3. every entry becomes the key (rank[src] << vb | rank[dst]) carrying its entry index;
//      one radix sort of the 2m keys yields the symmetric CSR with rows sorted by rank;
//   4. each row splits at its own rank: the part above it is the row of the degree-oriented
//      CSR (edge id = position in the oriented array); the part below gets its edge id by a
//      binary search in the neighbour's oriented row, which also proves the input symmetric.
//
// Layout in HBM (n vertices, m undirected edges, all uint32):
//   s_ptr[n+1], s_len[n], s_split[n]   symmetric rows (lower ranks, then higher ranks)
//   s_col[2m], s_eid[2m]               neighbour rank and edge id per symmetric entry
//   o_ptr[n+1], o_col[m], e_src[m]     oriented CSR/COO; edge id = index
//   sorted_entry[2m]                   input entry index of each symmetric entry

#include "kt_device.cuh"
#include "kt_engine.h"

namespace kt {

namespace {

constexpr int kThreads = 256;
constexpr uint32_t kBigRow = 2048;  // rows this long are compacted by a whole block
constexpr uint32_t kTinyRow = 8;    // rows this short are compacted by one thread

inline uint32_t grid_for(uint64_t n, int threads = kThreads) {
    uint64_t b = (n + threads - 1) / threads;
    return (uint32_t)(b == 0 ? 1 : b);
}

// Degree histogram with per-warp aggregation: lanes holding the same source add once (inputs
// listed row by row put a hub's many entries in the same warps).
__global__ void k_degree(const uint32_t* __restrict__ src, const uint32_t* __restrict__ dst, uint64_t entries,
                         uint32_t n, uint32_t* __restrict__ deg, uint32_t* __restrict__ ctrl) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t err = 0, s = 0xffffffffu;
    if (i < entries) {
        s = src[i];
        const uint32_t d = dst[i];
        if (s >= n || d >= n) {
            err = kErrBadVertex;
            s = 0xffffffffu;
        } else if (s == d) {
            err = kErrSelfLoop;
        }
    }
    const uint32_t peers = __match_any_sync(kFullMask, s);
    if (s != 0xffffffffu && lane_id() == (uint32_t)(__ffs(peers) - 1)) atomicAdd(&deg[s], __popc(peers));
    err = __reduce_or_sync(kFullMask, err);
    if (err && lane_id() == 0) atomicOr(&ctrl[kCtrlError], err);
}

__global__ void k_rank_keys(const uint32_t* __restrict__ deg, uint32_t n, unsigned vb, uint64_t* __restrict__ keys) {
    uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < n) keys[v] = ((uint64_t)deg[v] << vb) | v;
}

// Orientation by vertex id (KT_DIRECTED_BY_INDEX, graph.cu:194-207 without the relabel of
// kernel.cu:13-20): rank[v] = v; row_len[v] = degree.
__global__ void k_rank_identity(const uint32_t* __restrict__ deg, uint32_t n, uint32_t* __restrict__ rank,
                                uint32_t* __restrict__ row_len) {
    uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < n) {
        rank[v] = v;
        row_len[v] = deg[v];
    } else if (v == n) {
        row_len[n] = 0;
    }
}

// rank[v] = sorted position; row_len[rank] = degree (row lengths of the symmetric CSR).
__global__ void k_rank_scatter(const uint64_t* __restrict__ sorted, uint32_t n, unsigned vb,
                               uint32_t* __restrict__ rank, uint32_t* __restrict__ row_len) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) {
        uint64_t key = sorted[p];
        rank[(uint32_t)(key & ((1ull << vb) - 1))] = p;
        row_len[p] = (uint32_t)(key >> vb);
    } else if (p == n) {
        row_len[n] = 0;
    }
}

// An id >= n (already flagged by k_degree; the call fails at the end of the build) is read as
// vertex 0, so that every kernel up to that check indexes inside its arrays.
__global__ void k_edge_keys(const uint32_t* __restrict__ src, const uint32_t* __restrict__ dst, uint64_t entries,
                            uint32_t n, const uint32_t* __restrict__ rank, unsigned vb, uint64_t* __restrict__ keys,
                            uint32_t* __restrict__ vals) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < entries) {
        const uint32_t s = src[i], d = dst[i];
        keys[i] = ((uint64_t)rank[s < n ? s : 0] << vb) | rank[d < n ? d : 0];
        vals[i] = (uint32_t)i;
    }
}

__global__ void k_split_init(const uint32_t* __restrict__ s_ptr, uint32_t n, uint32_t* __restrict__ s_split,
                             uint32_t* __restrict__ s_len) {
    uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < n) {
        s_split[r] = s_ptr[r + 1];
        s_len[r] = s_ptr[r + 1] - s_ptr[r];
    }
}

// Neighbour column, duplicate check and the start of each row's higher-rank part.
__global__ void k_csr_fill(const uint64_t* __restrict__ keys, uint64_t entries, unsigned vb,
                           const uint32_t* __restrict__ s_ptr, uint32_t* __restrict__ s_col,
                           uint32_t* __restrict__ s_split, uint32_t* __restrict__ ctrl) {
    uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t err = 0;
    if (p < entries) {
        const uint64_t mask = (1ull << vb) - 1;
        uint64_t key = keys[p];
        uint32_t row = (uint32_t)(key >> vb), col = (uint32_t)(key & mask);
        s_col[p] = col;
        uint64_t prev = p > 0 ? keys[p - 1] : ~0ull;
        if (p > 0 && prev == key) err = kErrDuplicate;
        if (col > row && (p == s_ptr[row] || (uint32_t)(prev >> vb) != row || (uint32_t)(prev & mask) < row))
            s_split[row] = (uint32_t)p;
    }
    err = __reduce_or_sync(kFullMask, err);
    if (err && lane_id() == 0) atomicOr(&ctrl[kCtrlError], err);
}

__global__ void k_out_len(const uint32_t* __restrict__ s_ptr, const uint32_t* __restrict__ s_split, uint32_t n,
                          uint32_t* __restrict__ out_len) {
    uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < n) out_len[r] = s_ptr[r + 1] - s_split[r];
    else if (r == n) out_len[n] = 0;
}

// Higher-rank entries become oriented edges; their edge id is their oriented position.
__global__ void k_orient(const uint64_t* __restrict__ keys, uint64_t entries, unsigned vb,
                         const uint32_t* __restrict__ s_split, const uint32_t* __restrict__ o_ptr,
                         uint32_t* __restrict__ o_col, uint32_t* __restrict__ e_src, uint32_t* __restrict__ s_eid,
                         uint32_t m) {
    uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < entries) {
        uint64_t key = keys[p];
        uint32_t row = (uint32_t)(key >> vb), col = (uint32_t)(key & ((1ull << vb) - 1));
        if (col > row) {
            uint32_t j = o_ptr[row] + (uint32_t)(p - s_split[row]);
            if (j < m) {
                o_col[j] = col;
                e_src[j] = row;
                s_eid[p] = j;
            }
        }
    }
}

// fence[f] = o_col[32 f]: the first level of every search in an oriented row (fenced_lower_bound).
__global__ void k_fences(const uint32_t* __restrict__ o_col, uint32_t m, uint32_t* __restrict__ fence) {
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if ((uint64_t)f * 32 < m) fence[f] = o_col[(uint64_t)f * 32];
}

// Lower-rank entries (row r, column c < r) take the id of edge (c, r) from c's oriented row.
// The oriented CSR must hold exactly m = entries / 2 edges; an input that is not symmetric can
// leave rows that do not nest in [0, m): they are flagged, never searched.
__global__ void k_in_eid(const uint64_t* __restrict__ keys, uint64_t entries, unsigned vb, uint32_t n, uint32_t m,
                         const uint32_t* __restrict__ o_ptr, const uint32_t* __restrict__ o_col,
                         const uint32_t* __restrict__ fence, uint32_t* __restrict__ s_eid,
                         uint32_t* __restrict__ ctrl) {
    uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t err = 0;
    if (p == 0 && o_ptr[n] != m) err = kErrAsymmetric;
    if (p < entries) {
        uint64_t key = keys[p];
        uint32_t row = (uint32_t)(key >> vb), col = (uint32_t)(key & ((1ull << vb) - 1));
        if (col < row) {
            const uint32_t lo = o_ptr[col], hi = o_ptr[col + 1];
            uint32_t idx = 0xffffffffu;
            if (lo <= hi && hi <= m) {
                const uint32_t len = hi - lo;
                idx = fenced_lower_bound(o_col, fence, lo, hi, row) - lo;
                if (idx >= len || o_col[lo + idx] != row) idx = 0xffffffffu;
            }
            if (idx != 0xffffffffu) s_eid[p] = lo + idx;
            else { s_eid[p] = 0; err = kErrAsymmetric; }
        }
    }
    err = __reduce_or_sync(kFullMask, err);
    if (err && lane_id() == 0) atomicOr(&ctrl[kCtrlError], err);
}

// Edge id of each input entry, kept apart from s_eid because peeling compacts the rows.
__global__ void k_entry_eid(const uint32_t* __restrict__ sorted_entry, const uint32_t* __restrict__ s_eid,
                            uint64_t entries, uint32_t* __restrict__ entry_eid) {
    uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < entries) entry_eid[sorted_entry[p]] = s_eid[p];
}

// First rank whose symmetric row has at least `thr` entries (rows grow with rank: ranks are
// ascending degree), written to ctrl[slot].
__global__ void k_find_big_row(const uint32_t* __restrict__ s_ptr, uint32_t n, uint32_t thr,
                               uint32_t* __restrict__ ctrl, uint32_t slot) {
    uint32_t lo = 0, len = n;
    while (len > 0) {
        uint32_t half = len >> 1;
        uint32_t r = lo + half;
        if (s_ptr[r + 1] - s_ptr[r] < thr) {
            lo = r + 1;
            len -= half + 1;
        } else {
            len = half;
        }
    }
    ctrl[slot] = lo;
}

unsigned bits_for(uint64_t n) {
    unsigned b = 1;
    while (b < 64 && (1ull << b) < n) ++b;
    return b;
}

int error_status(uint32_t err) {
    if (err & kErrBadVertex) return fail(KT_ERR_INVALID_ARG, "an entry names a vertex id >= num_nodes");
    if (err & kErrSelfLoop) return fail(KT_ERR_SELF_LOOP, "Edges from a vertex to itself are not allowed!");
    if (err & kErrDuplicate) return fail(KT_ERR_NOT_SYMMETRIC, "duplicate entry in the input edge list");
    if (err & kErrAsymmetric) return fail(KT_ERR_NOT_SYMMETRIC, "entry (u,v) without its reverse (v,u)");
    if (err & kErrTimeout) return fail(KT_ERR_TIMEOUT, "a bounded device wait expired");
    return KT_OK;
}

// Synchronizes and converts the device error word into a status.
int sync_and_check(kt_engine* e) {
    int rc = check_cuda(cudaMemcpyAsync(e->h_ctrl, e->ctrl, sizeof(uint32_t) * kCtrlWords, cudaMemcpyDeviceToHost,
                                        e->stream), "read control block");
    if (rc) return rc;
    rc = check_cuda(cudaStreamSynchronize(e->stream), "build synchronize");
    if (rc) return rc;
    return error_status(e->h_ctrl[kCtrlError]);
}

// Tiled COO/CSR (coo2tiledcoocsr, graph.cu:641-706): key = row << vb | dst with row =
// (src / ts * T + dst / ts) * ts + src % ts; the entry index rides along as the value.
__global__ void k_tile_keys(const uint32_t* __restrict__ src, const uint32_t* __restrict__ dst, uint64_t entries,
                            uint32_t n, uint32_t T, uint32_t ts, unsigned vb, uint64_t* __restrict__ keys,
                            uint32_t* __restrict__ ctrl) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t err = 0;
    if (i < entries) {
        const uint32_t s = src[i], d = dst[i];
        if (s >= n || d >= n) {
            err = kErrBadVertex;
            keys[i] = 0;
        } else {
            const uint64_t row = ((uint64_t)(s / ts) * T + d / ts) * ts + s % ts;
            keys[i] = (row << vb) | d;
        }
    }
    err = __reduce_or_sync(kFullMask, err);
    if (err && lane_id() == 0) atomicOr(&ctrl[kCtrlError], err);
}

// Sorted keys back to entries: the source from the row, the destination from the key.
__global__ void k_tile_entries(const uint64_t* __restrict__ keys, uint64_t entries, uint32_t T, uint32_t ts,
                               unsigned vb, uint32_t* __restrict__ src_out, uint32_t* __restrict__ dst_out) {
    const uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < entries) {
        const uint64_t key = keys[p];
        const uint64_t row = key >> vb;
        const uint64_t tile = row / ts;  // src tile * T + dst tile
        src_out[p] = (uint32_t)((tile / T) * ts + row % ts);
        dst_out[p] = (uint32_t)(key & ((1ull << vb) - 1));
    }
}

// tile_src_ptr[r] = first sorted position whose row is >= r (rows + 1 offsets).
__global__ void k_tile_ptr(const uint64_t* __restrict__ keys, uint64_t entries, unsigned vb, uint64_t rows,
                           uint32_t* __restrict__ ptr) {
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r > rows) return;
    uint64_t lo = 0, len = entries;
    while (len > 0) {
        const uint64_t half = len >> 1;
        if ((keys[lo + half] >> vb) < r) {
            lo += half + 1;
            len -= half + 1;
        } else {
            len = half;
        }
    }
    ptr[r] = (uint32_t)lo;
}

// Symmetrize and deduplicate: entry i becomes the undirected key (min << vb | max); ids >= n
// set kErrBadVertex (key 0, a self loop, dropped).
__global__ void k_canon_keys(const uint32_t* __restrict__ src, const uint32_t* __restrict__ dst, uint64_t entries,
                             uint32_t n, unsigned vb, uint64_t* __restrict__ keys, uint32_t* __restrict__ ctrl) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t err = 0;
    if (i < entries) {
        const uint32_t s = src[i], d = dst[i];
        if (s >= n || d >= n) {
            err = kErrBadVertex;
            keys[i] = 0;
        } else {
            keys[i] = ((uint64_t)(s < d ? s : d) << vb) | (s < d ? d : s);
        }
    }
    err = __reduce_or_sync(kFullMask, err);
    if (err && lane_id() == 0) atomicOr(&ctrl[kCtrlError], err);
}

// flag[p] = 1 for the first copy of each sorted key that is not a self loop; flag[entries] = 0.
__device__ __forceinline__ bool canon_first(const uint64_t* keys, uint64_t p, unsigned vb) {
    const uint64_t key = keys[p];
    return (key >> vb) != (key & ((1ull << vb) - 1)) && (p == 0 || keys[p - 1] != key);
}

__global__ void k_canon_flags(const uint64_t* __restrict__ keys, uint64_t entries, unsigned vb,
                              uint32_t* __restrict__ flag) {
    const uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < entries) flag[p] = canon_first(keys, p, vb) ? 1u : 0u;
    else if (p == entries) flag[p] = 0;
}

// Unique edge j (pos[p] after the scan) goes to j as (lo, hi) and to u + j as (hi, lo), where
// u = pos[entries]; nothing is written unless all 2u entries fit.
__global__ void k_canon_emit(const uint64_t* __restrict__ keys, uint64_t entries, unsigned vb,
                             const uint32_t* __restrict__ pos, uint64_t capacity, uint32_t* __restrict__ src_out,
                             uint32_t* __restrict__ dst_out) {
    const uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t u = pos[entries];
    if (p >= entries || 2 * u > capacity || !canon_first(keys, p, vb)) return;
    const uint64_t key = keys[p];
    const uint32_t lo = (uint32_t)(key >> vb), hi = (uint32_t)(key & ((1ull << vb) - 1));
    const uint64_t j = pos[p];
    src_out[j] = lo;
    dst_out[j] = hi;
    src_out[u + j] = hi;
    dst_out[u + j] = lo;
}

}  // namespace

int symmetrize(kt_engine* e, const uint32_t* d_src, const uint32_t* d_dst, uint64_t entries, uint32_t n,
               uint32_t* d_src_out, uint32_t* d_dst_out, uint64_t capacity, uint64_t* num_out) {
    *num_out = 0;
    if (entries >= 0xffffffffull) return fail(KT_ERR_TOO_LARGE, "more than 2^32-2 entries");
    if (entries && n == 0) return fail(KT_ERR_INVALID_ARG, "entries given for a graph with 0 vertices");
    if (entries == 0) return KT_OK;
    int rc;
    if ((n > e->cap_nodes || entries > e->cap_entries) &&
        (rc = reserve(e, n > e->cap_nodes ? n : e->cap_nodes, entries > e->cap_entries ? entries : e->cap_entries)))
        return rc;
    cudaStream_t st = e->stream;
    const unsigned vb = bits_for(n > 1 ? n : 2);
    if ((rc = check_cuda(cudaMemsetAsync(e->ctrl, 0, sizeof(uint32_t) * kCtrlWords, st), "clear control block")))
        return rc;
    k_canon_keys<<<grid_for(entries), kThreads, 0, st>>>(d_src, d_dst, entries, n, vb, e->key_a, e->ctrl);
    count_launch(e);
    if ((rc = check_launch(e, "k_canon_keys"))) return rc;
    int in_b = 0;
    if ((rc = radix_sort(e, e->key_a, nullptr, e->key_b, nullptr, entries, 2 * vb, &in_b))) return rc;
    const uint64_t* keys = in_b ? e->key_b : e->key_a;
    // the other key buffer (2 * entries words) holds the flags and, scanned in place, the positions
    uint32_t* pos = reinterpret_cast<uint32_t*>(in_b ? e->key_a : e->key_b);
    k_canon_flags<<<grid_for(entries + 1), kThreads, 0, st>>>(keys, entries, vb, pos);
    count_launch(e);
    if ((rc = check_launch(e, "k_canon_flags")) || (rc = exclusive_scan(e, pos, pos, entries + 1))) return rc;
    k_canon_emit<<<grid_for(entries), kThreads, 0, st>>>(keys, entries, vb, pos, capacity, d_src_out, d_dst_out);
    count_launch(e);
    if ((rc = check_launch(e, "k_canon_emit"))) return rc;
    uint32_t u = 0;
    if ((rc = check_cuda(cudaMemcpyAsync(&u, pos + entries, sizeof(uint32_t), cudaMemcpyDeviceToHost, st),
                         "read edge count")) ||
        (rc = sync_and_check(e)))
        return rc;
    *num_out = 2ull * u;
    if (2ull * u > capacity)
        return fail(KT_ERR_CAPACITY, "symmetrized graph has %llu entries, capacity %llu", 2ull * u,
                    (unsigned long long)capacity);
    return KT_OK;
}

int tiled_coocsr(kt_engine* e, const uint32_t* d_src, const uint32_t* d_dst, uint64_t entries, uint32_t n,
                 uint32_t tiles_per_dim, uint32_t* d_tile_src_ptr, uint32_t* d_src_out, uint32_t* d_dst_out) {
    if (tiles_per_dim == 0 || n == 0) return fail(KT_ERR_INVALID_ARG, "tiled layout needs tiles_per_dim >= 1 and n >= 1");
    if (entries >= 0xffffffffull) return fail(KT_ERR_TOO_LARGE, "more than 2^32-2 entries");
    const uint32_t T = tiles_per_dim;
    const uint32_t ts = (uint32_t)(((uint64_t)n + T - 1) / T);
    const uint64_t rows = (uint64_t)T * T * ts;
    const unsigned vb = bits_for(n > 1 ? n : 2);
    const unsigned rb = bits_for(rows + 1);
    if (rb + vb > 64) return fail(KT_ERR_TOO_LARGE, "tiles_per_dim %u too large for %u vertices", T, n);
    int rc;
    if ((n > e->cap_nodes || entries > e->cap_entries) &&
        (rc = reserve(e, n > e->cap_nodes ? n : e->cap_nodes, entries > e->cap_entries ? entries : e->cap_entries)))
        return rc;
    cudaStream_t st = e->stream;
    if ((rc = check_cuda(cudaMemsetAsync(e->ctrl, 0, sizeof(uint32_t) * kCtrlWords, st), "clear control block")))
        return rc;
    int in_b = 0;
    if (entries) {
        k_tile_keys<<<grid_for(entries), kThreads, 0, st>>>(d_src, d_dst, entries, n, T, ts, vb, e->key_a, e->ctrl);
        count_launch(e);
        if ((rc = check_launch(e, "k_tile_keys")) || (rc = sync_and_check(e))) return rc;
        if ((rc = radix_sort(e, e->key_a, nullptr, e->key_b, nullptr, entries, rb + vb, &in_b))) return rc;
        k_tile_entries<<<grid_for(entries), kThreads, 0, st>>>(in_b ? e->key_b : e->key_a, entries, T, ts, vb,
                                                              d_src_out, d_dst_out);
        count_launch(e);
        if ((rc = check_launch(e, "k_tile_entries"))) return rc;
    }
    k_tile_ptr<<<grid_for(rows + 1), kThreads, 0, st>>>(in_b ? e->key_b : e->key_a, entries, vb, rows, d_tile_src_ptr);
    count_launch(e);
    if ((rc = check_launch(e, "k_tile_ptr"))) return rc;
    return check_cuda(cudaStreamSynchronize(st), "synchronize");
}

int build_graph(kt_engine* e, const uint32_t* d_src, const uint32_t* d_dst, uint64_t entries, uint32_t n) {
    if (entries & 1) return fail(KT_ERR_NOT_SYMMETRIC, "odd number of entries (%llu): every edge needs both directions",
                                 (unsigned long long)entries);
    if (entries >= 0xffffffffull) return fail(KT_ERR_TOO_LARGE, "more than 2^32-2 entries");
    if (n > e->cap_nodes || entries > e->cap_entries) {
        int rc = reserve(e, n > e->cap_nodes ? n : e->cap_nodes, entries > e->cap_entries ? entries : e->cap_entries);
        if (rc) return rc;
    }
    e->n = n;
    e->entries = entries;
    e->m = (uint32_t)(entries / 2);
    e->sched_on_device = false;  // a call with a selector sets it after the build
    e->vb = bits_for(n > 1 ? n : 2);
    const unsigned vb = e->vb;
    cudaStream_t st = e->stream;
    int rc = check_cuda(cudaMemsetAsync(e->ctrl, 0, sizeof(uint32_t) * kCtrlWords, st), "clear control block");
    if (rc) return rc;
    if (n == 0) return entries ? fail(KT_ERR_INVALID_ARG, "entries given for a graph with 0 vertices") : KT_OK;

    // 1. degrees (and id / self-loop checks)
    rc = check_cuda(cudaMemsetAsync(e->deg, 0, sizeof(uint32_t) * n, st), "clear degrees");
    if (rc) return rc;
    if (entries) {
        k_degree<<<grid_for(entries), kThreads, 0, st>>>(d_src, d_dst, entries, n, e->deg, e->ctrl);
        count_launch(e);
        if ((rc = check_launch(e, "k_degree"))) return rc;
    }
    // (input errors are read back once, at the end of the build: every kernel before that
    // check indexes inside its arrays whatever the input)

    // 2. ranks: ascending (degree, id), or the ids themselves when orienting by index
    int in_b = 0;
    if (e->orient_by_index) {
        k_rank_identity<<<grid_for((uint64_t)n + 1), kThreads, 0, st>>>(e->deg, n, e->rank, e->s_len);
        count_launch(e);
        if ((rc = check_launch(e, "k_rank_identity"))) return rc;
    } else {
        k_rank_keys<<<grid_for(n), kThreads, 0, st>>>(e->deg, n, vb, e->key_a);
        count_launch(e);
        if ((rc = check_launch(e, "k_rank_keys"))) return rc;
        if ((rc = radix_sort(e, e->key_a, nullptr, e->key_b, nullptr, n, vb + bits_for(entries + 2), &in_b)))
            return rc;
        k_rank_scatter<<<grid_for((uint64_t)n + 1), kThreads, 0, st>>>(in_b ? e->key_b : e->key_a, n, vb, e->rank,
                                                                       e->s_len);
        count_launch(e);
        if ((rc = check_launch(e, "k_rank_scatter"))) return rc;
    }
    // row starts of the symmetric CSR (row r holds the neighbours of the rank-r vertex)
    if ((rc = exclusive_scan(e, e->s_len, e->s_ptr, (uint64_t)n + 1))) return rc;

    // 3. sort entries by (rank[src], rank[dst])
    if (entries) {
        k_edge_keys<<<grid_for(entries), kThreads, 0, st>>>(d_src, d_dst, entries, n, e->rank, vb, e->key_a,
                                                            e->val_a);
        count_launch(e);
        if ((rc = check_launch(e, "k_edge_keys"))) return rc;
        if ((rc = radix_sort(e, e->key_a, e->val_a, e->key_b, e->val_b, entries, 2 * vb, &in_b))) return rc;
    }
    const uint64_t* keys = in_b ? e->key_b : e->key_a;
    e->sorted_entry = in_b ? e->val_b : e->val_a;
    e->entry_eid = in_b ? e->val_a : e->val_b;  // the sort's other value buffer is free now

    // 4. columns, split points, oriented CSR, edge ids
    k_split_init<<<grid_for(n), kThreads, 0, st>>>(e->s_ptr, n, e->s_split, e->s_len);
    count_launch(e);
    if ((rc = check_launch(e, "k_split_init"))) return rc;
    if (entries) {
        k_csr_fill<<<grid_for(entries), kThreads, 0, st>>>(keys, entries, vb, e->s_ptr, e->s_col, e->s_split, e->ctrl);
        count_launch(e);
        if ((rc = check_launch(e, "k_csr_fill"))) return rc;
    }
    k_out_len<<<grid_for((uint64_t)n + 1), kThreads, 0, st>>>(e->s_ptr, e->s_split, n, e->o_ptr);
    count_launch(e);
    if ((rc = check_launch(e, "k_out_len"))) return rc;
    if ((rc = exclusive_scan(e, e->o_ptr, e->o_ptr, (uint64_t)n + 1))) return rc;
    if (entries) {
        k_orient<<<grid_for(entries), kThreads, 0, st>>>(keys, entries, vb, e->s_split, e->o_ptr, e->o_col, e->e_src,
                                                         e->s_eid, e->m);
        count_launch(e);
        if ((rc = check_launch(e, "k_orient"))) return rc;
    }
    if (e->m) {
        k_fences<<<grid_for((e->m + 31) / 32), kThreads, 0, st>>>(e->o_col, e->m, e->o_fence);
        count_launch(e);
        if ((rc = check_launch(e, "k_fences"))) return rc;
    }
    if (entries) {
        k_in_eid<<<grid_for(entries), kThreads, 0, st>>>(keys, entries, vb, n, e->m, e->o_ptr, e->o_col, e->o_fence,
                                                         e->s_eid, e->ctrl);
        count_launch(e);
        if ((rc = check_launch(e, "k_in_eid"))) return rc;
        k_entry_eid<<<grid_for(entries), kThreads, 0, st>>>(e->sorted_entry, e->s_eid, entries, e->entry_eid);
        count_launch(e);
        if ((rc = check_launch(e, "k_entry_eid"))) return rc;
    }
    k_find_big_row<<<1, 1, 0, st>>>(e->s_ptr, n, kBigRow, e->ctrl, kCtrlBigRow);
    count_launch(e);
    if ((rc = check_launch(e, "k_find_big_row"))) return rc;
    k_find_big_row<<<1, 1, 0, st>>>(e->s_ptr, n, kTinyRow + 1, e->ctrl, kCtrlTinyRow);
    count_launch(e);
    if ((rc = check_launch(e, "k_find_big_row"))) return rc;
    if (e->trusted) return KT_OK;  // same input: big_row and tiny_row as read before
    if ((rc = sync_and_check(e))) return rc;
    e->big_row = e->h_ctrl[kCtrlBigRow];
    e->tiny_row = e->h_ctrl[kCtrlTinyRow];
    return KT_OK;
}

}  // namespace kt
