// The device-resident engine: workspace layout in HBM and the internal stages.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "kt_internal.h"

// Most blocks of the selector's statistics launch (its per-block partials buffer).
constexpr uint32_t kSelMaxBlocks = 1024;

struct kt_engine {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_start = nullptr, ev_stop = nullptr, ev_built = nullptr, ev_counted = nullptr;
    cudaEvent_t ev_select = nullptr;  // after the build, before the selector's choice
    cudaEvent_t ev_copy[4] = {};      // host-buffer calls: around the input and output copies
    cudaEvent_t ev_peel0 = nullptr, ev_peel1 = nullptr;  // around the peel kernel launch
    cudaEvent_t ev_peeled = nullptr;  // decompositions: after the peel, before the per-entry output
    bool emit_timed = false;          // ev_peeled was recorded in this call
    bool peel_timed = false;
    uint64_t launches = 0;

    // Workspace arena: one allocation carved into the arrays below.
    void* arena = nullptr;
    size_t arena_bytes = 0;
    uint32_t cap_nodes = 0;
    uint64_t cap_entries = 0;

    // Sort buffers (2m entries): keys (src_rank << vb | dst_rank) and entry indices.
    uint64_t* key_a = nullptr;
    uint64_t* key_b = nullptr;
    uint32_t* val_a = nullptr;
    uint32_t* val_b = nullptr;
    // Per vertex (rank space unless noted).
    uint32_t* deg = nullptr;      // degree by original id
    uint32_t* rank = nullptr;     // original id -> rank
    uint32_t* s_ptr = nullptr;    // n+1: symmetric CSR row starts
    uint32_t* s_len = nullptr;    // n: live length of each symmetric row (after compaction)
    uint32_t* s_split = nullptr;  // n: first position of the row's higher-rank neighbours
    uint32_t* o_ptr = nullptr;    // n+1: oriented CSR row starts (edge id of a row's first edge)
    // Per symmetric entry (2m).
    uint32_t* s_col = nullptr;    // neighbour rank
    uint32_t* s_eid = nullptr;    // edge id of the entry
    uint32_t* sorted_entry = nullptr;  // input entry index at this sorted position (build only)
    uint32_t* entry_eid = nullptr;     // edge id of each input entry (outputs are gathered by it)
    // Per edge (m); edge id = position in the oriented CSR.
    uint32_t* o_col = nullptr;    // higher-rank endpoint
    uint32_t* o_fence = nullptr;  // o_fence[f] = o_col[32 f]: the first level of row searches
    uint32_t* e_src = nullptr;    // lower-rank endpoint
    uint32_t* sup = nullptr;      // support (alive triangles)
    uint32_t* rnd = nullptr;      // 0 while alive, else the peel round that removed it
    uint32_t* tr = nullptr;       // truss number (written at removal)
    uint32_t* q0 = nullptr;       // edges walked by whole blocks, by round parity
    uint32_t* q1 = nullptr;
    uint4* chunks0 = nullptr;     // peel work chunks, by round parity
    uint4* chunks1 = nullptr;
    uint32_t cap_chunks = 0;
    uint32_t big_row = 0;         // ranks >= big_row have rows of kBigRow entries or more
    uint32_t tiny_row = 0;        // ranks < tiny_row have rows of at most 8 entries
    // Scratch for scans and sort histograms.
    uint32_t* scan_tmp = nullptr;
    size_t scan_tmp_words = 0;
    uint32_t* hist = nullptr;
    size_t hist_words = 0;
    // Control block (device) and its pinned host mirror.
    uint32_t* ctrl = nullptr;
    uint32_t* h_ctrl = nullptr;
    // Per-round log: frontier size and level of each peel round.
    uint32_t* round_size = nullptr;
    uint32_t* round_level = nullptr;
    uint32_t* round_ns = nullptr;
    uint32_t cap_levels = 0;
    uint32_t* level_k = nullptr;      // per-level log (k, alive, start time, first frontier)
    uint32_t* level_alive = nullptr;
    uint32_t* level_ns = nullptr;
    uint32_t* level_front = nullptr;
    uint32_t cap_rounds = 0;
    // Staging for the host-buffer entry points.
    uint32_t* in_src = nullptr;
    uint32_t* in_dst = nullptr;
    uint32_t* out_u32 = nullptr;
    uint8_t* out_u8 = nullptr;
    uint32_t* aux = nullptr;       // batch staging: vertex offsets and per-graph k_max (own allocation)
    size_t aux_words = 0;
    uint32_t* tile_off = nullptr;  // tiled variant: first oriented position of each (vertex, column tile)
    size_t tile_off_words = 0;     //   (own allocation, made by the first tiled call)

    // Current graph.
    uint32_t n = 0;
    uint64_t entries = 0;
    uint32_t m = 0;
    uint32_t vb = 1;  // bits per rank in sort keys

    kt_schedule sched{8, 32, 85, 50, 0};  // kernel schedule (kt_engine_set_schedule)
    kt_variant variant{KT_DIRECTED_BY_DEGREE, KT_FORMAT_COOCSR, KT_RECOUNT_ALL, 512, 8, 8};  // single-k calls
    bool orient_by_index = false;      // the current build orients by vertex id (KT_DIRECTED_BY_INDEX)
    uint32_t variant_passes = 0;       // passes of the last undirected or tiled single-k call
    uint64_t wait_base_ns = 10ull * 1000 * 1000 * 1000;  // peel barrier wait limit: base ...
    uint64_t wait_ns_per_unit = 8;                        // ... plus per unit of covered work
    bool batch_call = false;           // the current call decomposes a batch of separate graphs
    kt_selector* selector = nullptr;   // learned schedule selector (kt_engine_set_selector)
    bool sched_on_device = false;      // this call's schedule is the selector's choice in ctrl[kPSched]
    uint32_t* sel_stats = nullptr;     // 16 u64: the selector's block ticket (word kTicket)
    uint64_t* sel_part = nullptr;      // per-block partial statistics (kSelMaxBlocks x 10 u64)
    float* sel_feat = nullptr;         // the 16 features
    uint32_t* sel_choice = nullptr;    // the selector's schedule index
    kt_stats stats{};
    int peel_mode = 0;          // 0 decomposition, 1 single-k peel, 2 k < 3, 3 single-k variant passes
    // Replay (kt_engine_replay): the last decomposition or single-k call on device buffers, and
    // its device pipeline as an instantiated CUDA graph once captured.  `trusted` marks a pipeline
    // run whose input already passed its checks: no host reads, no timing events (capturable).
    struct LastCall {
        int kind = 0;  // 0 none, 1 decomposition, 2 single-k truss
        const uint32_t* src = nullptr;
        const uint32_t* dst = nullptr;
        uint64_t entries = 0;
        uint32_t n = 0;
        uint32_t* truss = nullptr;
        uint32_t* k_max = nullptr;
        uint32_t k = 0;
        uint8_t* keep = nullptr;
        uint32_t big_row = 0, tiny_row = 0;  // read back by the call's build; a trusted build does not
    } last;
    cudaGraphExec_t replay = nullptr;
    bool replay_direct = false;      // the pipeline could not be captured: replays launch it directly
    uint64_t replay_launches = 0;    // kernel launches in one replay
    int replay_peel_mode = 0;
    bool trusted = false;
    bool replay_timing = false;      // last_ms of a replay is read when the stream has drained
    bool stats_ready = false;   // stats already read back from the device
};

namespace kt {

// Launch bookkeeping: every kernel launch of the engine goes through this.
inline void count_launch(kt_engine* e, uint64_t n = 1) { e->launches += n; }
int check_cuda(cudaError_t err, const char* what);
int check_launch(kt_engine* e, const char* what);

int reserve(kt_engine* e, uint32_t max_nodes, uint64_t max_entries);
// kt_engine_replay bookkeeping (kt_engine.cu)
void drop_replay(kt_engine* e);
void remember(kt_engine* e, const kt_engine::LastCall& c);
void forget(kt_engine* e);
size_t carve(kt_engine* e, char* base, uint32_t n, uint64_t N, bool staging);

// kt_sort.cu
int exclusive_scan(kt_engine* e, const uint32_t* in, uint32_t* out, uint64_t n);
int exclusive_scan_u64(kt_engine* e, const uint64_t* in, uint64_t* out, uint64_t n);
// Sorts (keys, vals) by the low `bits` bits of the keys; ping-pongs between a and b buffers
// and returns 0 if the result is in (key_a, val_a), 1 if in (key_b, val_b).  vals may be null.
int radix_sort(kt_engine* e, uint64_t* key_a, uint32_t* val_a, uint64_t* key_b, uint32_t* val_b,
               uint64_t n, unsigned bits, int* result_in_b);

// kt_build.cu: relabel by degree, orient, sort, symmetric + oriented CSR, edge ids.
int build_graph(kt_engine* e, const uint32_t* d_src, const uint32_t* d_dst, uint64_t entries, uint32_t n);

// Symmetric simple graph of an arbitrary entry list (directions merged, duplicates and self loops
// dropped): (lo, hi) pairs in sorted order, then the same pairs reversed; synchronous.
int symmetrize(kt_engine* e, const uint32_t* d_src, const uint32_t* d_dst, uint64_t entries, uint32_t n,
               uint32_t* d_src_out, uint32_t* d_dst_out, uint64_t capacity, uint64_t* num_out);

// Tiled COO/CSR of an entry list (the reference's tiled layout); synchronous.
int tiled_coocsr(kt_engine* e, const uint32_t* d_src, const uint32_t* d_dst, uint64_t entries, uint32_t n,
                 uint32_t tiles_per_dim, uint32_t* d_tile_src_ptr, uint32_t* d_src_out, uint32_t* d_dst_out);

// kt_support.cu: support of every edge (triangles through it) into e->sup.
int count_support(kt_engine* e);

// kt_peel.cu
int peel_decompose(kt_engine* e);
int peel_single_k(kt_engine* e, uint32_t k);
int emit_truss_per_entry(kt_engine* e, uint32_t* d_out, uint32_t* d_k_max);
int emit_keep(kt_engine* e, uint8_t* d_keep);
int emit_graph_kmax(kt_engine* e, const uint32_t* d_src, const uint32_t* d_dst, const uint32_t* d_offsets,
                    uint32_t num_graphs, const uint32_t* d_truss, uint32_t* d_kmax);
// kt_selector.cu: graph statistics and features of the built graph into e->sel_feat (and, with
// d_params, the selector's schedule index into e->sel_choice and that schedule into
// ctrl[kPSched..]); select_schedule runs the attached selector on the device and marks the call's
// schedule as device-chosen (e->sched_on_device; the support count and the peel read it there).
int graph_features(kt_engine* e, const float* d_params);
int select_schedule(kt_engine* e);
// Reads the peel's control block and round log (stream must be drained); reports timeouts.
int finish_stats(kt_engine* e);
// Launches a grid barrier that cannot complete and returns the status it reports.
int barrier_timeout_probe(kt_engine* e, uint64_t timeout_ns);
// kt_variants.cu: single-k truss by count-and-delete passes (undirected capped counts; tiled
// counts); edge states in e->rnd, so emit_keep applies.  Synchronous (one read per pass).
int ktruss_undirected(kt_engine* e, uint32_t k, bool recount_all, uint32_t group);
int ktruss_tiled(kt_engine* e, uint32_t k, bool recount_all, bool capped);

}  // namespace kt
