/*
 * ktruss_gb300.h — C ABI of libktruss_gb300, a GB300 (sm_103a) k-truss engine that drops in
 * for KTrussExplorer's k-truss path.
 *
 * Every entry point takes plain pointers and sizes and returns an int status (kt_status).
 * The last error message of the calling thread is available from kt_last_error().
 *
 * Reference interfaces replaced (paths are inside the ktruss-explorer project):
 *   kt_ktruss            <- void ktruss(COOGraph* graph, COOGraph* truss, Config config)
 *                           kernel.h:12, kernel.cu:9-39 (dispatch, relabel, GPU/CPU drivers)
 *   kt_verify            <- void verify(COOGraph* graph, Config config)         verify.cu:12-40
 *   kt_read_tsv          <- COOGraph* createCOOFromFile(const char* fileName)  graph.cu:37-79
 *   kt_write_tsv         <- void writeCOOGraphToFile(COOGraph*, const char*)   graph.cu:96-104
 *   kt_coo_alloc/free    <- createEmptyCOO / freeCOOGraph                       graph.cu:10-18, 81-85
 *   kt_config_default,
 *   kt_parse_args        <- Config parseArgs(int, char**)                       config.h:183-224
 *   kt_print_config,
 *   kt_print_config_csv  <- printConfig / printConfigAsCSV                      config.h:226-272
 * New (no counterpart in the reference, which computes one k per run):
 *   kt_decompose         per-edge truss numbers and k_max in one call (the reference obtains
 *                        them only by chaining ktruss() over k = 3, 4, ...)
 *   kt_engine_*          device-resident engine: persistent workspace, caller-owned device
 *                        buffers, one CUDA stream
 *   kt_gen_*             seeded synthetic graph generators
 */
#ifndef KTRUSS_GB300_H
#define KTRUSS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------------------- */
/* The reference reports errors by assert() or exit(0); each assert becomes a status here. */
typedef enum kt_status {
    KT_OK = 0,
    KT_ERR_INVALID_ARG = 1,     /* null pointer, bad enum value, bad size                     */
    KT_ERR_SELF_LOOP = 2,       /* graph.cu:54 "Edges from a vertex to itself are not allowed" */
    KT_ERR_NOT_SYMMETRIC = 3,   /* an entry (u,v) without its reverse (v,u), or a duplicate    */
    KT_ERR_CAPACITY = 4,        /* output capacity below the edge count (graph.cu:111,122)     */
    KT_ERR_UNSUPPORTED = 5,     /* processor=cpu: this library implements the GPU path only    */
    KT_ERR_CUDA = 6,            /* a CUDA runtime call failed                                   */
    KT_ERR_DEVICE_ALLOC = 7,    /* device memory exhausted                                     */
    KT_ERR_HOST_ALLOC = 8,
    KT_ERR_IO = 9,              /* file cannot be opened or parsed (graph.cu:47,52-53)          */
    KT_ERR_MISMATCH = 10,       /* verify: edge count or edge set differs (verify.cu:18,28-29)  */
    KT_ERR_TIMEOUT = 11,        /* a bounded device-side wait expired; the device stays usable */
    KT_ERR_NO_DEVICE = 12,
    KT_ERR_TOO_LARGE = 13,      /* graph exceeds the 32-bit index space of the layout          */
    KT_ERR_INTERNAL = 14        /* a device-side consistency bound was exceeded (a bug)        */
} kt_status;

/* ---- graph and configuration structs -------------------------------------------------- */

/* Same field order and types as COOGraph (graph.h:10-16).  An undirected graph stores each
 * edge twice, once per direction; num_edges counts both.  Vertex ids are 0-based. */
typedef struct kt_coo {
    uint32_t num_nodes;
    uint32_t num_edges;
    uint32_t capacity;
    uint32_t* src_idx;
    uint32_t* dst_idx;
} kt_coo;

/* Enum values of config.h:51-161. */
enum { KT_PROCESSOR_CPU = 0, KT_PROCESSOR_GPU = 1 };
enum { KT_UNDIRECTED = 0, KT_DIRECTED_BY_INDEX = 1, KT_DIRECTED_BY_DEGREE = 2 };
enum { KT_FORMAT_COOCSR = 0, KT_FORMAT_TILED_COOCSR = 1 };
enum { KT_RECOUNT_ALL = 0, KT_RECOUNT_AFFECTED = 1 };

/* Same field order as Config (config.h:163-181); the four enums are int32. */
typedef struct kt_config {
    const char* graph_file_name;
    uint32_t k;
    const char* compare_file_name;
    const char* out_file_name;
    uint32_t num_warmup_runs;
    uint32_t num_timed_runs;
    int32_t processor;
    int32_t directedness;
    int32_t input_format;
    uint32_t num_edge_remove_iter;
    int32_t recount;
    uint32_t block_size;
    uint32_t num_tiles;
    uint32_t num_parallel_tiles;
    uint32_t verbosity;
    uint32_t num_nodes; /* filled from the graph by the caller, as main.cu:23-24 does */
    uint32_t num_edges;
} kt_config;

/* Canonical undirected edge list (u < v, sorted, no duplicates), returned by generators. */
typedef struct kt_edges {
    uint32_t num_nodes;
    uint64_t num_edges;
    uint32_t* u;
    uint32_t* v;
} kt_edges;

/* ---- errors ---------------------------------------------------------------------------- */
const char* kt_last_error(void);
const char* kt_status_string(int status);

/* ---- configuration (config.h) --------------------------------------------------------- */
/* Defaults of parseArgs (config.h:184-199). */
void kt_config_default(kt_config* config);
/* getopt string "g:k:o:w:x:c:p:d:f:e:r:b:t:y:v:h" (config.h:201).  Returns KT_OK, or
 * KT_ERR_INVALID_ARG for an unknown option or enum value (the reference exits with status 0
 * there, config.h:62-63).  -h prints the usage text and returns KT_ERR_INVALID_ARG too. */
int kt_parse_args(int argc, char** argv, kt_config* config);
void kt_print_usage(void);
void kt_print_config(const kt_config* config);
void kt_print_config_csv(const kt_config* config);

/* ---- graph I/O (graph.cu) ------------------------------------------------------------- */
/* Allocates host arrays of `capacity` entries; num_edges = 0. */
int kt_coo_alloc(uint32_t num_nodes, uint32_t capacity, kt_coo* out);
void kt_coo_free(kt_coo* graph);
/* Reads "dst src x" lines, 1-based ids (graph.cu:51-62); num_nodes = largest id seen. */
int kt_read_tsv(const char* path, kt_coo* out);
/* Writes "dst+1 \t src+1 \t 1" per entry (graph.cu:96-104). */
int kt_write_tsv(const kt_coo* graph, const char* path);
/* Decomposition output: "dst+1 \t src+1 \t t(e)" per entry; readers of the reference format
 * ignore the third column (graph.cu:53). */
int kt_write_truss_tsv(const kt_coo* graph, const uint32_t* truss_per_entry, const char* path);

/* ---- the k-truss path ----------------------------------------------------------------- */
/* k-truss of `graph` for config->k (kernel.h:12).  `graph` holds a symmetric simple graph
 * (both directions, no self loops, no duplicates).  On return `truss` holds the edges of the
 * k-truss in both directions with the input's vertex ids, in unspecified order, and
 * truss->num_nodes = graph->num_nodes.  truss->capacity must be >= graph->num_edges.
 * Semantics follow the reference: k = 2 keeps every edge; k < 2 keeps none (k-2 wraps as an
 * unsigned value).  config->directedness, input_format, recount, num_edge_remove_iter,
 * block_size, num_tiles and num_parallel_tiles select the GPU schedule; the edge set returned
 * does not depend on them.  num_warmup_runs/num_timed_runs repeat the computation and, at
 * verbosity 0, print the config.h:247-272 CSV line with the time of each timed run.
 * Unlike the reference, `graph` is not relabeled in place.  processor = CPU returns
 * KT_ERR_UNSUPPORTED. */
int kt_ktruss(const kt_coo* graph, kt_coo* truss, const kt_config* config);

/* Full decomposition: truss_per_entry[i] = t(e) of the edge of entry i (same value for both
 * directions), where t(e) = max k such that e is in the k-truss (>= 2).  *k_max = max t(e)
 * (0 for a graph without edges).  config may be NULL (defaults). */
int kt_decompose(const kt_coo* graph, uint32_t* truss_per_entry, uint32_t* k_max,
                 const kt_config* config);

/* verify.cu:12-40: reads config->compare_file_name and compares edge sets (order-insensitive).
 * Returns KT_ERR_MISMATCH instead of aborting; prints "    PASSED" at verbosity >= 1. */
int kt_verify(const kt_coo* truss, const kt_config* config);

/* ---- device-resident engine ----------------------------------------------------------- */
typedef struct kt_engine kt_engine;

/* Statistics of the last engine call (filled by kt_engine_stats). */
typedef struct kt_stats {
    uint32_t num_nodes;          /* vertices of the built graph                              */
    uint64_t num_edges;          /* undirected edges m (= oriented edges E+)                 */
    uint32_t k_max;
    uint32_t num_levels;         /* peel levels that removed at least one edge               */
    uint32_t num_rounds;         /* peel rounds (frontier batches) executed                  */
    uint64_t triangles;          /* triangles of the input graph                             */
    uint64_t plain_alive_sum;    /* sum over the passes of the reference's full-recount
                                    schedule of the alive oriented edges E+_p                  */
    uint32_t plain_passes;       /* number of such passes                                    */
    uint64_t kernel_launches;    /* kernels launched by the engine since creation            */
    float last_ms;               /* device time of the last call (CUDA events)               */
    float build_ms;              /* of which: device CSR build (relabel, sort, orient)        */
    float support_ms;            /*           support count                                   */
    float peel_ms;               /*           peeling and output                              */
    uint32_t compactions;        /* in-place compactions of the adjacency rows while peeling   */
    float peel_phase_ms[6];      /* peel kernel time by phase (init, level scan, frontier
                                    collection, row compaction, mark, process), barrier to
                                    barrier, as seen by its first block                        */
    float peel_kernel_ms;        /* CUDA-event time of the peel kernel launch alone            */
    float select_ms;             /* learned selector: statistics, features and inference, one
                                    launch (0 without a selector); part of last_ms             */
    uint64_t walk_entries;       /* adjacency entries in the rows of all queued edges: the
                                    decrement work (a round that recounts instead does not walk
                                    its queued rows)                                          */
    float copy_in_ms;            /* host-buffer calls (kt_decompose, kt_decompose_batch): device
                                    time of the input copies host -> device                   */
    float copy_out_ms;           /*   and of the output copies device -> host (plus the emit
                                    of per-graph k_max in a batch)                            */
    float emit_ms;               /* decompositions: of peel_ms, the per-entry output (truss
                                    numbers and k_max) after the peel; 0 for other calls       */
} kt_stats;

/* Schedule of the engine's kernels (no counterpart in the reference, whose tuning knobs are the
 * -b/-t block and tile sizes).  Every schedule gives the same result; only the time differs. */
typedef struct kt_schedule {
    uint32_t support_group;    /* support count: lanes per oriented edge (4, 8, 16 or 32), or 0
                                  for the vertex-centric count with shared-memory hash tables   */
    uint32_t chunk_width;      /* row entries per peel work chunk (lanes per chunk): 8, 16 or 32  */
    uint32_t compact_percent;  /* compact the adjacency rows at a level start once the alive
                                  edges are below this percentage of the count at the last
                                  compaction: 1..99, or 0 = never                                */
    uint32_t recount_percent;  /* a peel round whose frontier holds at least this percentage of
                                  the alive edges removes it at once and recounts the support of
                                  the surviving edges from scratch (the reference's full
                                  recount) instead of decrementing it per destroyed triangle
                                  (its affected-edge recount, made exact): 1..100, or 0 = never */
    uint32_t peel_blocks;      /* peel kernel blocks per SM: 1 (64 registers a thread), 2 (32
                                  registers, twice the warps: hides DRAM latency once the graph
                                  outgrows L2), or 0 = 2 when the oriented CSR of a single graph
                                  exceeds L2, else 1 (batches: 1)                                 */
} kt_schedule;

/* The default schedule {8, 32, 85, 50, 0}. */
kt_schedule kt_schedule_default(void);

/* Creates an engine on `device` with its own non-blocking CUDA stream. */
int kt_engine_create(int device, kt_engine** out);
int kt_engine_destroy(kt_engine* engine);
/* Returns the engine's cudaStream_t (as void*). */
void* kt_engine_stream(kt_engine* engine);
/* Pre-allocates the device workspace for graphs up to these sizes, so that later calls of at
 * most this size do not allocate. */
int kt_engine_reserve(kt_engine* engine, uint32_t max_nodes, uint64_t max_entries);
/* Device-resident decomposition.  d_src/d_dst: num_entries entries on the engine's device
 * (symmetric simple graph, both directions).  d_truss_per_entry: num_entries outputs.
 * d_k_max: one uint32 on the device.  Work is enqueued on the engine stream; the call
 * returns once it is enqueued unless `sync` is nonzero. */
int kt_engine_decompose(kt_engine* engine, const uint32_t* d_src, const uint32_t* d_dst,
                        uint64_t num_entries, uint32_t num_nodes, uint32_t* d_truss_per_entry,
                        uint32_t* d_k_max, int sync);
/* The reference's variant switches for single-k truss calls (config.h:51-161; -d, -f, -r, -b, -t,
 * -y): every variant gives the same k-truss.  directedness KT_DIRECTED_BY_DEGREE (default) or
 * KT_DIRECTED_BY_INDEX orients edges from lower to higher degree rank or vertex id and runs the
 * engine's peel; recount KT_RECOUNT_ALL lets rounds that remove a large share of the edges recount
 * all survivors (the schedule's recount_percent), KT_RECOUNT_AFFECTED updates only the triangles
 * of removed edges (support decrements in every round).  KT_UNDIRECTED runs count-and-delete
 * passes over the symmetric rows with counts capped at k-2 (the reference's undirected variant;
 * with KT_RECOUNT_AFFECTED a pass recounts only edges next to the previous pass's deletions).
 * input_format KT_FORMAT_TILED_COOCSR counts support over the tiled COO/CSR layout (num_tiles x
 * num_tiles tiles, num_parallel_tiles column tiles of one edge processed in parallel) in recount
 * passes.  block_size: threads per block of the variant passes' kernels (the reference's -b). */
typedef struct kt_variant {
    int32_t directedness;
    int32_t input_format;
    int32_t recount;
    uint32_t block_size;
    uint32_t num_tiles;
    uint32_t num_parallel_tiles;
} kt_variant;
kt_variant kt_variant_default(void);
/* The variant of the engine's later kt_engine_ktruss calls (decompositions ignore it). */
int kt_engine_set_variant(kt_engine* engine, const kt_variant* variant);
int kt_engine_get_variant(kt_engine* engine, kt_variant* variant);
/* Device-resident single-k truss: d_keep[i] = 1 if entry i's edge is in the k-truss, else 0. */
int kt_engine_ktruss(kt_engine* engine, const uint32_t* d_src, const uint32_t* d_dst,
                     uint64_t num_entries, uint32_t num_nodes, uint32_t k, uint8_t* d_keep,
                     int sync);
/* Repeats the engine's last successful kt_engine_decompose or kt_engine_ktruss call on the same
 * device buffers, whose contents the caller has left unchanged: the reference's repeat runs
 * (-w/-x, kernel_ddc.cu:227-244), which rebuild the graph and run the whole k-truss again.  The
 * first replay captures the call's device pipeline (build, support count, peel, output) into a
 * CUDA graph without the input checks the call already made; later replays launch that graph.
 * A different call, a new schedule or selector, or a larger reservation drops the graph.
 * Statistics afterwards: everything but the per-phase times (0); last_ms is the replay's. */
int kt_engine_replay(kt_engine* engine, int sync);
/* How the next replay runs: 0 nothing to replay yet or not captured yet, 1 one launch of the
 * captured CUDA graph, 2 direct launches (the capture was refused). */
int kt_engine_replay_mode(const kt_engine* engine);
/* Batched decomposition (no counterpart in the reference): num_graphs graphs in one call, given
 * as one COO over disjoint vertex ranges — graph g owns vertices [d_vertex_offsets[g],
 * d_vertex_offsets[g+1]), num_graphs+1 offsets ending at num_nodes, and every entry stays inside
 * one graph (else KT_ERR_INVALID_ARG).  The batch runs as one graph: one build, one support
 * count and one persistent peel launch whose work chunks mix all graphs.  Outputs per entry as
 * in kt_engine_decompose, and d_k_max_per_graph[g] (0 for a graph without edges). */
int kt_engine_decompose_batch(kt_engine* engine, const uint32_t* d_src, const uint32_t* d_dst,
                              uint64_t num_entries, uint32_t num_nodes, const uint32_t* d_vertex_offsets,
                              uint32_t num_graphs, uint32_t* d_truss_per_entry, uint32_t* d_k_max_per_graph,
                              int sync);
/* The same with host buffers (copied to and from the device in the call). */
int kt_decompose_batch(const uint32_t* src, const uint32_t* dst, uint64_t num_entries, uint32_t num_nodes,
                       const uint32_t* vertex_offsets, uint32_t num_graphs, uint32_t* truss_per_entry,
                       uint32_t* k_max_per_graph);
/* Synchronizes the engine stream and fills *stats.  Returns KT_ERR_TIMEOUT if the last peel
 * kernel gave up on a grid barrier. */
int kt_engine_stats(kt_engine* engine, kt_stats* stats);
/* Per-round log of the last decomposition or single-k call: for each of the first `cap`
 * peel rounds, the frontier size, the level k and the device time in nanoseconds (any
 * pointer may be NULL).  *num_rounds receives the number of rounds run. */
int kt_engine_round_log(kt_engine* engine, uint32_t* size, uint32_t* level, uint32_t* ns, uint32_t cap,
                        uint32_t* num_rounds);
/* Per-level log of the last call: for each of the first `cap` peel levels, k, the alive edges at
 * its start, the device time of its start (alive-edge scan and first frontier) in nanoseconds,
 * and the size of its first frontier (any pointer may be NULL). */
int kt_engine_level_log(kt_engine* engine, uint32_t* k, uint32_t* alive, uint32_t* ns, uint32_t* frontier,
                        uint32_t cap, uint32_t* num_levels);
/* Sets the schedule of the engine's later calls (KT_ERR_INVALID_ARG for a value outside the
 * ranges above); kt_engine_get_schedule reads it. */
int kt_engine_set_schedule(kt_engine* engine, const kt_schedule* schedule);
int kt_engine_get_schedule(kt_engine* engine, kt_schedule* schedule);

/* Wait limit of the peel kernel's grid barriers (no counterpart in the reference, whose loop is
 * driven from the host): every wait is bounded by base_ns plus ns_per_unit for each unit of work
 * the wait can legitimately cover - each row entry slot of the work chunks queued for the round
 * that the barrier closes (row entries rounded up to whole chunks),
 * each edge (twice) for a level phase - after which the kernel returns KT_ERR_TIMEOUT instead of
 * waiting forever.  Defaults: 10 s and 8 ns.  base_ns must be at least 1 microsecond. */
int kt_engine_set_wait_limit(kt_engine* engine, uint64_t base_ns, uint32_t ns_per_unit);
int kt_engine_get_wait_limit(kt_engine* engine, uint64_t* base_ns, uint32_t* ns_per_unit);
/* Statistics of the last call of the host-buffer entry points (kt_ktruss, kt_decompose,
 * kt_decompose_batch), including the device time of their copies (copy_in_ms, copy_out_ms). */
int kt_last_stats(kt_stats* stats);
/* Schedule of the engine behind the host-buffer entry points (kt_ktruss, kt_decompose,
 * kt_decompose_batch). */
int kt_set_schedule(const kt_schedule* schedule);
int kt_get_schedule(kt_schedule* schedule);
/* The autotuner's built-in grid of schedules: support_group {4, 8, 16} x chunk_width
 * {8, 16, 32} x compact_percent {0, 85} x recount_percent {0, 50}, peel_blocks 0 (36).  Writes
 * min(36, cap) schedules to `out` (may be NULL) and returns 36. */
uint32_t kt_schedule_grid(kt_schedule* out, uint32_t cap);
/* Autotuner (no counterpart in the reference).  Decomposes the given device graph once per
 * candidate schedule and `repeats` times each
 * (>= 1), and keeps the candidate with the least device time of support count plus peel (CUDA
 * events; the CSR build does not depend on the schedule).  candidates: num_candidates schedules,
 * or NULL for the built-in grid.  ms (optional): the least time of each candidate.  On return the
 * engine runs with the fastest schedule, also written to *best (optional).  Callers tune on a
 * sample of the graphs they will run and reuse the schedule for the rest. */
int kt_engine_autotune(kt_engine* engine, const uint32_t* d_src, const uint32_t* d_dst, uint64_t num_entries,
                       uint32_t num_nodes, const kt_schedule* candidates, uint32_t num_candidates,
                       uint32_t repeats, float* ms, kt_schedule* best);
/* The same for batches: times each candidate the way kt_engine_decompose_batch runs it, on the
 * union of a sample batch's graphs (d_src/d_dst/num_nodes as for that call).  A batch's peel
 * always runs one block per SM, while a single graph of the same size whose oriented CSR outgrows
 * L2 runs two (peel_blocks 0), so tuning a large union as one graph measures another kernel. */
int kt_engine_autotune_batch(kt_engine* engine, const uint32_t* d_src, const uint32_t* d_dst,
                             uint64_t num_entries, uint32_t num_nodes, const kt_schedule* candidates,
                             uint32_t num_candidates, uint32_t repeats, float* ms, kt_schedule* best);
/* ---- symmetrize and deduplicate ----------------------------------------------------------
 * Turns an arbitrary entry list on the device (one or both directions, duplicates, self loops)
 * into the symmetric simple graph the k-truss calls take: each undirected edge {u, v}, u != v,
 * once as (min, max) in sorted order at positions [0, u), then reversed at [u, 2u).  *num_out =
 * 2u; KT_ERR_CAPACITY (nothing written) if 2u > capacity; KT_ERR_INVALID_ARG for an id >=
 * num_nodes.  The reference's reader requires files that already list both directions
 * (graph.cu:37-79); this is the device-side sort and dedup for inputs that do not.  Synchronous. */
int kt_engine_symmetrize(kt_engine* engine, const uint32_t* d_src, const uint32_t* d_dst, uint64_t num_entries,
                         uint32_t num_nodes, uint32_t* d_src_out, uint32_t* d_dst_out, uint64_t capacity,
                         uint64_t* num_out);

/* ---- tiled COO/CSR layout (coo2tiledcoocsr, graph.cu:641-706) ---------------------------
 * The reference's tiled layout of an entry list, built on the device: tile_size =
 * ceil(num_nodes / tiles_per_dim); entry (s, d) lies in row (s / tile_size * tiles_per_dim +
 * d / tile_size) * tile_size + s % tile_size; d_tile_src_ptr receives tiles_per_dim^2 * tile_size
 * + 1 row offsets, d_src_out / d_dst_out the entries ordered by row and, within a row, by
 * destination.  The engine's own kernels do not read tiles; this serves callers of the reference's
 * tiled format.  Synchronous. */
int kt_engine_tiled_coocsr(kt_engine* engine, const uint32_t* d_src, const uint32_t* d_dst, uint64_t num_entries,
                           uint32_t num_nodes, uint32_t tiles_per_dim, uint32_t* d_tile_src_ptr, uint32_t* d_src_out,
                           uint32_t* d_dst_out);

/* ---- device-side TSV ingest (replaces createCOOFromFile, graph.cu:37-79) ------------------
 * The same format as kt_read_tsv - "dst src x" triples of unsigned decimal numbers separated by
 * any whitespace, 1-based ids, x ignored - parsed on the device into 0-based entries in the
 * caller's device buffers (entry i: d_src[i] = src-1, d_dst[i] = dst-1, in file order).
 * *num_nodes = the largest id.  Statuses as kt_read_tsv (KT_ERR_IO for a malformed text, a 0
 * id or an incomplete triple, KT_ERR_SELF_LOOP), and KT_ERR_CAPACITY when the text holds more
 * than `capacity` entries (nothing is written then). */
int kt_engine_parse_tsv(kt_engine* engine, const char* d_text, uint64_t bytes, uint32_t* d_src, uint32_t* d_dst,
                        uint64_t capacity, uint64_t* num_entries, uint32_t* num_nodes);
/* The same for a file: its bytes are copied to the device (pinned staging) and parsed there. */
int kt_engine_read_tsv(kt_engine* engine, const char* path, uint32_t* d_src, uint32_t* d_dst, uint64_t capacity,
                       uint64_t* num_entries, uint32_t* num_nodes);

/* ---- learned schedule selector (no counterpart in the reference) ------------------------
 * A small MLP (16 -> 64 -> 64 -> 19, ReLU, FP32, hand-written CUDA kernels for inference,
 * training and Adam) that reads 16 statistics of a built graph and predicts its schedule from
 * the autotuner's grid: the variant (support_group x chunk_width x compact_percent, 18 classes)
 * and the recount switch (recount_percent 50 or 0).  It is trained on timings of the grid's 36
 * schedules (kt_engine_autotune with ms output) measured on graphs like the ones it will see.
 * Every schedule gives the same truss numbers: a wrong prediction only costs time. */
#define KT_SELECTOR_FEATURES 16
#define KT_SELECTOR_VARIANTS 18
#define KT_SELECTOR_SCHEDULES 36
#define KT_SELECTOR_PARAMS 6483
typedef struct kt_selector kt_selector;
/* A selector on `device` with seeded He-uniform weights and identity standardization. */
int kt_selector_create(int device, uint64_t seed, kt_selector** out);
int kt_selector_destroy(kt_selector* selector);
/* Parameters (KT_SELECTOR_PARAMS floats: W1[64][16], b1[64], W2[64][64], b2[64], W3[19][64],
 * b3[19]) and the input standardization (mean, scale: 16 floats each); any pointer may be NULL. */
int kt_selector_get_params(kt_selector* selector, float* params, float* mean, float* scale);
int kt_selector_set_params(kt_selector* selector, const float* params, const float* mean, const float* scale);
/* Trains on n graphs: features (n x 16, as kt_engine_features gives them) and times (n x 36 ms in
 * kt_schedule_grid order).  Sets the standardization from these features, then runs `epochs` of
 * Adam (learning rate lr) over minibatches of `batch` graphs in a seeded order.  Loss per graph:
 * softmax cross-entropy of the best variant plus the logistic loss of the recount switch.
 * epoch_loss (optional): mean loss of each epoch. */
int kt_selector_train(kt_selector* selector, const float* features, const float* times, uint32_t n, uint32_t epochs,
                      uint32_t batch, float lr, uint64_t seed, float* epoch_loss);
/* Mean loss and its gradient (KT_SELECTOR_PARAMS floats, optional) over all n graphs at the
 * current parameters and standardization. */
int kt_selector_gradient(kt_selector* selector, const float* features, const float* times, uint32_t n, float* grad,
                         float* loss);
/* Predicted schedules of n graphs from their features. */
int kt_selector_predict(kt_selector* selector, const float* features, uint32_t n, kt_schedule* out);
/* Builds the graph and returns its 16 features (computed on the device). */
int kt_engine_features(kt_engine* engine, const uint32_t* d_src, const uint32_t* d_dst, uint64_t num_entries,
                       uint32_t num_nodes, float* features);
/* With a selector attached, every decomposition (single graph or batch) computes the features
 * of the built graph and runs the network on the device; the support count and the peel read the
 * chosen schedule from device memory, so the call enqueues its whole pipeline without waiting
 * (kt_engine_get_schedule and the statistics report the choice once the call has finished).  NULL
 * detaches it; the engine keeps the last schedule it reported. */
int kt_engine_set_selector(kt_engine* engine, kt_selector* selector);

/* Self-test of the bounded device waits: launches a grid barrier that one block never reaches,
 * with a wait limit of timeout_ns (at most 5 s).  Returns KT_ERR_TIMEOUT when the wait expired
 * and the kernel returned as designed; the engine stays usable afterwards. */
int kt_engine_selftest_barrier_timeout(kt_engine* engine, uint64_t timeout_ns);

/* Decomposition that allocates nothing (no counterpart in the reference).  For callers that
 * cannot let a library allocate device memory: programs whose device memory is owned by one
 * memory manager with a fixed budget, and latency-sensitive loops that cannot afford
 * cudaMalloc/cudaFree (which may synchronize the device).  Same inputs and outputs as
 * kt_engine_decompose on the current device and `stream` (a cudaStream_t, NULL = default stream);
 * all scratch lives in a 40 MiB static device array, held on every GPU where it is loaded until
 * the process exits.  CUDA loads modules lazily by default, so the array is usually backed at the
 * first call on a device (at context creation under CUDA_MODULE_LOADING=EAGER): that first call
 * can fail with a CUDA error when device memory is short; later calls allocate nothing.  Limits:
 * at most 524,288 entries (262,144 undirected edges) and 131,072 vertices, else
 * KT_ERR_TOO_LARGE.  The first call on a device sets the array up and should happen before any
 * stream capture.  Calls on a device share the array; they are serialized, and each call
 * synchronizes `stream` before it returns (overlapping work would race). */
int kt_decompose_noalloc(const uint32_t* d_src, const uint32_t* d_dst, uint64_t num_entries,
                         uint32_t num_nodes, uint32_t* d_truss_per_entry, uint32_t* d_k_max,
                         void* stream);

/* ---- seeded generators (no counterpart in the reference, which ships no data) --------- */
int kt_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c,
                uint64_t seed, kt_edges* out);
int kt_gen_er(uint32_t n, double p, uint64_t seed, kt_edges* out);
int kt_gen_ba(uint32_t n, uint32_t m, uint64_t seed, kt_edges* out);
int kt_gen_ws(uint32_t n, uint32_t k, double p, uint64_t seed, kt_edges* out);
int kt_gen_rgg(uint32_t n, double radius, uint64_t seed, kt_edges* out);
/* Adds `count` cliques of min_size..max_size random distinct vertices to the edge list
 * (u[i], v[i]) of a graph with num_nodes vertices; the result is canonical again. */
int kt_plant_cliques(uint32_t num_nodes, const uint32_t* u, const uint32_t* v, uint64_t num_edges,
                     uint32_t count, uint32_t min_size, uint32_t max_size, uint64_t seed, kt_edges* out);
/* A batch of num_graphs graphs as one edge list over disjoint vertex ranges: graph g owns
 * vertices [vertex_offsets[g], vertex_offsets[g+1]) (num_graphs+1 offsets written).  Sizes are
 * log-uniform in [n_min, n_max]; even graphs Barabasi-Albert (m in {2,4,8,16}), odd graphs
 * Watts-Strogatz (k in {6,10,20}, p = 0.1), each with 0-3 planted cliques of 8-64 vertices. */
int kt_gen_batch(uint32_t num_graphs, uint32_t n_min, uint32_t n_max, uint64_t seed, kt_edges* out,
                 uint32_t* vertex_offsets);
void kt_edges_free(kt_edges* graph);

#ifdef __cplusplus
}
#endif

#endif /* KTRUSS_GB300_H */
