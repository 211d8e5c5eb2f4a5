/*
 * ktruss_oracle.h — TEST INFRASTRUCTURE ONLY (the checker, never the product).
 *
 * A plain-C restatement of KTrussExplorer's CPU (Host) k-truss path, used by tests/,
 * by __graft_entry__.smoke() and by bench.py's CPU-baseline leg to check and time the
 * GPU engine.  Nothing in the product library links, loads or calls this code.
 *
 * Parity is pinned by tests/golden/: fixtures produced by running the reference's own
 * `ktruss -p cpu` executable (built from its sources by `make -C oracle ref`) on seeded
 * graphs, chained over k as described in ko_decompose_chain.
 *
 * Graph convention (graph.h:10-16): `num_entries` COO entries (src[i], dst[i]), 0-based,
 * an undirected edge stored once per direction.
 */
#ifndef KTRUSS_ORACLE_H
#define KTRUSS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { KO_UNDIRECTED = 0, KO_DIRECTED_BY_INDEX = 1, KO_DIRECTED_BY_DEGREE = 2 };
enum { KO_RECOUNT_ALL = 0, KO_RECOUNT_AFFECTED = 1 };

/* Optional per-pass log of the reference loop: alive oriented edges at the start of each
 * pass (count-and-prune iteration).  `cap` entries of `alive`; *num receives the pass count
 * (which may exceed cap; only the first cap are stored). */
typedef struct ko_pass_log {
    uint32_t cap;
    uint32_t num;
    uint64_t* alive;
    double loop_seconds; /* wall time of the count-and-prune loop alone: the span the reference's
                            k-truss timer covers (kernel_hdc.cu:213-229), without relabel and CSR build */
} ko_pass_log;

/* Per-level pass statistics of the reference chain, indexed by k: passes[k] count-and-prune
 * passes of the single-k run at k (on the (k-1)-truss), alive[k] the sum of their alive oriented
 * edge counts.  num = largest stored k + 1. */
typedef struct ko_level_log {
    uint32_t cap;
    uint32_t num;
    uint32_t* passes;
    uint64_t* alive;
} ko_level_log;

/* Single-k k-truss (kernel.cu:9-39 -> kernel_h.cu:11-68 -> kernel_h{d,u}c.cu).
 * Writes the surviving edges in both directions to out_src/out_dst (capacity num_entries)
 * and their count to *out_num.  Returns 0, or -1 on an allocation failure. */
int ko_ktruss(uint32_t num_nodes, uint32_t num_entries, const uint32_t* src, const uint32_t* dst,
              uint32_t k, int directedness, int recount, uint32_t num_edge_remove_iter,
              uint32_t* out_src, uint32_t* out_dst, uint32_t* out_num, ko_pass_log* log);

/* Decomposition by chaining single-k runs: k = 3, 4, ... each on the previous output,
 * directed-by-degree, recount all, until the output is empty.  truss_per_entry[i] = the
 * largest k whose output contains entry i's edge (2 if none).  *k_max = the largest such
 * k over all entries (0 without edges).  *plain_passes / *plain_alive_sum: number of
 * count-and-prune passes over all runs and the sum of their alive oriented edge counts. */
int ko_decompose_chain(uint32_t num_nodes, uint32_t num_entries, const uint32_t* src,
                       const uint32_t* dst, uint32_t* truss_per_entry, uint32_t* k_max,
                       uint32_t* plain_passes, uint64_t* plain_alive_sum);

/* Bounded sample of ko_decompose_chain for CPU timing: runs the chain's count-and-prune passes
 * in order and stops once `budget_s` seconds have passed (at a pass boundary, or inside a
 * pass's triangle count).  Reports the complete passes, the alive oriented edges they visited
 * plus those the cut count had merged, and the elapsed seconds. */
int ko_chain_sample(uint32_t num_nodes, uint32_t num_entries, const uint32_t* src, const uint32_t* dst,
                    double budget_s, uint32_t* passes_done, uint64_t* alive_done, double* seconds);

/* The same decomposition by serial peeling with exact support decrements (much faster;
 * checked against ko_decompose_chain).  Same outputs; also the number of peel rounds. */
int ko_decompose_peel(uint32_t num_nodes, uint32_t num_entries, const uint32_t* src,
                      const uint32_t* dst, uint32_t* truss_per_entry, uint32_t* k_max,
                      uint32_t* plain_passes, uint64_t* plain_alive_sum, uint32_t* num_rounds);

/* ko_decompose_peel with the per-level pass statistics of the reference chain (levels may be
 * NULL). */
int ko_decompose_peel_levels(uint32_t num_nodes, uint32_t num_entries, const uint32_t* src,
                             const uint32_t* dst, uint32_t* truss_per_entry, uint32_t* k_max,
                             uint32_t* plain_passes, uint64_t* plain_alive_sum, uint32_t* num_rounds,
                             ko_level_log* levels);

/* ko_decompose_peel_levels with its phases split over `threads` host threads: the same outputs
 * (the rounds are the same synchronous rounds; only the work inside each is shared). */
int ko_decompose_peel_mt(uint32_t num_nodes, uint32_t num_entries, const uint32_t* src,
                         const uint32_t* dst, uint32_t* truss_per_entry, uint32_t* k_max,
                         uint32_t* plain_passes, uint64_t* plain_alive_sum, uint32_t* num_rounds,
                         ko_level_log* levels, uint32_t threads);

/* Repeat runs of the reference's single-k loop (default variant: directed by degree, recount all,
 * no compaction) with its count and mark sweeps split over `threads` host threads: relabel,
 * orientation and CSR once; each of `runs` runs restores the CSR and times the count-and-prune
 * loop alone (run_seconds[i], run_passes[i]).  Writes the last run's truss edges (both
 * directions) like ko_ktruss.  Returns 0, or -1 on an allocation failure. */
int ko_ktruss_runs(uint32_t num_nodes, uint32_t num_entries, const uint32_t* src, const uint32_t* dst,
                   uint32_t k, uint32_t runs, uint32_t threads, uint32_t* out_src, uint32_t* out_dst,
                   uint32_t* out_num, double* run_seconds, uint32_t* run_passes);

/* R-MAT generator: the same graph as the engine's kt_gen_rmat for the same arguments (a
 * restatement of that seeded generator, so that the CPU baseline makes its input without the
 * product library).  Writes the canonical edges u < v sorted by (u, v), without duplicates or
 * self loops, into u/v (capacity edge_factor << scale) and their count to *num_edges.
 * Returns 0, or -1 on bad arguments or an allocation failure. */
int ko_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
                uint32_t* u, uint32_t* v, uint64_t* num_edges);

#ifdef __cplusplus
}
#endif

#endif
