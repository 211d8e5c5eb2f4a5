/*
 * ktruss_oracle.c — TEST INFRASTRUCTURE ONLY (the checker, never the product).
 *
 * Plain-C restatement of KTrussExplorer's CPU k-truss path.  Every function names the
 * reference lines it follows.  Parity of this restatement is pinned by the golden fixtures
 * in tests/golden/ (outputs of the reference's own `ktruss -p cpu` executable).
 *
 * Deliberate difference: sortByDegree (graph.cu:152-185) orders vertices with an unstable
 * quicksort, so ties between equal degrees fall in an arbitrary order; here ties are broken
 * by vertex id.  The k-truss edge set does not depend on the orientation, so outputs agree.
 */
#define _POSIX_C_SOURCE 200809L
#include "ktruss_oracle.h"

#include <stdlib.h>
#include <string.h>
#include <time.h>

#define KO_DELETED 0xffffffffu /* DELETED = UINT_MAX, graph.h:8 */
#define NOT_AFFECTED 0u        /* info.h:10-12 */
#define DIRECTLY_AFFECTED 1u
#define INDIRECTLY_AFFECTED 2u

/* COOCSRGraph (graph.h:40-47) */
typedef struct {
    uint32_t num_nodes, num_edges;
    uint32_t *ptr, *src, *dst;
} csr_t;

static void csr_free(csr_t* g) {
    free(g->ptr);
    free(g->src);
    free(g->dst);
    memset(g, 0, sizeof(*g));
}

static int cmp_u32(const void* a, const void* b) {
    uint32_t x = *(const uint32_t*)a, y = *(const uint32_t*)b;
    return x < y ? -1 : x > y;
}

static int cmp_u64(const void* a, const void* b) {
    uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? -1 : x > y;
}

/* coo2coocsr (graph.cu:372-412): histogram of sources, exclusive scan, binning in entry
 * order, then each row's destinations sorted ascending. */
static int coo2coocsr(uint32_t n, uint32_t m, const uint32_t* s, const uint32_t* d, csr_t* g) {
    g->num_nodes = n;
    g->num_edges = m;
    g->ptr = (uint32_t*)calloc((size_t)n + 1, sizeof(uint32_t));
    g->src = (uint32_t*)malloc(sizeof(uint32_t) * (m ? m : 1));
    g->dst = (uint32_t*)malloc(sizeof(uint32_t) * (m ? m : 1));
    if (!g->ptr || !g->src || !g->dst) { csr_free(g); return -1; }
    for (uint32_t e = 0; e < m; ++e) g->ptr[s[e] + 1]++;
    uint32_t sum = 0;
    for (uint32_t v = 0; v < n; ++v) { uint32_t c = g->ptr[v + 1]; g->ptr[v + 1] = sum; sum += c; }
    for (uint32_t e = 0; e < m; ++e) {
        uint32_t j = g->ptr[s[e] + 1]++;
        g->src[j] = s[e];
        g->dst[j] = d[e];
    }
    for (uint32_t v = 0; v < n; ++v)
        if (g->ptr[v + 1] - g->ptr[v] > 1) qsort(g->dst + g->ptr[v], g->ptr[v + 1] - g->ptr[v], sizeof(uint32_t), cmp_u32);
    return 0;
}

/* removeCOOCSRDeletedEdges (graph.cu:480-509): stable compaction, then row pointers rebuilt
 * by histogram + scan. */
static void remove_deleted(csr_t* g) {
    uint32_t w = 0;
    for (uint32_t e = 0; e < g->num_edges; ++e)
        if (g->dst[e] != KO_DELETED) { g->src[w] = g->src[e]; g->dst[w] = g->dst[e]; ++w; }
    g->num_edges = w;
    memset(g->ptr, 0, sizeof(uint32_t) * ((size_t)g->num_nodes + 1));
    for (uint32_t e = 0; e < w; ++e) g->ptr[g->src[e]]++;
    uint32_t sum = 0;
    for (uint32_t v = 0; v < g->num_nodes; ++v) { uint32_t c = g->ptr[v]; g->ptr[v] = sum; sum += c; }
    g->ptr[g->num_nodes] = sum;
}

typedef struct {
    uint32_t changed;
    uint32_t* num_triangles;
    uint32_t* node_affected;
    uint32_t* edge_affected;
} info_t; /* Info, info.h:14-19 */

/* Optional wall-clock deadline for ko_chain_sample (0 = none); checked between passes and every
 * 4096 edges of a directed count.  When a count is cut, g_cut_alive holds the alive edges it had
 * merged. */
static double g_deadline = 0.0;
static int g_deadline_hit = 0;
static int g_cut_in_count = 0;
static uint64_t g_cut_alive = 0;

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* count_triangles, directed CSR (kernel_hdc.cu:11-49): merge of the two sorted out-lists,
 * each match credits the edge and both other edges of the triangle. */
static void count_directed(csr_t* g, info_t* in, int check_deleted, int recount_all) {
    uint64_t merged = 0;
    for (uint32_t e = 0; e < g->num_edges; ++e) {
        if (g_deadline > 0.0 && (e & 4095u) == 0 && now_s() > g_deadline) {
            g_deadline_hit = 1;
            g_cut_in_count = 1;
            g_cut_alive = merged;
            return;
        }
        if (!(recount_all || in->edge_affected[e] == DIRECTLY_AFFECTED || in->edge_affected[e] == INDIRECTLY_AFFECTED)) continue;
        uint32_t dst = g->dst[e];
        if (check_deleted && dst == KO_DELETED) continue;
        ++merged;
        uint32_t e1 = g->ptr[g->src[e]], end1 = g->ptr[g->src[e] + 1];
        uint32_t e2 = g->ptr[dst], end2 = g->ptr[dst + 1];
        while (e1 < end1 && e2 < end2) {
            uint32_t d1 = g->dst[e1];
            if (check_deleted && d1 == KO_DELETED) { ++e1; continue; }
            uint32_t d2 = g->dst[e2];
            if (check_deleted && d2 == KO_DELETED) { ++e2; continue; }
            if (d1 < d2) ++e1;
            else if (d1 > d2) ++e2;
            else {
                ++in->num_triangles[e];
                ++in->num_triangles[e1];
                ++in->num_triangles[e2];
                ++e1;
                ++e2;
            }
        }
    }
}

/* count_triangles, undirected CSR (kernel_huc.cu:11-49): per-entry intersection, skipped when
 * a list is shorter than k-2, stopped once k-2 triangles are found; only DIRECTLY affected
 * entries are counted in affected mode. */
static void count_undirected(csr_t* g, uint32_t k, info_t* in, int check_deleted, int recount_all) {
    for (uint32_t e = 0; e < g->num_edges; ++e) {
        if (!(recount_all || in->edge_affected[e] == DIRECTLY_AFFECTED)) continue;
        uint32_t dst = g->dst[e];
        if (check_deleted && dst == KO_DELETED) continue;
        uint32_t e1 = g->ptr[g->src[e]], end1 = g->ptr[g->src[e] + 1];
        uint32_t e2 = g->ptr[dst], end2 = g->ptr[dst + 1];
        if (!(end1 - e1 >= k - 2 && end2 - e2 >= k - 2)) continue;
        while (e1 < end1 && e2 < end2 && in->num_triangles[e] < k - 2) {
            uint32_t d1 = g->dst[e1];
            if (check_deleted && d1 == KO_DELETED) { ++e1; continue; }
            uint32_t d2 = g->dst[e2];
            if (check_deleted && d2 == KO_DELETED) { ++e2; continue; }
            if (d1 < d2) ++e1;
            else if (d1 > d2) ++e2;
            else { ++e1; ++e2; ++in->num_triangles[e]; }
        }
    }
}

/* mark_deleted_edges (kernel_hdc.cu:51-70, kernel_huc.cu:51-70): identical in both variants. */
static void mark_deleted(csr_t* g, uint32_t k, info_t* in, int check_deleted, int recount_all) {
    for (uint32_t e = 0; e < g->num_edges; ++e) {
        if (!(recount_all || in->edge_affected[e] == DIRECTLY_AFFECTED)) continue;
        uint32_t dst = g->dst[e];
        if (check_deleted && dst == KO_DELETED) continue;
        if (in->num_triangles[e] < k - 2) { /* unsigned: k < 2 wraps, deleting every edge */
            g->dst[e] = KO_DELETED;
            in->changed = 1;
            if (!recount_all) {
                in->node_affected[g->src[e]] = DIRECTLY_AFFECTED;
                in->node_affected[dst] = DIRECTLY_AFFECTED;
            }
        }
    }
}

/* mark_directly_affected_edges: directed (kernel_hdc.cu:72-90) also promotes the other
 * endpoint to INDIRECTLY affected; undirected (kernel_huc.cu:72-85) does not. */
static void mark_directly(csr_t* g, info_t* in, int check_deleted, int directed) {
    for (uint32_t e = 0; e < g->num_edges; ++e) {
        uint32_t a = NOT_AFFECTED, dst = g->dst[e];
        if (!check_deleted || dst != KO_DELETED) {
            uint32_t src = g->src[e];
            if (in->node_affected[src] == DIRECTLY_AFFECTED || in->node_affected[dst] == DIRECTLY_AFFECTED) {
                a = DIRECTLY_AFFECTED;
                if (directed) {
                    if (in->node_affected[src] != DIRECTLY_AFFECTED) in->node_affected[src] = INDIRECTLY_AFFECTED;
                    else if (in->node_affected[dst] != DIRECTLY_AFFECTED) in->node_affected[dst] = INDIRECTLY_AFFECTED;
                }
            }
        }
        in->edge_affected[e] = a;
    }
}

/* mark_indirectly_affected_edges (kernel_hdc.cu:92-105), directed only. */
static void mark_indirectly(csr_t* g, info_t* in, int check_deleted) {
    for (uint32_t e = 0; e < g->num_edges; ++e) {
        uint32_t dst = g->dst[e];
        if (check_deleted && dst == KO_DELETED) continue;
        if (in->edge_affected[e] == DIRECTLY_AFFECTED) continue;
        if (in->node_affected[g->src[e]] == INDIRECTLY_AFFECTED || in->node_affected[dst] == INDIRECTLY_AFFECTED)
            in->edge_affected[e] = INDIRECTLY_AFFECTED;
    }
}

static uint64_t alive_edges(const csr_t* g) {
    uint64_t c = 0;
    for (uint32_t e = 0; e < g->num_edges; ++e) c += g->dst[e] != KO_DELETED;
    return c;
}

/* The peel loop shared by kernel_hdc.cu:107-201 and kernel_huc.cu:87-179. */
static void peel_loop(csr_t* g, uint32_t k, int directed, int recount, uint32_t num_edge_remove_iter,
                      info_t* in, uint32_t num_slots, ko_pass_log* log) {
    const int all = recount == KO_RECOUNT_ALL;
    uint32_t iter = 0, has_deleted = 0, changed;
    if (!all) /* initInfo (info.cu:71-79): every edge starts DIRECTLY affected */
        for (uint32_t e = 0; e < num_slots; ++e) in->edge_affected[e] = DIRECTLY_AFFECTED;
    if (log) log->num = 0;
    do {
        if (g_deadline > 0.0 && now_s() > g_deadline) { g_deadline_hit = 1; break; }
        /* clearIterInfo (info.cu:96-104) */
        in->changed = 0;
        memset(in->num_triangles, 0, sizeof(uint32_t) * num_slots);
        if (!all) memset(in->node_affected, 0, sizeof(uint32_t) * g->num_nodes);
        if (log) {
            uint64_t a = alive_edges(g);
            if (!directed) a /= 2; /* undirected CSR holds both directions */
            if (log->num < log->cap) log->alive[log->num] = a;
            log->num++;
        }
        if (directed) count_directed(g, in, has_deleted, all);
        else count_undirected(g, k, in, has_deleted, all);
        if (g_deadline_hit) break; /* a count cut by the deadline: the pass is abandoned */
        mark_deleted(g, k, in, has_deleted, all);
        changed = in->changed;
        if (changed) {
            if (iter < num_edge_remove_iter) { remove_deleted(g); has_deleted = 0; }
            else has_deleted = 1;
            if (k == 3) break; /* kernel_hdc.cu:169-172 */
            if (!all) {
                mark_directly(g, in, has_deleted, directed);
                if (directed) mark_indirectly(g, in, has_deleted);
            }
        }
        ++iter;
    } while (changed);
    if (has_deleted) remove_deleted(g);
}

/* sortByDegree (graph.cu:152-185): vertices ordered by ascending out-degree of the
 * symmetric COO (ties by id here), edges relabeled; new2old kept for unsort (graph.cu:187). */
static int sort_by_degree(uint32_t n, uint32_t m, uint32_t* s, uint32_t* d, uint32_t* new2old) {
    uint32_t* deg = (uint32_t*)calloc(n ? n : 1, sizeof(uint32_t));
    uint32_t* old2new = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
    uint32_t maxd = 0;
    if (!deg || !old2new) { free(deg); free(old2new); return -1; }
    for (uint32_t e = 0; e < m; ++e) deg[s[e]]++;
    for (uint32_t v = 0; v < n; ++v) if (deg[v] > maxd) maxd = deg[v];
    uint32_t* cnt = (uint32_t*)calloc((size_t)maxd + 2, sizeof(uint32_t));
    if (!cnt) { free(deg); free(old2new); return -1; }
    for (uint32_t v = 0; v < n; ++v) cnt[deg[v] + 1]++;
    for (uint32_t x = 0; x <= maxd; ++x) cnt[x + 1] += cnt[x];
    for (uint32_t v = 0; v < n; ++v) { uint32_t r = cnt[deg[v]]++; new2old[r] = v; old2new[v] = r; }
    for (uint32_t e = 0; e < m; ++e) { s[e] = old2new[s[e]]; d[e] = old2new[d[e]]; }
    free(cnt);
    free(deg);
    free(old2new);
    return 0;
}

int ko_ktruss(uint32_t num_nodes, uint32_t num_entries, const uint32_t* src, const uint32_t* dst,
              uint32_t k, int directedness, int recount, uint32_t num_edge_remove_iter,
              uint32_t* out_src, uint32_t* out_dst, uint32_t* out_num, ko_pass_log* log) {
    const int directed = directedness != KO_UNDIRECTED;
    int rc = -1;
    uint32_t *s = NULL, *d = NULL, *new2old = NULL, *ds = NULL, *dd = NULL;
    info_t in;
    csr_t g;
    memset(&in, 0, sizeof(in));
    memset(&g, 0, sizeof(g));
    s = (uint32_t*)malloc(sizeof(uint32_t) * (num_entries ? num_entries : 1));
    d = (uint32_t*)malloc(sizeof(uint32_t) * (num_entries ? num_entries : 1));
    new2old = (uint32_t*)malloc(sizeof(uint32_t) * (num_nodes ? num_nodes : 1));
    if (!s || !d || !new2old) goto done;
    memcpy(s, src, sizeof(uint32_t) * num_entries);
    memcpy(d, dst, sizeof(uint32_t) * num_entries);
    /* kernel.cu:13-20: relabel only for directed-by-degree */
    if (directedness == KO_DIRECTED_BY_DEGREE && sort_by_degree(num_nodes, num_entries, s, d, new2old)) goto done;

    /* kernel_h.cu:24-30, undirected2directedCOO (graph.cu:194-207): keep src < dst */
    uint32_t m = num_entries;
    if (directed) {
        ds = (uint32_t*)malloc(sizeof(uint32_t) * (num_entries / 2 + 1));
        dd = (uint32_t*)malloc(sizeof(uint32_t) * (num_entries / 2 + 1));
        if (!ds || !dd) goto done;
        m = 0;
        for (uint32_t e = 0; e < num_entries; ++e)
            if (s[e] < d[e]) { ds[m] = s[e]; dd[m] = d[e]; ++m; }
    }
    if (coo2coocsr(num_nodes, m, directed ? ds : s, directed ? dd : d, &g)) goto done;

    /* createInfo (info.cu:7-20): slots sized E/2 when directed */
    uint32_t slots = directed ? num_entries / 2 : num_entries;
    if (slots < m) slots = m;
    in.num_triangles = (uint32_t*)calloc(slots ? slots : 1, sizeof(uint32_t));
    in.node_affected = (uint32_t*)calloc(num_nodes ? num_nodes : 1, sizeof(uint32_t));
    in.edge_affected = (uint32_t*)calloc(slots ? slots : 1, sizeof(uint32_t));
    if (!in.num_triangles || !in.node_affected || !in.edge_affected) goto done;

    {
        const double t_loop = now_s();
        peel_loop(&g, k, directed, recount, num_edge_remove_iter, &in, slots, log);
        if (log) log->loop_seconds = now_s() - t_loop;
    }

    /* coocsr2coo (graph.cu:548-554), then directed2undirectedCOO (graph.cu:239-251) and
     * unsort (graph.cu:187-192) */
    uint32_t w = 0;
    for (uint32_t e = 0; e < g.num_edges; ++e) { out_src[w] = g.src[e]; out_dst[w] = g.dst[e]; ++w; }
    if (directed) {
        uint32_t nd = w;
        for (uint32_t e = 0; e < nd; ++e)
            if (out_src[e] != out_dst[e]) { out_src[w] = out_dst[e]; out_dst[w] = out_src[e]; ++w; }
    }
    if (directedness == KO_DIRECTED_BY_DEGREE)
        for (uint32_t e = 0; e < w; ++e) { out_src[e] = new2old[out_src[e]]; out_dst[e] = new2old[out_dst[e]]; }
    *out_num = w;
    rc = 0;
done:
    free(s); free(d); free(new2old); free(ds); free(dd);
    free(in.num_triangles); free(in.node_affected); free(in.edge_affected);
    csr_free(&g);
    return rc;
}

static inline uint64_t edge_key(uint32_t a, uint32_t b) {
    return a < b ? ((uint64_t)a << 32) | b : ((uint64_t)b << 32) | a;
}

/* Whether key is in the sorted array keys[0..n). */
static int contains(const uint64_t* keys, uint32_t n, uint64_t key) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        uint32_t mid = lo + (hi - lo) / 2;
        if (keys[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    return lo < n && keys[lo] == key;
}

int ko_decompose_chain(uint32_t num_nodes, uint32_t num_entries, const uint32_t* src,
                       const uint32_t* dst, uint32_t* truss_per_entry, uint32_t* k_max,
                       uint32_t* plain_passes, uint64_t* plain_alive_sum) {
    int rc = -1;
    uint32_t *cs = NULL, *cd = NULL, *os = NULL, *od = NULL;
    uint64_t *keys = NULL, *alive = NULL;
    uint32_t cur = num_entries, k;
    uint32_t passes = 0;
    uint64_t alive_sum = 0;
    ko_pass_log log;
    cs = (uint32_t*)malloc(sizeof(uint32_t) * (num_entries ? num_entries : 1));
    cd = (uint32_t*)malloc(sizeof(uint32_t) * (num_entries ? num_entries : 1));
    os = (uint32_t*)malloc(sizeof(uint32_t) * (num_entries ? num_entries : 1));
    od = (uint32_t*)malloc(sizeof(uint32_t) * (num_entries ? num_entries : 1));
    keys = (uint64_t*)malloc(sizeof(uint64_t) * (num_entries ? num_entries : 1));
    alive = (uint64_t*)malloc(sizeof(uint64_t) * 65536);
    if (!cs || !cd || !os || !od || !keys || !alive) goto done;
    memcpy(cs, src, sizeof(uint32_t) * num_entries);
    memcpy(cd, dst, sizeof(uint32_t) * num_entries);
    for (uint32_t i = 0; i < num_entries; ++i) truss_per_entry[i] = 2;
    *k_max = num_entries ? 2 : 0;
    log.cap = 65536;
    log.alive = alive;
    for (k = 3; cur > 0; ++k) {
        uint32_t nout = 0;
        if (ko_ktruss(num_nodes, cur, cs, cd, k, KO_DIRECTED_BY_DEGREE, KO_RECOUNT_ALL, 0, os, od, &nout, &log)) goto done;
        passes += log.num;
        for (uint32_t p = 0; p < log.num && p < log.cap; ++p) alive_sum += log.alive[p];
        if (nout == 0) break;
        for (uint32_t i = 0; i < nout; ++i) keys[i] = edge_key(os[i], od[i]);
        qsort(keys, nout, sizeof(uint64_t), cmp_u64);
        for (uint32_t i = 0; i < num_entries; ++i)
            if (truss_per_entry[i] == k - 1 && contains(keys, nout, edge_key(src[i], dst[i]))) truss_per_entry[i] = k;
        *k_max = k;
        memcpy(cs, os, sizeof(uint32_t) * nout);
        memcpy(cd, od, sizeof(uint32_t) * nout);
        cur = nout;
    }
    if (plain_passes) *plain_passes = passes;
    if (plain_alive_sum) *plain_alive_sum = alive_sum;
    rc = 0;
done:
    free(cs); free(cd); free(os); free(od); free(keys); free(alive);
    return rc;
}

int ko_chain_sample(uint32_t num_nodes, uint32_t num_entries, const uint32_t* src, const uint32_t* dst,
                    double budget_s, uint32_t* passes_done, uint64_t* alive_done, double* seconds) {
    int rc = -1;
    uint32_t *cs = NULL, *cd = NULL, *os = NULL, *od = NULL;
    uint64_t* alive = NULL;
    uint32_t cur = num_entries, passes = 0;
    uint64_t alive_sum = 0;
    ko_pass_log log;
    const double t0 = now_s();
    cs = (uint32_t*)malloc(sizeof(uint32_t) * (num_entries ? num_entries : 1));
    cd = (uint32_t*)malloc(sizeof(uint32_t) * (num_entries ? num_entries : 1));
    os = (uint32_t*)malloc(sizeof(uint32_t) * (num_entries ? num_entries : 1));
    od = (uint32_t*)malloc(sizeof(uint32_t) * (num_entries ? num_entries : 1));
    alive = (uint64_t*)malloc(sizeof(uint64_t) * 65536);
    if (!cs || !cd || !os || !od || !alive) goto done;
    memcpy(cs, src, sizeof(uint32_t) * num_entries);
    memcpy(cd, dst, sizeof(uint32_t) * num_entries);
    log.cap = 65536;
    log.alive = alive;
    g_deadline = t0 + budget_s;
    g_deadline_hit = 0;
    g_cut_in_count = 0;
    g_cut_alive = 0;
    for (uint32_t k = 3; cur > 0 && !g_deadline_hit; ++k) {
        uint32_t nout = 0;
        if (ko_ktruss(num_nodes, cur, cs, cd, k, KO_DIRECTED_BY_DEGREE, KO_RECOUNT_ALL, 0, os, od, &nout, &log)) goto done;
        /* a pass cut by the deadline counts only the alive edges its count had merged
         * (log.num counts started passes) */
        uint32_t full = log.num;
        if (g_cut_in_count && full > 0) {
            --full;
            alive_sum += g_cut_alive;
        }
        for (uint32_t p = 0; p < full && p < log.cap; ++p) alive_sum += log.alive[p];
        passes += full;
        if (nout == 0) break;
        memcpy(cs, os, sizeof(uint32_t) * nout);
        memcpy(cd, od, sizeof(uint32_t) * nout);
        cur = nout;
    }
    *passes_done = passes;
    *alive_done = alive_sum;
    *seconds = now_s() - t0;
    rc = 0;
done:
    g_deadline = 0.0;
    free(cs); free(cd); free(os); free(od); free(alive);
    return rc;
}

/* Exact serial peeling.  Level k removes, in synchronous rounds, the alive edges whose
 * support is below k-2; removing an edge destroys each of its alive triangles once.  When
 * several edges of one triangle fall in the same round, the one with the smallest id applies
 * the triangle's decrement to the surviving edges.  The rounds coincide with the count-and-
 * prune passes of the reference loop, so the pass statistics of ko_decompose_chain follow.
 * The triangles of a removed edge (x, y) are found by walking the shorter of the two symmetric
 * rows against the other (merged, or binary-searched when it is more than 16 times longer);
 * rows are sorted, keep removed entries (the round stamps filter them) and are compacted at a
 * level start once the alive edges fell below 70 % of the last compaction.  With `levels`, the per-level pass counts and alive-edge sums of the
 * reference chain are stored by k (entries 0..cap-1; levels above cap-1 are not stored). */
static uint32_t row_find(const uint32_t* col, uint32_t lo, uint32_t hi, uint32_t w) {
    while (lo < hi) {
        uint32_t mid = lo + (hi - lo) / 2;
        if (col[mid] < w) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

int ko_decompose_peel_levels(uint32_t num_nodes, uint32_t num_entries, const uint32_t* src,
                             const uint32_t* dst, uint32_t* truss_per_entry, uint32_t* k_max,
                             uint32_t* plain_passes, uint64_t* plain_alive_sum, uint32_t* num_rounds,
                             ko_level_log* levels) {
    int rc = -1;
    uint32_t m = 0, n = num_nodes;
    uint64_t* keys = NULL;
    uint32_t *ptr = NULL, *col = NULL, *eid = NULL, *fill = NULL, *sup = NULL, *rnd = NULL, *tr = NULL;
    uint32_t *F = NULL, *NF = NULL, *rlen = NULL;
    if (levels) {
        for (uint32_t i = 0; i < levels->cap; ++i) { levels->passes[i] = 0; levels->alive[i] = 0; }
        levels->num = 0;
    }
#define KO_LEVEL_PASS(kk, a)                                                       \
    do {                                                                           \
        if (levels && (kk) < levels->cap) {                                        \
            levels->passes[kk]++;                                                  \
            levels->alive[kk] += (a);                                              \
            if ((kk) + 1 > levels->num) levels->num = (kk) + 1;                    \
        }                                                                          \
    } while (0)
    keys = (uint64_t*)malloc(sizeof(uint64_t) * (num_entries ? num_entries : 1));
    if (!keys) goto done;
    for (uint32_t i = 0; i < num_entries; ++i)
        if (src[i] < dst[i]) keys[m++] = ((uint64_t)src[i] << 32) | dst[i];
    qsort(keys, m, sizeof(uint64_t), cmp_u64);
    ptr = (uint32_t*)calloc((size_t)n + 1, sizeof(uint32_t));
    col = (uint32_t*)malloc(sizeof(uint32_t) * (2 * (size_t)m + 1));
    eid = (uint32_t*)malloc(sizeof(uint32_t) * (2 * (size_t)m + 1));
    fill = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)n + 1));
    sup = (uint32_t*)calloc((size_t)m + 1, sizeof(uint32_t));
    rnd = (uint32_t*)calloc((size_t)m + 1, sizeof(uint32_t));
    tr = (uint32_t*)calloc((size_t)m + 1, sizeof(uint32_t));
    F = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)m + 1));
    NF = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)m + 1));
    rlen = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)n + 1));
    if (!ptr || !col || !eid || !fill || !sup || !rnd || !tr || !F || !NF || !rlen) goto done;
    for (uint32_t e = 0; e < m; ++e) { ptr[(keys[e] >> 32) + 1]++; ptr[(uint32_t)keys[e] + 1]++; }
    for (uint32_t v = 0; v < n; ++v) ptr[v + 1] += ptr[v];
    memcpy(fill, ptr, sizeof(uint32_t) * n);
    /* keys are sorted by (u, v): row v receives its smaller neighbours u in ascending order
     * before any larger neighbour, so every row comes out sorted. */
    for (uint32_t e = 0; e < m; ++e) {
        uint32_t u = (uint32_t)(keys[e] >> 32), v = (uint32_t)keys[e];
        col[fill[v]] = u; eid[fill[v]++] = e;
    }
    for (uint32_t e = 0; e < m; ++e) {
        uint32_t u = (uint32_t)(keys[e] >> 32), v = (uint32_t)keys[e];
        col[fill[u]] = v; eid[fill[u]++] = e;
    }
    /* initial support: per oriented edge (u, v), u < v, the common neighbours above v (each
     * triangle u < v < w counted once, crediting its three edges) */
    for (uint32_t e = 0; e < m; ++e) {
        uint32_t u = (uint32_t)(keys[e] >> 32), v = (uint32_t)keys[e];
        uint32_t a = row_find(col, ptr[u], ptr[u + 1], v + 1), ae = ptr[u + 1];
        uint32_t b = row_find(col, ptr[v], ptr[v + 1], v + 1), be = ptr[v + 1];
        if ((uint64_t)(ae - a) > 16ull * (be - b) || (uint64_t)(be - b) > 16ull * (ae - a)) {
            /* one tail much longer: walk the shorter, binary-search the longer */
            const int a_short = ae - a <= be - b;
            uint32_t s0 = a_short ? a : b, s1 = a_short ? ae : be, l0 = a_short ? b : a, l1 = a_short ? be : ae;
            for (; s0 < s1; ++s0) {
                const uint32_t x = row_find(col, l0, l1, col[s0]);
                if (x < l1 && col[x] == col[s0]) { sup[e]++; sup[eid[s0]]++; sup[eid[x]]++; }
            }
            continue;
        }
        while (a < ae && b < be) {
            if (col[a] < col[b]) ++a;
            else if (col[a] > col[b]) ++b;
            else { sup[e]++; sup[eid[a]]++; sup[eid[b]]++; ++a; ++b; }
        }
    }
    /* Pass statistics of the reference chain (ko_decompose_chain): level 3 is one pass over
     * all m edges (kernel_hdc.cu:169-172 stops after the first pass); each level k >= 4 up to
     * k_max+1 takes one pass per round that removes edges plus a final pass that removes
     * nothing, each pass seeing the edges alive at its start. */
    for (uint32_t v = 0; v < n; ++v) rlen[v] = ptr[v + 1] - ptr[v];
    uint64_t alive = m, alive_sum = m, alive_at_compaction = m;
    uint32_t k = 3, r = 0, passes = m ? 1 : 0;
    if (m) KO_LEVEL_PASS(3u, (uint64_t)m);
    while (alive) {
        uint32_t nf = 0, mn = 0xffffffffu;
        if (alive * 10 < alive_at_compaction * 7) {
            /* drop the removed edges' entries from the rows (order kept) */
            for (uint32_t v = 0; v < n; ++v) {
                uint32_t w = ptr[v];
                for (uint32_t a = ptr[v]; a < ptr[v] + rlen[v]; ++a)
                    if (!rnd[eid[a]]) { col[w] = col[a]; eid[w] = eid[a]; ++w; }
                rlen[v] = w - ptr[v];
            }
            alive_at_compaction = alive;
        }
        for (uint32_t e = 0; e < m; ++e)
            if (!rnd[e]) { if (sup[e] < k - 2) F[nf++] = e; if (sup[e] < mn) mn = sup[e]; }
        if (!nf) {
            /* levels k .. mn+2 remove nothing: one pass each (levels >= 4) */
            for (uint32_t kk = k > 3 ? k : 4; kk < mn + 3; ++kk) { passes++; alive_sum += alive; KO_LEVEL_PASS(kk, alive); }
            k = mn + 3;
            continue;
        }
        while (nf) {
            if (k >= 4) { passes++; alive_sum += alive; KO_LEVEL_PASS(k, alive); }
            ++r;
            for (uint32_t i = 0; i < nf; ++i) { rnd[F[i]] = r; tr[F[i]] = k - 1; }
            uint32_t nn = 0;
            for (uint32_t i = 0; i < nf; ++i) {
                uint32_t e = F[i];
                uint32_t x = (uint32_t)(keys[e] >> 32), y = (uint32_t)keys[e];
                if (rlen[x] > rlen[y]) { uint32_t t = x; x = y; y = t; }
                const uint32_t yb = ptr[y], ye = ptr[y] + rlen[y], xe = ptr[x] + rlen[x];
                /* rows of similar length are merged; a much longer row is binary-searched */
                const int search = (uint64_t)rlen[y] > 16ull * rlen[x];
                uint32_t b = yb;
                for (uint32_t a = ptr[x]; a < xe; ++a) {
                    const uint32_t w = col[a];
                    if (search) b = row_find(col, yb, ye, w);
                    else while (b < ye && col[b] < w) ++b;
                    if (b == ye) { if (search) continue; break; }
                    if (col[b] != w) continue;
                    uint32_t ex = eid[a], ey = eid[b];
                    if ((rnd[ex] && rnd[ex] != r) || (rnd[ey] && rnd[ey] != r)) continue; /* already gone */
                    if ((rnd[ex] == r && ex < e) || (rnd[ey] == r && ey < e)) continue;   /* owned by a smaller id */
                    if (!rnd[ex] && sup[ex]-- == k - 2) NF[nn++] = ex;
                    if (!rnd[ey] && sup[ey]-- == k - 2) NF[nn++] = ey;
                }
            }
            alive -= nf;
            uint32_t* t = F; F = NF; NF = t;
            nf = nn;
        }
        if (k >= 4) { passes++; alive_sum += alive; KO_LEVEL_PASS(k, alive); }
        ++k;
    }
#undef KO_LEVEL_PASS
    for (uint32_t e = 0; e < m; ++e) if (tr[e] == 0) tr[e] = 2;
    uint32_t km = 0;
    for (uint32_t e = 0; e < m; ++e) if (tr[e] > km) km = tr[e];
    *k_max = m ? km : 0;
    /* entries -> edge ids */
    for (uint32_t i = 0; i < num_entries; ++i) {
        uint64_t key = edge_key(src[i], dst[i]);
        uint32_t lo = 0, hi = m;
        while (lo < hi) { uint32_t mid = lo + (hi - lo) / 2; if (keys[mid] < key) lo = mid + 1; else hi = mid; }
        truss_per_entry[i] = (lo < m && keys[lo] == key) ? tr[lo] : 0;
    }
    if (plain_passes) *plain_passes = passes;
    if (plain_alive_sum) *plain_alive_sum = alive_sum;
    if (num_rounds) *num_rounds = r;
    rc = 0;
done:
    free(keys); free(ptr); free(col); free(eid); free(fill); free(sup); free(rnd); free(tr); free(F); free(NF);
    free(rlen);
    return rc;
}

int ko_decompose_peel(uint32_t num_nodes, uint32_t num_entries, const uint32_t* src,
                      const uint32_t* dst, uint32_t* truss_per_entry, uint32_t* k_max,
                      uint32_t* plain_passes, uint64_t* plain_alive_sum, uint32_t* num_rounds) {
    return ko_decompose_peel_levels(num_nodes, num_entries, src, dst, truss_per_entry, k_max, plain_passes,
                                    plain_alive_sum, num_rounds, NULL);
}

/* ---- The same peel on several host threads --------------------------------------------------
 * ko_decompose_peel_mt computes exactly what ko_decompose_peel_levels computes (same rounds, same
 * ownership rule, same pass statistics); only the work inside each phase is split over threads:
 * the initial support count, the level scan that collects a frontier, the marking of the frontier,
 * the walks of the frontier's rows (support decrements are atomic; edges whose support falls
 * from k-2 to k-3 are appended to the next frontier with an atomic counter), the row compaction
 * and the entry -> edge map.  Thread 0 runs the level / round loop between the phases; phases are
 * separated by barriers, so each round sees the stamps of the previous round complete.  Frontier
 * order differs from the serial peel, which does not change any result (a round's frontier is a
 * set; the ownership rule compares edge ids). */
#include <pthread.h>

/* A reusable barrier whose participant count can be lowered before its first use completes. */
typedef struct {
    pthread_mutex_t mu;
    pthread_cond_t cv;
    uint32_t count, waiting, gen;
} ko_barrier;

static void ko_bar_wait(ko_barrier* b) {
    pthread_mutex_lock(&b->mu);
    const uint32_t g = b->gen;
    if (++b->waiting >= b->count) {
        b->waiting = 0;
        b->gen++;
        pthread_cond_broadcast(&b->cv);
    } else {
        while (g == b->gen) pthread_cond_wait(&b->cv, &b->mu);
    }
    pthread_mutex_unlock(&b->mu);
}

enum { KO_PH_STOP = 0, KO_PH_SUPPORT, KO_PH_SCAN, KO_PH_MARK, KO_PH_WALK, KO_PH_COMPACT, KO_PH_MAP };

typedef struct {
    uint32_t n, m, num_entries;
    const uint32_t *src, *dst;
    const uint64_t* keys;
    uint32_t *ptr, *col, *eid, *sup, *rnd, *tr, *rlen, *F, *NF, *truss_per_entry;
    int phase;
    uint32_t k, r, nf, nn, next;
    uint32_t mn[64];
    uint32_t threads;
    ko_barrier bar;
} ko_mt;

#define KO_CHUNK 256u

static uint32_t ko_take(ko_mt* c) { return __atomic_fetch_add(&c->next, KO_CHUNK, __ATOMIC_RELAXED); }

static void ko_mt_phase(ko_mt* c, uint32_t tid) {
    const uint32_t k = c->k;
    switch (c->phase) {
    case KO_PH_SUPPORT:
        for (uint32_t e0; (e0 = ko_take(c)) < c->m;) {
            const uint32_t e1 = e0 + KO_CHUNK < c->m ? e0 + KO_CHUNK : c->m;
            for (uint32_t e = e0; e < e1; ++e) {
                uint32_t u = (uint32_t)(c->keys[e] >> 32), v = (uint32_t)c->keys[e];
                uint32_t a = row_find(c->col, c->ptr[u], c->ptr[u + 1], v + 1), ae = c->ptr[u + 1];
                uint32_t b = row_find(c->col, c->ptr[v], c->ptr[v + 1], v + 1), be = c->ptr[v + 1];
                uint32_t cnt = 0;
                if ((uint64_t)(ae - a) > 16ull * (be - b) || (uint64_t)(be - b) > 16ull * (ae - a)) {
                    const int a_short = ae - a <= be - b;
                    uint32_t s0 = a_short ? a : b, s1 = a_short ? ae : be, l0 = a_short ? b : a, l1 = a_short ? be : ae;
                    for (; s0 < s1; ++s0) {
                        const uint32_t x = row_find(c->col, l0, l1, c->col[s0]);
                        if (x < l1 && c->col[x] == c->col[s0]) {
                            ++cnt;
                            __atomic_fetch_add(&c->sup[c->eid[s0]], 1u, __ATOMIC_RELAXED);
                            __atomic_fetch_add(&c->sup[c->eid[x]], 1u, __ATOMIC_RELAXED);
                        }
                    }
                } else {
                    while (a < ae && b < be) {
                        if (c->col[a] < c->col[b]) ++a;
                        else if (c->col[a] > c->col[b]) ++b;
                        else {
                            ++cnt;
                            __atomic_fetch_add(&c->sup[c->eid[a]], 1u, __ATOMIC_RELAXED);
                            __atomic_fetch_add(&c->sup[c->eid[b]], 1u, __ATOMIC_RELAXED);
                            ++a; ++b;
                        }
                    }
                }
                if (cnt) __atomic_fetch_add(&c->sup[e], cnt, __ATOMIC_RELAXED);
            }
        }
        break;
    case KO_PH_SCAN: {
        uint32_t mn = 0xffffffffu;
        for (uint32_t e0; (e0 = ko_take(c)) < c->m;) {
            const uint32_t e1 = e0 + KO_CHUNK < c->m ? e0 + KO_CHUNK : c->m;
            for (uint32_t e = e0; e < e1; ++e)
                if (!c->rnd[e]) {
                    if (c->sup[e] < k - 2) c->F[__atomic_fetch_add(&c->nf, 1u, __ATOMIC_RELAXED)] = e;
                    if (c->sup[e] < mn) mn = c->sup[e];
                }
        }
        c->mn[tid] = mn;
        break;
    }
    case KO_PH_MARK:
        for (uint32_t i0; (i0 = ko_take(c)) < c->nf;) {
            const uint32_t i1 = i0 + KO_CHUNK < c->nf ? i0 + KO_CHUNK : c->nf;
            for (uint32_t i = i0; i < i1; ++i) { c->rnd[c->F[i]] = c->r; c->tr[c->F[i]] = k - 1; }
        }
        break;
    case KO_PH_WALK:
        for (uint32_t i0; (i0 = __atomic_fetch_add(&c->next, 1u, __ATOMIC_RELAXED)) < c->nf;) {
            const uint32_t e = c->F[i0], r = c->r;
            uint32_t x = (uint32_t)(c->keys[e] >> 32), y = (uint32_t)c->keys[e];
            if (c->rlen[x] > c->rlen[y]) { uint32_t t = x; x = y; y = t; }
            const uint32_t yb = c->ptr[y], ye = c->ptr[y] + c->rlen[y], xe = c->ptr[x] + c->rlen[x];
            const int search = (uint64_t)c->rlen[y] > 16ull * c->rlen[x];
            uint32_t b = yb;
            for (uint32_t a = c->ptr[x]; a < xe; ++a) {
                const uint32_t w = c->col[a];
                if (search) b = row_find(c->col, yb, ye, w);
                else while (b < ye && c->col[b] < w) ++b;
                if (b == ye) { if (search) continue; break; }
                if (c->col[b] != w) continue;
                const uint32_t ex = c->eid[a], ey = c->eid[b];
                if ((c->rnd[ex] && c->rnd[ex] != r) || (c->rnd[ey] && c->rnd[ey] != r)) continue;
                if ((c->rnd[ex] == r && ex < e) || (c->rnd[ey] == r && ey < e)) continue;
                if (!c->rnd[ex] && __atomic_fetch_sub(&c->sup[ex], 1u, __ATOMIC_RELAXED) == k - 2)
                    c->NF[__atomic_fetch_add(&c->nn, 1u, __ATOMIC_RELAXED)] = ex;
                if (!c->rnd[ey] && __atomic_fetch_sub(&c->sup[ey], 1u, __ATOMIC_RELAXED) == k - 2)
                    c->NF[__atomic_fetch_add(&c->nn, 1u, __ATOMIC_RELAXED)] = ey;
            }
        }
        break;
    case KO_PH_COMPACT:
        for (uint32_t v0; (v0 = ko_take(c)) < c->n;) {
            const uint32_t v1 = v0 + KO_CHUNK < c->n ? v0 + KO_CHUNK : c->n;
            for (uint32_t v = v0; v < v1; ++v) {
                uint32_t w = c->ptr[v];
                for (uint32_t a = c->ptr[v]; a < c->ptr[v] + c->rlen[v]; ++a)
                    if (!c->rnd[c->eid[a]]) { c->col[w] = c->col[a]; c->eid[w] = c->eid[a]; ++w; }
                c->rlen[v] = w - c->ptr[v];
            }
        }
        break;
    case KO_PH_MAP:
        for (uint32_t i0; (i0 = ko_take(c)) < c->num_entries;) {
            const uint32_t i1 = i0 + KO_CHUNK < c->num_entries ? i0 + KO_CHUNK : c->num_entries;
            for (uint32_t i = i0; i < i1; ++i) {
                uint64_t key = edge_key(c->src[i], c->dst[i]);
                uint32_t lo = 0, hi = c->m;
                while (lo < hi) { uint32_t mid = lo + (hi - lo) / 2; if (c->keys[mid] < key) lo = mid + 1; else hi = mid; }
                c->truss_per_entry[i] = (lo < c->m && c->keys[lo] == key) ? c->tr[lo] : 0;
            }
        }
        break;
    default:
        break;
    }
}

typedef struct { ko_mt* c; uint32_t tid; } ko_worker_arg;

static void* ko_worker(void* p) {
    ko_worker_arg* a = (ko_worker_arg*)p;
    for (;;) {
        ko_bar_wait(&a->c->bar);
        if (a->c->phase == KO_PH_STOP) break;
        ko_mt_phase(a->c, a->tid);
        ko_bar_wait(&a->c->bar);
    }
    return NULL;
}

/* Thread 0: runs one phase on all threads and returns when every thread has finished it. */
static void ko_run(ko_mt* c, int phase) {
    c->phase = phase;
    c->next = 0;
    ko_bar_wait(&c->bar);
    ko_mt_phase(c, 0);
    ko_bar_wait(&c->bar);
}

int ko_decompose_peel_mt(uint32_t num_nodes, uint32_t num_entries, const uint32_t* src,
                         const uint32_t* dst, uint32_t* truss_per_entry, uint32_t* k_max,
                         uint32_t* plain_passes, uint64_t* plain_alive_sum, uint32_t* num_rounds,
                         ko_level_log* levels, uint32_t threads) {
    int rc = -1;
    ko_mt c;
    memset(&c, 0, sizeof(c));
    uint32_t m = 0, n = num_nodes, started = 0;
    uint64_t* keys = NULL;
    uint32_t* fill = NULL;
    pthread_t th[64];
    ko_worker_arg args[64];
    if (threads < 1) threads = 1;
    if (threads > 64) threads = 64;
    if (levels) {
        for (uint32_t i = 0; i < levels->cap; ++i) { levels->passes[i] = 0; levels->alive[i] = 0; }
        levels->num = 0;
    }
#define KO_LEVEL_PASS(kk, a)                                                       \
    do {                                                                           \
        if (levels && (kk) < levels->cap) {                                        \
            levels->passes[kk]++;                                                  \
            levels->alive[kk] += (a);                                              \
            if ((kk) + 1 > levels->num) levels->num = (kk) + 1;                    \
        }                                                                          \
    } while (0)
    keys = (uint64_t*)malloc(sizeof(uint64_t) * (num_entries ? num_entries : 1));
    if (!keys) goto done;
    for (uint32_t i = 0; i < num_entries; ++i)
        if (src[i] < dst[i]) keys[m++] = ((uint64_t)src[i] << 32) | dst[i];
    qsort(keys, m, sizeof(uint64_t), cmp_u64);
    c.n = n; c.m = m; c.num_entries = num_entries; c.src = src; c.dst = dst; c.keys = keys;
    c.truss_per_entry = truss_per_entry; c.threads = threads;
    c.ptr = (uint32_t*)calloc((size_t)n + 1, sizeof(uint32_t));
    c.col = (uint32_t*)malloc(sizeof(uint32_t) * (2 * (size_t)m + 1));
    c.eid = (uint32_t*)malloc(sizeof(uint32_t) * (2 * (size_t)m + 1));
    fill = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)n + 1));
    c.sup = (uint32_t*)calloc((size_t)m + 1, sizeof(uint32_t));
    c.rnd = (uint32_t*)calloc((size_t)m + 1, sizeof(uint32_t));
    c.tr = (uint32_t*)calloc((size_t)m + 1, sizeof(uint32_t));
    c.F = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)m + 1));
    c.NF = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)m + 1));
    c.rlen = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)n + 1));
    if (!c.ptr || !c.col || !c.eid || !fill || !c.sup || !c.rnd || !c.tr || !c.F || !c.NF || !c.rlen) goto done;
    for (uint32_t e = 0; e < m; ++e) { c.ptr[(keys[e] >> 32) + 1]++; c.ptr[(uint32_t)keys[e] + 1]++; }
    for (uint32_t v = 0; v < n; ++v) c.ptr[v + 1] += c.ptr[v];
    memcpy(fill, c.ptr, sizeof(uint32_t) * n);
    for (uint32_t e = 0; e < m; ++e) {
        uint32_t u = (uint32_t)(keys[e] >> 32), v = (uint32_t)keys[e];
        c.col[fill[v]] = u; c.eid[fill[v]++] = e;
    }
    for (uint32_t e = 0; e < m; ++e) {
        uint32_t u = (uint32_t)(keys[e] >> 32), v = (uint32_t)keys[e];
        c.col[fill[u]] = v; c.eid[fill[u]++] = e;
    }
    for (uint32_t v = 0; v < n; ++v) c.rlen[v] = c.ptr[v + 1] - c.ptr[v];
    for (uint32_t t = 0; t < 64; ++t) c.mn[t] = 0xffffffffu;
    pthread_mutex_init(&c.bar.mu, NULL);
    pthread_cond_init(&c.bar.cv, NULL);
    c.bar.count = threads;
    for (started = 1; started < threads; ++started) {
        args[started].c = &c;
        args[started].tid = started;
        if (pthread_create(&th[started], NULL, ko_worker, &args[started])) break;
    }
    if (started < threads) { /* fewer threads could be started: go on with those */
        pthread_mutex_lock(&c.bar.mu);
        c.bar.count = started;
        c.threads = started;
        pthread_mutex_unlock(&c.bar.mu);
        threads = started;
    }
    ko_run(&c, KO_PH_SUPPORT);
    {
        uint64_t alive = m, alive_sum = m, alive_at_compaction = m;
        uint32_t k = 3, r = 0, passes = m ? 1 : 0;
        if (m) KO_LEVEL_PASS(3u, (uint64_t)m);
        while (alive) {
            if (alive * 10 < alive_at_compaction * 7) {
                ko_run(&c, KO_PH_COMPACT);
                alive_at_compaction = alive;
            }
            c.k = k;
            c.nf = 0;
            ko_run(&c, KO_PH_SCAN);
            uint32_t mn = 0xffffffffu;
            for (uint32_t t = 0; t < threads; ++t) if (c.mn[t] < mn) mn = c.mn[t];
            if (!c.nf) {
                for (uint32_t kk = k > 3 ? k : 4; kk < mn + 3; ++kk) { passes++; alive_sum += alive; KO_LEVEL_PASS(kk, alive); }
                k = mn + 3;
                continue;
            }
            while (c.nf) {
                if (k >= 4) { passes++; alive_sum += alive; KO_LEVEL_PASS(k, alive); }
                ++r;
                c.r = r;
                ko_run(&c, KO_PH_MARK);
                c.nn = 0;
                ko_run(&c, KO_PH_WALK);
                alive -= c.nf;
                uint32_t* t = c.F; c.F = c.NF; c.NF = t;
                c.nf = c.nn;
            }
            if (k >= 4) { passes++; alive_sum += alive; KO_LEVEL_PASS(k, alive); }
            ++k;
        }
        for (uint32_t e = 0; e < m; ++e) if (c.tr[e] == 0) c.tr[e] = 2;
        uint32_t km = 0;
        for (uint32_t e = 0; e < m; ++e) if (c.tr[e] > km) km = c.tr[e];
        *k_max = m ? km : 0;
        ko_run(&c, KO_PH_MAP);
        if (plain_passes) *plain_passes = passes;
        if (plain_alive_sum) *plain_alive_sum = alive_sum;
        if (num_rounds) *num_rounds = r;
    }
#undef KO_LEVEL_PASS
    rc = 0;
    c.phase = KO_PH_STOP;
    if (started > 1) {
        ko_bar_wait(&c.bar);
        for (uint32_t t = 1; t < started; ++t) pthread_join(th[t], NULL);
    }
    pthread_mutex_destroy(&c.bar.mu);
    pthread_cond_destroy(&c.bar.cv);
done:
    free(keys); free(c.ptr); free(c.col); free(c.eid); free(fill); free(c.sup); free(c.rnd); free(c.tr);
    free(c.F); free(c.NF); free(c.rlen);
    return rc;
}

/* ---- Timed repeat runs of the reference loop on several host threads ---------------------------
 * ko_ktruss_runs mirrors the reference CLI's repeat runs (-w warm-up, -x timed; kernel_hdc.cu:
 * 207-242) of the default variant (directed by degree, recount all, no compaction): the graph is
 * relabeled, oriented and converted to CSR once; every run restores the CSR (as the reference's
 * coo2coocsr between runs) and then runs the count-and-prune loop of kernel_hdc.cu:107-201 to
 * convergence, timed alone like the reference's k-truss timer.  The loop's two data-parallel
 * sweeps - the triangle count (count_triangles, kernel_hdc.cu:11-49: per-edge merges whose
 * increments of the other two edges' counters become atomic) and the deletion mark
 * (kernel_hdc.cu:51-70) - are split over `threads` host threads; passes, edge sets and results are
 * those of the serial loop. */
typedef struct {
    csr_t* g;
    uint32_t* tri;
    uint32_t k, has_deleted, changed, next;
    int phase; /* 0 stop, 1 count, 2 mark */
    ko_barrier bar;
} ko_runs_ctx;

static void ko_runs_phase(ko_runs_ctx* c) {
    csr_t* g = c->g;
    const uint32_t chk = c->has_deleted, chunk = 64;
    if (c->phase == 1) {
        for (uint32_t e0; (e0 = __atomic_fetch_add(&c->next, chunk, __ATOMIC_RELAXED)) < g->num_edges;) {
            const uint32_t e1 = e0 + chunk < g->num_edges ? e0 + chunk : g->num_edges;
            for (uint32_t e = e0; e < e1; ++e) {
                const uint32_t dst = g->dst[e];
                if (chk && dst == KO_DELETED) continue;
                uint32_t e1p = g->ptr[g->src[e]], end1 = g->ptr[g->src[e] + 1];
                uint32_t e2p = g->ptr[dst], end2 = g->ptr[dst + 1];
                uint32_t cnt = 0;
                while (e1p < end1 && e2p < end2) {
                    const uint32_t d1 = g->dst[e1p];
                    if (chk && d1 == KO_DELETED) { ++e1p; continue; }
                    const uint32_t d2 = g->dst[e2p];
                    if (chk && d2 == KO_DELETED) { ++e2p; continue; }
                    if (d1 < d2) ++e1p;
                    else if (d1 > d2) ++e2p;
                    else {
                        ++cnt;
                        __atomic_fetch_add(&c->tri[e1p], 1u, __ATOMIC_RELAXED);
                        __atomic_fetch_add(&c->tri[e2p], 1u, __ATOMIC_RELAXED);
                        ++e1p;
                        ++e2p;
                    }
                }
                if (cnt) __atomic_fetch_add(&c->tri[e], cnt, __ATOMIC_RELAXED);
            }
        }
    } else if (c->phase == 2) {
        uint32_t changed = 0;
        for (uint32_t e0; (e0 = __atomic_fetch_add(&c->next, 4096u, __ATOMIC_RELAXED)) < g->num_edges;) {
            const uint32_t e1 = e0 + 4096u < g->num_edges ? e0 + 4096u : g->num_edges;
            for (uint32_t e = e0; e < e1; ++e) {
                if (chk && g->dst[e] == KO_DELETED) continue;
                if (c->tri[e] < c->k - 2) { g->dst[e] = KO_DELETED; changed = 1; }
            }
        }
        if (changed) __atomic_store_n(&c->changed, 1u, __ATOMIC_RELAXED);
    }
}

typedef struct { ko_runs_ctx* c; } ko_runs_arg;

static void* ko_runs_worker(void* p) {
    ko_runs_ctx* c = ((ko_runs_arg*)p)->c;
    for (;;) {
        ko_bar_wait(&c->bar);
        if (c->phase == 0) break;
        ko_runs_phase(c);
        ko_bar_wait(&c->bar);
    }
    return NULL;
}

static void ko_runs_go(ko_runs_ctx* c, int phase) {
    c->phase = phase;
    c->next = 0;
    ko_bar_wait(&c->bar);
    ko_runs_phase(c);
    ko_bar_wait(&c->bar);
}

int ko_ktruss_runs(uint32_t num_nodes, uint32_t num_entries, const uint32_t* src, const uint32_t* dst,
                   uint32_t k, uint32_t runs, uint32_t threads, uint32_t* out_src, uint32_t* out_dst,
                   uint32_t* out_num, double* run_seconds, uint32_t* run_passes) {
    int rc = -1;
    uint32_t *s = NULL, *d = NULL, *new2old = NULL, *ds = NULL, *dd = NULL, *pristine = NULL;
    csr_t g;
    ko_runs_ctx c;
    pthread_t th[64];
    ko_runs_arg arg;
    uint32_t started = 1;
    memset(&g, 0, sizeof(g));
    memset(&c, 0, sizeof(c));
    if (threads < 1) threads = 1;
    if (threads > 64) threads = 64;
    s = (uint32_t*)malloc(sizeof(uint32_t) * (num_entries ? num_entries : 1));
    d = (uint32_t*)malloc(sizeof(uint32_t) * (num_entries ? num_entries : 1));
    new2old = (uint32_t*)malloc(sizeof(uint32_t) * (num_nodes ? num_nodes : 1));
    ds = (uint32_t*)malloc(sizeof(uint32_t) * (num_entries / 2 + 1));
    dd = (uint32_t*)malloc(sizeof(uint32_t) * (num_entries / 2 + 1));
    if (!s || !d || !new2old || !ds || !dd) goto done;
    memcpy(s, src, sizeof(uint32_t) * num_entries);
    memcpy(d, dst, sizeof(uint32_t) * num_entries);
    if (sort_by_degree(num_nodes, num_entries, s, d, new2old)) goto done;
    uint32_t m = 0;
    for (uint32_t e = 0; e < num_entries; ++e)
        if (s[e] < d[e]) { ds[m] = s[e]; dd[m] = d[e]; ++m; }
    if (coo2coocsr(num_nodes, m, ds, dd, &g)) goto done;
    pristine = (uint32_t*)malloc(sizeof(uint32_t) * (m ? m : 1));
    c.tri = (uint32_t*)calloc(m ? m : 1, sizeof(uint32_t));
    if (!pristine || !c.tri) goto done;
    memcpy(pristine, g.dst, sizeof(uint32_t) * m);
    c.g = &g;
    c.k = k;
    pthread_mutex_init(&c.bar.mu, NULL);
    pthread_cond_init(&c.bar.cv, NULL);
    c.bar.count = threads;
    arg.c = &c;
    for (started = 1; started < threads; ++started)
        if (pthread_create(&th[started], NULL, ko_runs_worker, &arg)) break;
    if (started < threads) {
        pthread_mutex_lock(&c.bar.mu);
        c.bar.count = started;
        pthread_mutex_unlock(&c.bar.mu);
    }
    for (uint32_t run = 0; run < runs; ++run) {
        memcpy(g.dst, pristine, sizeof(uint32_t) * m); /* restore the graph (untimed) */
        g.num_edges = m;
        uint32_t passes = 0;
        const double t0 = now_s();
        c.has_deleted = 0;
        for (;;) {
            memset(c.tri, 0, sizeof(uint32_t) * m);
            c.changed = 0;
            ++passes;
            ko_runs_go(&c, 1);
            ko_runs_go(&c, 2);
            if (!c.changed) break;
            c.has_deleted = 1;
            if (k == 3) break; /* kernel_hdc.cu:169-172 */
        }
        if (run_seconds) run_seconds[run] = now_s() - t0;
        if (run_passes) run_passes[run] = passes;
    }
    c.phase = 0;
    if (started > 1) {
        ko_bar_wait(&c.bar);
        for (uint32_t t = 1; t < started; ++t) pthread_join(th[t], NULL);
    }
    pthread_mutex_destroy(&c.bar.mu);
    pthread_cond_destroy(&c.bar.cv);
    /* output of the last run, both directions, original labels (as ko_ktruss) */
    {
        uint32_t w = 0;
        for (uint32_t e = 0; e < m; ++e)
            if (g.dst[e] != KO_DELETED) { out_src[w] = g.src[e]; out_dst[w] = g.dst[e]; ++w; }
        const uint32_t nd = w;
        for (uint32_t e = 0; e < nd; ++e) { out_src[w] = out_dst[e]; out_dst[w] = out_src[e]; ++w; }
        for (uint32_t e = 0; e < w; ++e) { out_src[e] = new2old[out_src[e]]; out_dst[e] = new2old[out_dst[e]]; }
        *out_num = runs ? w : 0;
    }
    rc = 0;
done:
    free(s); free(d); free(new2old); free(ds); free(dd); free(pristine); free(c.tri);
    csr_free(&g);
    return rc;
}

/* ---- R-MAT generator ------------------------------------------------------------------------
 * Restates the engine's seeded kt_gen_rmat draw for draw: every random decision is a
 * SplitMix64-finalised counter (key = mix(seed ^ mix(stream + C)), draw i = mix(key + i * G)),
 * edge i takes draws 32 i + l for its levels l = 0 .. scale-1, and a draw r picks the quadrant
 * by integer thresholds t_a = floor(a 2^64), t_ab, t_abc: source bit = r >= t_ab, destination
 * bit = (t_a <= r < t_ab) or r >= t_abc.  Pairs are made canonical (min, max), sorted, and
 * duplicates and self loops dropped. */
static inline uint64_t ko_mix64(uint64_t z) {
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

static uint64_t ko_threshold(double p) {
    if (!(p > 0.0)) return 0;
    if (p >= 1.0) return UINT64_MAX;
    return (uint64_t)(p * 18446744073709551616.0);
}

/* LSD radix sort of keys on their low `bits` bits, 8 bits per pass. */
static int ko_radix_sort(uint64_t* keys, uint64_t n, unsigned bits) {
    uint64_t* tmp = (uint64_t*)malloc(sizeof(uint64_t) * (n ? n : 1));
    if (!tmp) return -1;
    uint64_t *from = keys, *to = tmp;
    for (unsigned shift = 0; shift < bits; shift += 8) {
        uint64_t cnt[257];
        memset(cnt, 0, sizeof(cnt));
        for (uint64_t i = 0; i < n; ++i) cnt[((from[i] >> shift) & 255u) + 1]++;
        for (int d = 0; d < 256; ++d) cnt[d + 1] += cnt[d];
        for (uint64_t i = 0; i < n; ++i) to[cnt[(from[i] >> shift) & 255u]++] = from[i];
        uint64_t* t = from; from = to; to = t;
    }
    if (from != keys) memcpy(keys, from, sizeof(uint64_t) * n);
    free(tmp);
    return 0;
}

int ko_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
                uint32_t* u, uint32_t* v, uint64_t* num_edges) {
    if (scale == 0 || scale > 31 || edge_factor == 0 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0) return -1;
    const uint64_t m = (uint64_t)edge_factor << scale;
    const uint64_t ta = ko_threshold(a), tab = ko_threshold(a + b), tabc = ko_threshold(a + b + c);
    const uint64_t key = ko_mix64(seed ^ ko_mix64(1ull + 0x5851f42d4c957f2dull)); /* stream 1 */
    uint64_t* keys = (uint64_t*)malloc(sizeof(uint64_t) * (m ? m : 1));
    if (!keys) return -1;
    for (uint64_t i = 0; i < m; ++i) {
        uint32_t s = 0, d = 0;
        for (uint32_t l = 0; l < scale; ++l) {
            const uint64_t r = ko_mix64(key + (i * 32 + l) * 0x9e3779b97f4a7c15ull);
            const uint32_t sb = r >= tab, db = (r >= ta && r < tab) || r >= tabc;
            s |= sb << l;
            d |= db << l;
        }
        const uint32_t lo = s < d ? s : d, hi = s < d ? d : s;
        keys[i] = ((uint64_t)lo << scale) | hi;
    }
    if (ko_radix_sort(keys, m, 2 * scale)) { free(keys); return -1; }
    const uint64_t vmask = (1ull << scale) - 1;
    uint64_t w = 0;
    for (uint64_t i = 0; i < m; ++i) {
        const uint64_t k = keys[i];
        if ((k >> scale) == (k & vmask)) continue;
        if (w > 0 && keys[w - 1] == k) continue;
        keys[w++] = k;
    }
    for (uint64_t i = 0; i < w; ++i) { u[i] = (uint32_t)(keys[i] >> scale); v[i] = (uint32_t)(keys[i] & vmask); }
    *num_edges = w;
    free(keys);
    return 0;
}
