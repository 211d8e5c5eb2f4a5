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

    peel_loop(&g, k, directed, recount, num_edge_remove_iter, &in, slots, log);

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
 * prune passes of the reference loop, so the pass statistics of ko_decompose_chain follow. */
int ko_decompose_peel(uint32_t num_nodes, uint32_t num_entries, const uint32_t* src,
                      const uint32_t* dst, uint32_t* truss_per_entry, uint32_t* k_max,
                      uint32_t* plain_passes, uint64_t* plain_alive_sum, uint32_t* num_rounds) {
    int rc = -1;
    uint32_t m = 0, n = num_nodes;
    uint64_t* keys = NULL;
    uint32_t *ptr = NULL, *col = NULL, *eid = NULL, *fill = NULL, *sup = NULL, *rnd = NULL, *tr = NULL;
    uint32_t *F = NULL, *NF = NULL;
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
    if (!ptr || !col || !eid || !fill || !sup || !rnd || !tr || !F || !NF) goto done;
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
    /* rows: smaller neighbours were appended first (ascending), then larger ones (ascending) */
    for (uint32_t e = 0; e < m; ++e) {
        uint32_t u = (uint32_t)(keys[e] >> 32), v = (uint32_t)keys[e];
        uint32_t a = ptr[u], ae = ptr[u + 1], b = ptr[v], be = ptr[v + 1];
        while (a < ae && b < be) {
            if (col[a] < col[b]) ++a;
            else if (col[a] > col[b]) ++b;
            else { sup[e]++; ++a; ++b; }
        }
    }
    /* Pass statistics of the reference chain (ko_decompose_chain): level 3 is one pass over
     * all m edges (kernel_hdc.cu:169-172 stops after the first pass); each level k >= 4 up to
     * k_max+1 takes one pass per round that removes edges plus a final pass that removes
     * nothing, each pass seeing the edges alive at its start. */
    uint64_t alive = m, alive_sum = m;
    uint32_t k = 3, r = 0, passes = m ? 1 : 0;
    while (alive) {
        uint32_t nf = 0, mn = 0xffffffffu;
        for (uint32_t e = 0; e < m; ++e)
            if (!rnd[e]) { if (sup[e] < k - 2) F[nf++] = e; if (sup[e] < mn) mn = sup[e]; }
        if (!nf) {
            /* levels k .. mn+2 remove nothing: one pass each (levels >= 4) */
            for (uint32_t kk = k > 3 ? k : 4; kk < mn + 3; ++kk) { passes++; alive_sum += alive; }
            k = mn + 3;
            continue;
        }
        while (nf) {
            if (k >= 4) { passes++; alive_sum += alive; }
            ++r;
            for (uint32_t i = 0; i < nf; ++i) { rnd[F[i]] = r; tr[F[i]] = k - 1; }
            uint32_t nn = 0;
            for (uint32_t i = 0; i < nf; ++i) {
                uint32_t e = F[i];
                uint32_t u = (uint32_t)(keys[e] >> 32), v = (uint32_t)keys[e];
                uint32_t a = ptr[u], ae = ptr[u + 1], b = ptr[v], be = ptr[v + 1];
                while (a < ae && b < be) {
                    if (col[a] < col[b]) { ++a; continue; }
                    if (col[a] > col[b]) { ++b; continue; }
                    uint32_t x = eid[a], y = eid[b];
                    ++a; ++b;
                    if ((rnd[x] && rnd[x] != r) || (rnd[y] && rnd[y] != r)) continue; /* already gone */
                    if ((rnd[x] == r && x < e) || (rnd[y] == r && y < e)) continue;     /* owned by a smaller id */
                    if (!rnd[x] && sup[x]-- == k - 2) NF[nn++] = x;
                    if (!rnd[y] && sup[y]-- == k - 2) NF[nn++] = y;
                }
            }
            alive -= nf;
            uint32_t* t = F; F = NF; NF = t;
            nf = nn;
        }
        if (k >= 4) { passes++; alive_sum += alive; }
        ++k;
    }
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
    return rc;
}
