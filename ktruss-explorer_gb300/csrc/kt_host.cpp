// Host side of the drop-in boundary: errors, configuration (config.h), graph I/O (graph.cu)
// and verification (verify.cu).  No CUDA here.

#include "kt_internal.h"

#include <algorithm>
#include <cerrno>
#include <cstdarg>
#include <cstdlib>
#include <cstring>
#include <getopt.h>
#include <thread>
#include <vector>

namespace kt {

// Fixed-size per-thread message buffer: recording an error never touches the heap.
static thread_local char g_last_error[1024];

int fail(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
    return code;
}

void clear_error() { g_last_error[0] = '\0'; }

}  // namespace kt

using kt::fail;

extern "C" {

const char* kt_last_error(void) { return kt::g_last_error; }

const char* kt_status_string(int s) {
    switch (s) {
        case KT_OK: return "ok";
        case KT_ERR_INVALID_ARG: return "invalid argument";
        case KT_ERR_SELF_LOOP: return "self loop in input";
        case KT_ERR_NOT_SYMMETRIC: return "input is not a symmetric simple graph";
        case KT_ERR_CAPACITY: return "output capacity too small";
        case KT_ERR_UNSUPPORTED: return "unsupported configuration";
        case KT_ERR_CUDA: return "CUDA error";
        case KT_ERR_DEVICE_ALLOC: return "device allocation failed";
        case KT_ERR_HOST_ALLOC: return "host allocation failed";
        case KT_ERR_IO: return "I/O error";
        case KT_ERR_MISMATCH: return "verification mismatch";
        case KT_ERR_TIMEOUT: return "device wait timed out";
        case KT_ERR_NO_DEVICE: return "no CUDA device";
        case KT_ERR_TOO_LARGE: return "graph too large";
        case KT_ERR_INTERNAL: return "internal consistency check failed";
        default: return "unknown status";
    }
}

// ---- configuration: config.h ---------------------------------------------------------------

void kt_config_default(kt_config* c) {
    if (!c) return;
    // parseArgs defaults (config.h:184-199)
    c->graph_file_name = "data/loc-gowalla_edges_adj.tsv";
    c->k = 3;
    c->compare_file_name = "data/loc-gowalla_edges_adj.tsv.3.reference.tsv";
    c->out_file_name = nullptr;
    c->num_warmup_runs = 0;
    c->num_timed_runs = 1;
    c->processor = KT_PROCESSOR_GPU;
    c->directedness = KT_DIRECTED_BY_DEGREE;
    c->input_format = KT_FORMAT_COOCSR;
    c->num_edge_remove_iter = 0;
    c->recount = KT_RECOUNT_ALL;
    c->block_size = 512;
    c->num_tiles = 8;
    c->num_parallel_tiles = 8;
    c->verbosity = 1;
    c->num_nodes = 0;
    c->num_edges = 0;
}

void kt_print_usage(void) {
    // usage() text of config.h:11-49
    fprintf(stderr,
            "\nUsage:  ./ktruss [options]"
            "\n"
            "\nOptions:"
            "\n    -g <graphFileName>       Name of file with input graph (default = data/loc-gowalla_edges_adj.tsv)"
            "\n    -k <k>                   k (default = 3)"
            "\n    -c <compareFileName>     Name of file to compare to when verifying result (default = data/loc-gowalla_edges_adj.tsv.3.reference.tsv)"
            "\n    -o <outFileName>         Name of ouput file to write result to (by default, the result will not be written to a file)"
            "\n    -w <numWarmupRuns>       Number of warmup runs (default = 0)"
            "\n    -x <numTimedRuns>        Number of timed runs (default = 1)"
            "\n    -p <processor>           Processor to run on. Options:"
            "\n                                 cpu - CPU"
            "\n                                 gpu - GPU (default)"
            "\n    -d <directedness>        Directedness of graph. Options:"
            "\n                                 undirected - use undirected graph as is"
            "\n                                 directed-by-index - only keep edges from vertices with lower index to vertices with higher index"
            "\n                                 directed-by-degree - only keep edges from lower degree vertices to higher degree vertices (default)"
            "\n    -f <inputFormat>         Format of the graph. Options:"
            "\n                                 coocsr - convert to hybrid COO/CSR graph before processing (default)"
            "\n                                 tiled-coocsr - convert to hybrid COO/CSR graph with tiling before processing"
            "\n    -e <numEdgeRemoveIter>   Number of initial iterations during which edges are to be removed (default = 0)"
            "\n    -r <recount>             Which edges to recount triangles for. Options:"
            "\n                                 all - recount triangles for all undeleted edges every iteration (default)"
            "\n                                 affected - recount triangles for only edges affected by deletions in the previous iteration"
            "\n    -b <blockSize>           Number of threads per block in k-truss kernel (default = 512)"
            "\n                                 NOTE: -b only has effect with option: -p gpu"
            "\n    -t <numTiles>            Number of tiles for tiled COO/CSR (default = 8)"
            "\n                                 NOTE: -t only has effect with option: -f tiled-coocsr"
            "\n    -y <numParallelTiles>    Number of tiles for tiled COO/CSR to process in parallel on the GPU (default = 8)"
            "\n                                 NOTE: -y only has effect with options: -p gpu -f tiled-coocsr"
            "\n    -v <verbosity>           Options:"
            "\n                                 0 - show k-truss time only in CSV format"
            "\n                                 1 - show allocation, copy, and conversion times (default)"
            "\n                                 2 - show per-iteration times"
            "\n    -h                       Help"
            "\n"
            "\n");
}

static int parse_enum(const char* s, const char* const* names, int count, int* out) {
    for (int i = 0; i < count; ++i)
        if (strcmp(s, names[i]) == 0) { *out = i; return 1; }
    return 0;
}

static const char* const kProcessor[] = {"cpu", "gpu"};
static const char* const kDirectedness[] = {"undirected", "directed-by-index", "directed-by-degree"};
static const char* const kFormat[] = {"coocsr", "tiled-coocsr"};
static const char* const kRecount[] = {"all", "affected"};

int kt_parse_args(int argc, char** argv, kt_config* c) {
    if (!c || argc < 0 || (argc > 0 && !argv)) return fail(KT_ERR_INVALID_ARG, "kt_parse_args: null argument");
    kt_config_default(c);
    optind = 1;
    int opt;
    // atoi semantics as in config.h:203-215 (so "-k -1" wraps to a large unsigned k)
    while ((opt = getopt(argc, argv, "g:k:o:w:x:c:p:d:f:e:r:b:t:y:v:h")) >= 0) {
        switch (opt) {
            case 'g': c->graph_file_name = optarg; break;
            case 'k': c->k = (uint32_t)atoi(optarg); break;
            case 'c': c->compare_file_name = optarg; break;
            case 'o': c->out_file_name = optarg; break;
            case 'w': c->num_warmup_runs = (uint32_t)atoi(optarg); break;
            case 'x': c->num_timed_runs = (uint32_t)atoi(optarg); break;
            case 'p':
                if (!parse_enum(optarg, kProcessor, 2, &c->processor))
                    return fail(KT_ERR_INVALID_ARG, "Unrecognized -p option: %s", optarg);
                break;
            case 'd':
                if (!parse_enum(optarg, kDirectedness, 3, &c->directedness))
                    return fail(KT_ERR_INVALID_ARG, "Unrecognized -d option: %s", optarg);
                break;
            case 'f':
                if (!parse_enum(optarg, kFormat, 2, &c->input_format))
                    return fail(KT_ERR_INVALID_ARG, "Unrecognized -f option: %s", optarg);
                break;
            case 'e': c->num_edge_remove_iter = (uint32_t)atoi(optarg); break;
            case 'r':
                if (!parse_enum(optarg, kRecount, 2, &c->recount))
                    return fail(KT_ERR_INVALID_ARG, "Unrecognized -r option: %s", optarg);
                break;
            case 'b': c->block_size = (uint32_t)atoi(optarg); break;
            case 't': c->num_tiles = (uint32_t)atoi(optarg); break;
            case 'y': c->num_parallel_tiles = (uint32_t)atoi(optarg); break;
            case 'v': c->verbosity = (uint32_t)atoi(optarg); break;
            case 'h': kt_print_usage(); return fail(KT_ERR_INVALID_ARG, "help requested");
            default: fprintf(stderr, "\nUnrecognized option!\n"); kt_print_usage();
                return fail(KT_ERR_INVALID_ARG, "Unrecognized option");
        }
    }
    return KT_OK;
}

static const char* name_of(int v, const char* const* names, int count) {
    return (v >= 0 && v < count) ? names[v] : "?";
}

void kt_print_config(const kt_config* c) {
    if (!c) return;
    // printConfig (config.h:226-245)
    printf("    Graph: %s\n", c->graph_file_name);
    printf("        # vertices = %u\n", c->num_nodes);
    printf("        # edges = %u\n", c->num_edges);
    printf("    k: %u\n", c->k);
    printf("    Processor: %s\n", name_of(c->processor, kProcessor, 2));
    if (c->processor == KT_PROCESSOR_GPU) printf("        Block size = %u\n", c->block_size);
    printf("    Directedness: %s\n", name_of(c->directedness, kDirectedness, 3));
    printf("    Input format: %s\n", name_of(c->input_format, kFormat, 2));
    if (c->input_format == KT_FORMAT_TILED_COOCSR) {
        printf("        Number of tiles = %u\n", c->num_tiles);
        if (c->processor == KT_PROCESSOR_GPU)
            printf("        Number of tiles processed in parallel = %u\n", c->num_parallel_tiles);
    }
    printf("    Number of initial iterations to remove edges: %u\n", c->num_edge_remove_iter);
    printf("    Recount strategy: %s\n", name_of(c->recount, kRecount, 2));
}

void kt_print_config_csv(const kt_config* c) {
    if (!c) return;
    // printConfigAsCSV (config.h:247-272); the caller appends "<t> ms"
    printf("%s, ", c->graph_file_name);
    printf("%u, ", c->num_nodes);
    printf("%u, ", c->num_edges);
    printf("%u, ", c->k);
    printf("%s, ", name_of(c->processor, kProcessor, 2));
    printf("%s, ", name_of(c->directedness, kDirectedness, 3));
    printf("%s, ", name_of(c->input_format, kFormat, 2));
    printf("%u, ", c->num_edge_remove_iter);
    printf("%s, ", name_of(c->recount, kRecount, 2));
    if (c->processor == KT_PROCESSOR_GPU) printf("%u, ", c->block_size);
    else printf("N/A, ");
    if (c->input_format == KT_FORMAT_TILED_COOCSR) {
        printf("%u, ", c->num_tiles);
        if (c->processor == KT_PROCESSOR_GPU) printf("%u, ", c->num_parallel_tiles);
        else printf("N/A, ");
    } else {
        printf("N/A, N/A, ");
    }
}

// ---- graph I/O: graph.cu ---------------------------------------------------------------------

int kt_coo_alloc(uint32_t num_nodes, uint32_t capacity, kt_coo* out) {
    if (!out) return fail(KT_ERR_INVALID_ARG, "kt_coo_alloc: null output");
    out->num_nodes = num_nodes;
    out->num_edges = 0;
    out->capacity = capacity;
    out->src_idx = (uint32_t*)malloc(sizeof(uint32_t) * (capacity ? capacity : 1));
    out->dst_idx = (uint32_t*)malloc(sizeof(uint32_t) * (capacity ? capacity : 1));
    if (!out->src_idx || !out->dst_idx) {
        free(out->src_idx);
        free(out->dst_idx);
        out->src_idx = out->dst_idx = nullptr;
        return fail(KT_ERR_HOST_ALLOC, "kt_coo_alloc: cannot allocate %u entries", capacity);
    }
    return KT_OK;
}

void kt_coo_free(kt_coo* g) {
    if (!g) return;
    free(g->src_idx);
    free(g->dst_idx);
    g->src_idx = g->dst_idx = nullptr;
    g->num_edges = g->capacity = 0;
}

// Fast unsigned decimal scanner over a memory buffer; returns false at end of input.
static bool next_uint(const char*& p, const char* end, uint64_t* v, bool* ok) {
    while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
    if (p >= end) return false;
    if (*p < '0' || *p > '9') { *ok = false; return false; }
    uint64_t x = 0;
    while (p < end && *p >= '0' && *p <= '9') {
        x = x * 10 + (uint64_t)(*p - '0');
        if (x > 0xffffffffull) { *ok = false; return false; }
        ++p;
    }
    *v = x;
    return true;
}

int kt_read_tsv(const char* path, kt_coo* out) {
    // createCOOFromFile (graph.cu:37-79): triples "dst src x", 1-based ids, x ignored
    if (!path || !out) return fail(KT_ERR_INVALID_ARG, "kt_read_tsv: null argument");
    memset(out, 0, sizeof(*out));
    FILE* fp = fopen(path, "rb");
    if (!fp) return fail(KT_ERR_IO, "cannot open %s: %s", path, strerror(errno));
    std::vector<char> buf;
    {
        fseek(fp, 0, SEEK_END);
        long sz = ftell(fp);
        fseek(fp, 0, SEEK_SET);
        if (sz < 0) { fclose(fp); return fail(KT_ERR_IO, "cannot size %s", path); }
        buf.resize((size_t)sz);
        if (sz > 0 && fread(buf.data(), 1, (size_t)sz, fp) != (size_t)sz) {
            fclose(fp);
            return fail(KT_ERR_IO, "short read on %s", path);
        }
        fclose(fp);
    }
    std::vector<uint32_t> s, d;
    const char* p = buf.data();
    const char* end = p + buf.size();
    uint32_t num_nodes = 0;
    bool ok = true;
    uint64_t a, b, x;
    uint64_t line = 0;
    while (next_uint(p, end, &a, &ok)) {
        ++line;
        if (!next_uint(p, end, &b, &ok) || !next_uint(p, end, &x, &ok))
            return fail(KT_ERR_IO, "%s: entry %llu is not a 'dst src x' triple", path, (unsigned long long)line);
        if (a == 0 || b == 0) return fail(KT_ERR_IO, "%s: entry %llu has a 0 vertex id (ids are 1-based)", path, (unsigned long long)line);
        if (a == b) return fail(KT_ERR_SELF_LOOP, "%s: entry %llu: Edges from a vertex to itself are not allowed!", path, (unsigned long long)line);
        if (s.size() >= 0xffffffffull) return fail(KT_ERR_TOO_LARGE, "%s: more than 2^32-1 entries", path);
        d.push_back((uint32_t)(a - 1));
        s.push_back((uint32_t)(b - 1));
        if (a > num_nodes) num_nodes = (uint32_t)a;
        if (b > num_nodes) num_nodes = (uint32_t)b;
    }
    if (!ok) return fail(KT_ERR_IO, "%s: malformed number after entry %llu", path, (unsigned long long)line);
    int rc = kt_coo_alloc(num_nodes, (uint32_t)s.size(), out);
    if (rc) return rc;
    memcpy(out->src_idx, s.data(), sizeof(uint32_t) * s.size());
    memcpy(out->dst_idx, d.data(), sizeof(uint32_t) * d.size());
    out->num_edges = (uint32_t)s.size();
    return KT_OK;
}

// Decimal digits of x at p; returns the end.
static char* put_u64(char* p, uint64_t x) {
    char tmp[20];
    int n = 0;
    do {
        tmp[n++] = (char)('0' + x % 10);
        x /= 10;
    } while (x);
    while (n) *p++ = tmp[--n];
    return p;
}

// Lines "dst+1 \t src+1 \t third" of entries [e0, e1) into out (at most 33 bytes a line).
static size_t format_entries(const kt_coo* g, const uint32_t* third, uint64_t e0, uint64_t e1, char* out) {
    char* p = out;
    for (uint64_t e = e0; e < e1; ++e) {
        p = put_u64(p, (uint64_t)g->dst_idx[e] + 1);
        *p++ = '\t';
        p = put_u64(p, (uint64_t)g->src_idx[e] + 1);
        *p++ = '\t';
        p = put_u64(p, third ? third[e] : 1u);
        *p++ = '\n';
    }
    return (size_t)(p - out);
}

// The reference writes one fprintf per entry (graph.cu:96-104); here batches of entries are
// formatted by all host threads, each into its own buffer, and written in order.
static int write_entries(const kt_coo* g, const uint32_t* third, const char* path) {
    FILE* fp = fopen(path, "wb");
    if (!fp) return fail(KT_ERR_IO, "cannot open %s for writing: %s", path, strerror(errno));
    const uint64_t m = g->num_edges;
    const unsigned hw = std::thread::hardware_concurrency();
    const uint64_t threads = std::max<uint64_t>(1, std::min<uint64_t>(hw ? hw : 1, 32));
    const uint64_t per = 1u << 18;  // entries per thread and batch
    std::vector<std::vector<char>> bufs(threads, std::vector<char>(per * 33));
    std::vector<size_t> used(threads);
    bool failed = false;
    for (uint64_t b0 = 0; b0 < m && !failed; b0 += per * threads) {
        std::vector<std::thread> pool;
        for (uint64_t t = 0; t < threads; ++t) {
            const uint64_t e0 = std::min(m, b0 + t * per), e1 = std::min(m, e0 + per);
            used[t] = 0;
            if (e0 < e1) pool.emplace_back([&, t, e0, e1] { used[t] = format_entries(g, third, e0, e1, bufs[t].data()); });
        }
        for (auto& th : pool) th.join();
        for (uint64_t t = 0; t < threads && !failed; ++t)
            if (used[t] && fwrite(bufs[t].data(), 1, used[t], fp) != used[t]) failed = true;
    }
    if (fclose(fp) != 0 || failed) return fail(KT_ERR_IO, "write to %s failed", path);
    return KT_OK;
}

int kt_write_tsv(const kt_coo* g, const char* path) {
    // writeCOOGraphToFile (graph.cu:96-104)
    if (!g || !path) return fail(KT_ERR_INVALID_ARG, "kt_write_tsv: null argument");
    return write_entries(g, nullptr, path);
}

int kt_write_truss_tsv(const kt_coo* g, const uint32_t* truss, const char* path) {
    if (!g || !truss || !path) return fail(KT_ERR_INVALID_ARG, "kt_write_truss_tsv: null argument");
    return write_entries(g, truss, path);
}

// ---- verify: verify.cu -----------------------------------------------------------------------

int kt_verify(const kt_coo* truss, const kt_config* c) {
    // verify.cu:12-40: read the comparison file, compare counts, then compare both edge lists in
    // a canonical order (coo2coocsr sorts each row).  Sorting all (src, dst) pairs gives the
    // same canonical order.
    if (!truss || !c || !c->compare_file_name) return fail(KT_ERR_INVALID_ARG, "kt_verify: null argument");
    kt_coo ref;
    int rc = kt_read_tsv(c->compare_file_name, &ref);
    if (rc) return rc;
    if (ref.num_edges != truss->num_edges) {
        uint32_t a = truss->num_edges, b = ref.num_edges;
        kt_coo_free(&ref);
        return fail(KT_ERR_MISMATCH, "edge count %u differs from %u in %s", a, b, c->compare_file_name);
    }
    std::vector<uint64_t> x(truss->num_edges), y(ref.num_edges);
    for (uint32_t i = 0; i < truss->num_edges; ++i) x[i] = ((uint64_t)truss->src_idx[i] << 32) | truss->dst_idx[i];
    for (uint32_t i = 0; i < ref.num_edges; ++i) y[i] = ((uint64_t)ref.src_idx[i] << 32) | ref.dst_idx[i];
    kt_coo_free(&ref);
    std::sort(x.begin(), x.end());
    std::sort(y.begin(), y.end());
    for (size_t i = 0; i < x.size(); ++i)
        if (x[i] != y[i])
            return fail(KT_ERR_MISMATCH, "edge (%u,%u) differs from reference (%u,%u)", (uint32_t)(x[i] >> 32) + 1,
                        (uint32_t)x[i] + 1, (uint32_t)(y[i] >> 32) + 1, (uint32_t)y[i] + 1);
    if (c->verbosity >= 1) printf("    PASSED\n");
    return KT_OK;
}

}  // extern "C"
