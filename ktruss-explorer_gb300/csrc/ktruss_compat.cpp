// libktruss_compat.so: the reference's C++ entry point `void ktruss(COOGraph*, COOGraph*, Config)`
// (kernel.h:12) over the C ABI of libktruss_gb300, for programs built against the reference's
// headers (main.cu:31 calls it).

#include "ktruss_compat.h"

#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "ktruss_gb300.h"

static_assert(sizeof(COOGraph) == sizeof(kt_coo), "COOGraph layout");
static_assert(offsetof(COOGraph, srcIdx) == offsetof(kt_coo, src_idx), "COOGraph layout");
static_assert(offsetof(COOGraph, dstIdx) == offsetof(kt_coo, dst_idx), "COOGraph layout");
static_assert(sizeof(Config) == sizeof(kt_config), "Config layout");
static_assert(offsetof(Config, processor) == offsetof(kt_config, processor), "Config layout");
static_assert(offsetof(Config, recount) == offsetof(kt_config, recount), "Config layout");
static_assert(offsetof(Config, numEdges) == offsetof(kt_config, num_edges), "Config layout");
static_assert((int)GPU == KT_PROCESSOR_GPU && (int)DIRECTED_BY_DEGREE == KT_DIRECTED_BY_DEGREE &&
                  (int)TILED_COOCSR == KT_FORMAT_TILED_COOCSR && (int)AFFECTED == KT_RECOUNT_AFFECTED,
              "enum values");

void ktruss(COOGraph* graph, COOGraph* truss, Config config) {
    kt_coo in, out;
    kt_config c;
    std::memcpy(&in, graph, sizeof in);
    std::memcpy(&out, truss, sizeof out);
    std::memcpy(&c, &config, sizeof c);
    const int rc = kt_ktruss(&in, &out, &c);
    if (rc != KT_OK) {
        std::fprintf(stderr, "ktruss: %s (%s)\n", kt_last_error(), kt_status_string(rc));
        std::abort();
    }
    truss->numNodes = out.num_nodes;
    truss->numEdges = out.num_edges;
}
