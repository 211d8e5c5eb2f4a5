// Drives the reference's own k-truss entry point, `void ktruss(COOGraph*, COOGraph*, Config)`
// (kernel.h:12), compiled from its unmodified sources, over many configurations of one graph that is
// read once with the reference's own reader (createCOOFromFile, graph.cu:37-79).  Configurations
// are command lines of the reference CLI, parsed by its own parseArgs (config.h:183-224), one per
// line on standard input.  A line "chain <K> <options>" instead decomposes the graph by chaining
// single-k runs k = 3, 4, ..., K (each on the previous output) with the options that follow.  K is
// the graph's k_max: the reference's GPU path cannot run the level after it, whose k-truss is
// empty (with no edge left, removeCOOCSRDeletedEdgesOnDevice launches histogram_kernel with zero
// blocks, graph.cu:541, and the thrust scan that follows aborts on that launch error).
//
// Output per run (the reference prints its own "<CSV config>, <ms> ms" lines with -v 0):
//   RESULT k=<k> edges=<undirected truss edges> hash=<order-free hash of the edge set>
// so a caller can check the edge sets against another implementation.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "config.h"
#include "graph.h"
#include "kernel.h"

namespace {

uint64_t mix(uint64_t z) {
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

// Undirected edge count and an order-free hash (sum of mixed canonical keys) of a COO edge set.
void summarize(const COOGraph* t, unsigned* edges, uint64_t* hash) {
    uint64_t h = 0;
    unsigned c = 0;
    for (unsigned e = 0; e < t->numEdges; ++e) {
        const unsigned a = t->srcIdx[e], b = t->dstIdx[e];
        if (a < b) {
            h += mix(((uint64_t)a << 32) | b);
            ++c;
        }
    }
    *edges = c;
    *hash = h;
}

COOGraph* copy_of(const COOGraph* g) {
    COOGraph* c = createEmptyCOO(g->numNodes, g->numEdges ? g->numEdges : 1);
    c->numEdges = g->numEdges;
    std::memcpy(c->srcIdx, g->srcIdx, sizeof(unsigned) * g->numEdges);
    std::memcpy(c->dstIdx, g->dstIdx, sizeof(unsigned) * g->numEdges);
    return c;
}

Config parse_line(const std::string& line, const char* graph_file) {
    std::vector<std::string> tok{"ktruss"};
    size_t i = 0;
    while (i < line.size()) {
        while (i < line.size() && line[i] == ' ') ++i;
        size_t j = i;
        while (j < line.size() && line[j] != ' ') ++j;
        if (j > i) tok.push_back(line.substr(i, j - i));
        i = j;
    }
    std::vector<char*> argv;
    for (auto& t : tok) argv.push_back(&t[0]);
    optind = 1;
    Config c = parseArgs((int)argv.size(), argv.data());
    c.graphFileName = graph_file;
    return c;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s <graph.tsv> < configurations\n", argv[0]);
        return 2;
    }
    COOGraph* graph = createCOOFromFile(argv[1]);
    std::fprintf(stderr, "read %u vertices, %u entries\n", graph->numNodes, graph->numEdges);
    char buf[4096];
    while (std::fgets(buf, sizeof(buf), stdin)) {
        std::string line(buf);
        while (!line.empty() && (line.back() == '\n' || line.back() == '\r')) line.pop_back();
        if (line.empty()) continue;
        const bool chain = line.compare(0, 5, "chain") == 0;
        unsigned last_k = 0;
        std::string opts = line;
        if (chain) {
            opts = line.substr(5);
            size_t i = opts.find_first_not_of(' ');
            last_k = (unsigned)std::strtoul(opts.c_str() + (i == std::string::npos ? 0 : i), nullptr, 10);
            i = opts.find(' ', i == std::string::npos ? 0 : i);
            opts = i == std::string::npos ? std::string() : opts.substr(i);
        }
        Config c = parse_line(opts, argv[1]);
        if (!chain) {
            COOGraph* g = copy_of(graph);  // ktruss relabels its input in place (kernel.cu:18)
            COOGraph* t = createEmptyCOO(g->numNodes, g->numEdges ? g->numEdges : 1);
            c.numNodes = g->numNodes;
            c.numEdges = g->numEdges;
            ktruss(g, t, c);
            unsigned edges;
            uint64_t h;
            summarize(t, &edges, &h);
            std::printf("RESULT k=%u edges=%u hash=%016llx\n", c.k, edges, (unsigned long long)h);
            std::fflush(stdout);
            freeCOOGraph(g);
            freeCOOGraph(t);
            continue;
        }
        COOGraph* cur = copy_of(graph);
        for (unsigned k = 3; cur->numEdges > 0 && k <= last_k; ++k) {
            COOGraph* in = copy_of(cur);
            COOGraph* t = createEmptyCOO(in->numNodes, in->numEdges);
            Config ck = c;
            ck.k = k;
            ck.numNodes = in->numNodes;
            ck.numEdges = in->numEdges;
            ktruss(in, t, ck);
            unsigned edges;
            uint64_t h;
            summarize(t, &edges, &h);
            std::printf("RESULT k=%u edges=%u hash=%016llx\n", k, edges, (unsigned long long)h);
            std::fflush(stdout);
            freeCOOGraph(in);
            freeCOOGraph(cur);
            cur = t;
        }
        freeCOOGraph(cur);
        std::printf("CHAIN DONE\n");
        std::fflush(stdout);
    }
    freeCOOGraph(graph);
    return 0;
}
