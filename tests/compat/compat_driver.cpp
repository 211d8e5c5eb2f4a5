// Test driver for libktruss_compat.so, written only against ktruss_compat.h (the reference's
// structs and entry point): reads a "dst src x" TSV, calls ktruss() and prints the truss edges.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "ktruss_compat.h"

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    FILE* fp = std::fopen(argv[1], "r");
    if (!fp) return 2;
    std::vector<unsigned> src, dst;
    unsigned a, b, x, n = 0;
    while (std::fscanf(fp, "%u %u %u", &a, &b, &x) == 3) {
        dst.push_back(a - 1);
        src.push_back(b - 1);
        n = a > n ? a : n;
        n = b > n ? b : n;
    }
    std::fclose(fp);
    COOGraph g{n, (unsigned)src.size(), (unsigned)src.size(), src.data(), dst.data()};
    std::vector<unsigned> ts(src.size() + 1), td(src.size() + 1);
    COOGraph t{n, 0, (unsigned)src.size(), ts.data(), td.data()};
    Config c{};
    c.graphFileName = argv[1];
    c.k = (unsigned)std::atoi(argv[2]);
    c.compareFileName = "";
    c.numTimedRuns = 1;
    c.processor = GPU;
    c.directedness = DIRECTED_BY_DEGREE;
    c.inputFormat = COOCSR;
    c.recount = ALL;
    c.blockSize = 512;
    c.numTiles = 8;
    c.numParallelTiles = 8;
    c.verbosity = 1;
    c.numNodes = g.numNodes;
    c.numEdges = g.numEdges;
    ktruss(&g, &t, c);
    for (unsigned i = 0; i < t.numEdges; ++i) std::printf("%u %u\n", t.srcIdx[i], t.dstIdx[i]);
    return 0;
}
