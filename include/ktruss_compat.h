// ktruss_compat.h — C++ declarations with the same names and memory layout as KTrussExplorer's
// k-truss entry point and structs, so that code written against the reference links against
// libktruss_compat.so unchanged:
//   struct COOGraph                       graph.h:10-16
//   enum Processor, Directedness,
//        InputFormat, Recount             config.h:51-161 (same enumerator values)
//   struct Config                         config.h:163-181
//   void ktruss(COOGraph*, COOGraph*, Config)   kernel.h:12
// The reference's own config.h/graph.h declare the same types; use one or the other.
#ifndef KTRUSS_COMPAT_H
#define KTRUSS_COMPAT_H

struct COOGraph {
    unsigned int numNodes;
    unsigned int numEdges;
    unsigned int capacity;
    unsigned int* srcIdx;
    unsigned int* dstIdx;
};

enum Processor { CPU, GPU };
enum Directedness { UNDIRECTED, DIRECTED_BY_INDEX, DIRECTED_BY_DEGREE };
enum InputFormat { COOCSR, TILED_COOCSR };
enum Recount { ALL, AFFECTED };

struct Config {
    const char* graphFileName;
    unsigned int k;
    const char* compareFileName;
    const char* outFileName;
    unsigned int numWarmupRuns;
    unsigned int numTimedRuns;
    Processor processor;
    Directedness directedness;
    InputFormat inputFormat;
    unsigned int numEdgeRemoveIter;
    Recount recount;
    unsigned int blockSize;
    unsigned int numTiles;
    unsigned int numParallelTiles;
    unsigned int verbosity;
    unsigned int numNodes;
    unsigned int numEdges;
};

// k-truss of `graph` into `truss` (capacity >= graph->numEdges), both directions, 0-based ids.
// Runs the GB300 engine; on an error it prints the message and aborts, as the reference's
// asserts do.  Unlike the reference, `graph` is left unchanged (not relabeled in place).
void ktruss(COOGraph* graph, COOGraph* truss, Config config);

#endif
