// Calls the reference's own host tiled builder (coo2tiledcoocsr in its compiled graph.o) on an
// entry list read from stdin ("n m T" then m lines "src dst") and prints the tiled arrays, so that
// tests can pin the oracle's restatement to it.  The two structs are declared here with the
// reference's field order (graph.h) so that the linker finds the same C++ symbols.
#include <cstdio>
#include <cstdlib>

struct COOGraph {
    unsigned int numNodes;
    unsigned int numEdges;
    unsigned int capacity;
    unsigned int* srcIdx;
    unsigned int* dstIdx;
};

struct TiledCOOCSRGraph {
    unsigned int numNodes;
    unsigned int numEdges;
    unsigned int tilesPerDim;
    unsigned int tileSize;
    unsigned int capacity;
    unsigned int* tileSrcPtr;
    unsigned int* srcIdx;
    unsigned int* dstIdx;
};

struct TiledCOOCSRGraph* createEmptyTiledCOOCSR(unsigned int numNodes, unsigned int tilesPerDim, unsigned int capacity);
void coo2tiledcoocsr(struct COOGraph* cooGraph, struct TiledCOOCSRGraph* graph);

int main() {
    unsigned int n, m, t;
    if (scanf("%u %u %u", &n, &m, &t) != 3) return 1;
    COOGraph g;
    g.numNodes = n;
    g.numEdges = m;
    g.capacity = m ? m : 1;
    g.srcIdx = (unsigned int*)malloc(sizeof(unsigned int) * g.capacity);
    g.dstIdx = (unsigned int*)malloc(sizeof(unsigned int) * g.capacity);
    for (unsigned int i = 0; i < m; ++i)
        if (scanf("%u %u", &g.srcIdx[i], &g.dstIdx[i]) != 2) return 1;
    TiledCOOCSRGraph* tg = createEmptyTiledCOOCSR(n, t, g.capacity);
    coo2tiledcoocsr(&g, tg);
    const unsigned int rows = tg->tilesPerDim * tg->tilesPerDim * tg->tileSize;
    printf("%u %u\n", tg->tileSize, rows);
    for (unsigned int r = 0; r <= rows; ++r) printf("%u\n", tg->tileSrcPtr[r]);
    for (unsigned int i = 0; i < m; ++i) printf("%u %u\n", tg->srcIdx[i], tg->dstIdx[i]);
    return 0;
}
