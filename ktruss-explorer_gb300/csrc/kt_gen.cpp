// Seeded synthetic graph generators (host C++).
//
// The reference ships no data: its default GraphChallenge input and the matching
// `*.3.reference.tsv` are external (config.h:185-187, .gitignore:3).  These generators
// produce the seeded stand-ins the k-truss engine is tested and measured on: Erdos-Renyi,
// R-MAT, Barabasi-Albert, Watts-Strogatz, random geometric graphs and planted cliques.
//
// Every random decision is drawn from a counter-based hash (SplitMix64 finaliser of
// seed/stream/counter), and every comparison is done on integers or on doubles whose
// computation is exact, so the same seed gives the same graph on x86-64 and AArch64.
// This file must be compiled with -ffp-contract=off (the random geometric generator
// compares squared distances and must not be contracted into FMAs).
//
// Output: canonical undirected simple graphs, i.e. pairs u < v, sorted by (u, v),
// without duplicates or self loops.  Both directions (the reference's COO convention,
// graph.cu:37-79) are produced by the caller when needed.

#include "kt_internal.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <unordered_set>
#include <vector>

namespace {

inline uint64_t mix64(uint64_t z) {
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

// Independent streams per generator phase; counter i selects the draw.
struct Rng {
    uint64_t key;
    Rng(uint64_t seed, uint64_t stream) : key(mix64(seed ^ mix64(stream + 0x5851f42d4c957f2dull))) {}
    uint64_t at(uint64_t i) const { return mix64(key + i * 0x9e3779b97f4a7c15ull); }
};

// Probability p in [0,1] as a threshold on a uniform 64-bit draw (draw < t  <=>  success).
inline uint64_t prob_threshold(double p) {
    if (!(p > 0.0)) return 0;
    if (p >= 1.0) return UINT64_MAX;
    return (uint64_t)(p * 18446744073709551616.0);
}

// Uniform integer in [0, n) from a 64-bit draw (multiply-high; bias below 2^-32 for n < 2^32).
inline uint32_t bounded(uint64_t r, uint32_t n) {
    return (uint32_t)(((unsigned __int128)r * n) >> 64);
}

inline uint64_t pack(uint32_t a, uint32_t b) {
    uint32_t u = a < b ? a : b, v = a < b ? b : a;
    return ((uint64_t)u << 32) | v;
}

unsigned worker_count() {
    unsigned t = std::thread::hardware_concurrency();
    if (t == 0) t = 1;
    return t > 32 ? 32 : t;
}

// LSD radix sort of 64-bit keys on the low `bits` bits, multi-threaded per pass.
void radix_sort_u64(std::vector<uint64_t>& keys, unsigned bits) {
    const size_t n = keys.size();
    if (n < (1u << 16)) { std::sort(keys.begin(), keys.end()); return; }
    std::vector<uint64_t> tmp(n);
    const unsigned T = worker_count();
    const size_t chunk = (n + T - 1) / T;
    std::vector<size_t> hist((size_t)T * 2048);
    for (unsigned shift = 0; shift < bits; shift += 11) {
        std::fill(hist.begin(), hist.end(), 0);
        std::vector<std::thread> th;
        for (unsigned t = 0; t < T; ++t)
            th.emplace_back([&, t] {
                size_t lo = t * chunk, hi = std::min(n, lo + chunk);
                size_t* h = &hist[(size_t)t * 2048];
                for (size_t i = lo; i < hi; ++i) ++h[(keys[i] >> shift) & 2047];
            });
        for (auto& x : th) x.join();
        th.clear();
        size_t sum = 0;
        for (unsigned d = 0; d < 2048; ++d)
            for (unsigned t = 0; t < T; ++t) {
                size_t c = hist[(size_t)t * 2048 + d];
                hist[(size_t)t * 2048 + d] = sum;
                sum += c;
            }
        for (unsigned t = 0; t < T; ++t)
            th.emplace_back([&, t] {
                size_t lo = t * chunk, hi = std::min(n, lo + chunk);
                size_t* h = &hist[(size_t)t * 2048];
                for (size_t i = lo; i < hi; ++i) tmp[h[(keys[i] >> shift) & 2047]++] = keys[i];
            });
        for (auto& x : th) x.join();
        keys.swap(tmp);
    }
}

unsigned bits_for(uint64_t n) {
    unsigned b = 1;
    while (b < 64 && (1ull << b) < n) ++b;
    return b;
}

// Sort, dedup, drop self loops and store into a kt_edges result.  Keys arrive packed as
// (u << 32 | v) with u < v; they are re-packed as (u << vb | v) so the radix sort only
// touches 2*vb bits.
int finish(std::vector<uint64_t>& keys, uint32_t num_nodes, kt_edges* out) {
    const unsigned vb = bits_for(num_nodes);
    for (auto& k : keys) k = ((k >> 32) << vb) | (k & 0xffffffffull);
    radix_sort_u64(keys, 2 * vb);
    const uint64_t vmask = (1ull << vb) - 1;
    size_t w = 0;
    for (size_t i = 0; i < keys.size(); ++i) {
        uint64_t k = keys[i];
        if ((k >> vb) == (k & vmask)) continue;
        if (w > 0 && keys[w - 1] == k) continue;
        keys[w++] = k;
    }
    keys.resize(w);
    out->num_nodes = num_nodes;
    out->num_edges = w;
    out->u = (uint32_t*)malloc(sizeof(uint32_t) * (w ? w : 1));
    out->v = (uint32_t*)malloc(sizeof(uint32_t) * (w ? w : 1));
    if (!out->u || !out->v) { free(out->u); free(out->v); out->u = out->v = nullptr; return KT_ERR_HOST_ALLOC; }
    for (size_t i = 0; i < w; ++i) { out->u[i] = (uint32_t)(keys[i] >> vb); out->v[i] = (uint32_t)(keys[i] & vmask); }
    return KT_OK;
}

template <class F>
void parallel_for(size_t n, F f) {
    const unsigned T = worker_count();
    if (n < 4096 || T == 1) { f((size_t)0, n); return; }
    const size_t chunk = (n + T - 1) / T;
    std::vector<std::thread> th;
    for (unsigned t = 0; t < T; ++t) {
        size_t lo = t * chunk, hi = std::min(n, lo + chunk);
        if (lo >= hi) break;
        th.emplace_back([=] { f(lo, hi); });
    }
    for (auto& x : th) x.join();
}

}  // namespace

extern "C" {

int kt_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c,
                uint64_t seed, kt_edges* out) {
    if (!out) return KT_ERR_INVALID_ARG;
    memset(out, 0, sizeof(*out));
    if (scale == 0 || scale > 31 || edge_factor == 0) return KT_ERR_INVALID_ARG;
    if (a < 0 || b < 0 || c < 0 || a + b + c > 1.0) return KT_ERR_INVALID_ARG;
    const uint64_t m = (uint64_t)edge_factor << scale;
    const uint64_t ta = prob_threshold(a), tab = prob_threshold(a + b), tabc = prob_threshold(a + b + c);
    std::vector<uint64_t> keys(m);
    Rng rng(seed, 1);
    parallel_for(m, [&](size_t lo, size_t hi) {
        for (size_t i = lo; i < hi; ++i) {
            uint32_t s = 0, d = 0;
            for (uint32_t l = 0; l < scale; ++l) {
                uint64_t r = rng.at((uint64_t)i * 32 + l);
                // quadrant: [0,a) top-left, [a,a+b) top-right, [a+b,a+b+c) bottom-left, rest bottom-right
                uint32_t sb = r >= tab, db = (r >= ta && r < tab) || r >= tabc;
                s |= sb << l;
                d |= db << l;
            }
            keys[i] = pack(s, d);
        }
    });
    return finish(keys, 1u << scale, out);
}

int kt_gen_er(uint32_t n, double p, uint64_t seed, kt_edges* out) {
    if (!out) return KT_ERR_INVALID_ARG;
    memset(out, 0, sizeof(*out));
    if (n < 2 || p < 0 || p > 1) return KT_ERR_INVALID_ARG;
    Rng rng(seed, 2);
    std::vector<uint64_t> keys;
    if (n <= 16384) {
        // exact G(n, p): one Bernoulli draw per vertex pair
        const uint64_t t = prob_threshold(p);
        std::vector<std::vector<uint64_t>> part(n);
        parallel_for(n, [&](size_t lo, size_t hi) {
            for (size_t i = lo; i < hi; ++i)
                for (uint32_t j = (uint32_t)i + 1; j < n; ++j)
                    if (rng.at((uint64_t)i * n + j) < t) part[i].push_back(pack((uint32_t)i, j));
        });
        for (auto& v : part) keys.insert(keys.end(), v.begin(), v.end());
    } else {
        // large n: G(n, M) with M = round(p * n(n-1)/2) draws, duplicates merged
        const double pairs = (double)n * (double)(n - 1) / 2.0;
        const uint64_t M = (uint64_t)(p * pairs + 0.5);
        keys.resize(M);
        parallel_for(M, [&](size_t lo, size_t hi) {
            for (size_t i = lo; i < hi; ++i) {
                uint32_t a = bounded(rng.at(2 * i), n), b = bounded(rng.at(2 * i + 1), n);
                keys[i] = pack(a, b);
            }
        });
    }
    return finish(keys, n, out);
}

int kt_gen_ba(uint32_t n, uint32_t m, uint64_t seed, kt_edges* out) {
    if (!out) return KT_ERR_INVALID_ARG;
    memset(out, 0, sizeof(*out));
    if (m == 0 || n <= m + 1) return KT_ERR_INVALID_ARG;
    Rng rng(seed, 3);
    uint64_t ctr = 0;
    std::vector<uint64_t> keys;
    std::vector<uint32_t> ends;  // every edge endpoint once: sampling it is degree-proportional
    keys.reserve((size_t)n * m);
    ends.reserve((size_t)2 * n * m);
    for (uint32_t i = 0; i <= m; ++i)
        for (uint32_t j = i + 1; j <= m; ++j) {
            keys.push_back(pack(i, j));
            ends.push_back(i);
            ends.push_back(j);
        }
    std::vector<uint32_t> picked;
    for (uint32_t v = m + 1; v < n; ++v) {
        picked.clear();
        while (picked.size() < m) {
            uint32_t t = ends[bounded(rng.at(ctr++), (uint32_t)ends.size())];
            if (std::find(picked.begin(), picked.end(), t) == picked.end()) picked.push_back(t);
        }
        for (uint32_t t : picked) {
            keys.push_back(pack(v, t));
            ends.push_back(v);
            ends.push_back(t);
        }
    }
    return finish(keys, n, out);
}

int kt_gen_ws(uint32_t n, uint32_t k, double p, uint64_t seed, kt_edges* out) {
    if (!out) return KT_ERR_INVALID_ARG;
    memset(out, 0, sizeof(*out));
    if (k < 2 || (k & 1) || k >= n || p < 0 || p > 1) return KT_ERR_INVALID_ARG;
    Rng rng(seed, 4);
    const uint64_t t = prob_threshold(p);
    uint64_t ctr = 0;
    std::vector<uint64_t> keys;
    keys.reserve((size_t)n * (k / 2));
    for (uint32_t i = 0; i < n; ++i)
        for (uint32_t j = 1; j <= k / 2; ++j) keys.push_back(pack(i, (i + j) % n));
    std::unordered_set<uint64_t> present(keys.begin(), keys.end());
    // rewire each lattice edge (i, i+j) with probability p to (i, w), w uniform, avoiding
    // self loops and existing edges; lattice edge e was created by source e / (k/2)
    for (size_t e = 0; e < keys.size(); ++e) {
        if (rng.at(ctr++) >= t) continue;
        const uint32_t i = (uint32_t)(e / (k / 2));
        for (int tries = 0; tries < 64; ++tries) {
            uint32_t w = bounded(rng.at(ctr++), n);
            uint64_t nk = pack(i, w);
            if (w == i || present.count(nk)) continue;
            present.erase(keys[e]);
            present.insert(nk);
            keys[e] = nk;
            break;
        }
    }
    return finish(keys, n, out);
}

int kt_gen_rgg(uint32_t n, double radius, uint64_t seed, kt_edges* out) {
    if (!out) return KT_ERR_INVALID_ARG;
    memset(out, 0, sizeof(*out));
    if (n < 2 || !(radius > 0) || radius > 1) return KT_ERR_INVALID_ARG;
    Rng rng(seed, 5);
    std::vector<double> x(n), y(n);
    for (uint32_t i = 0; i < n; ++i) {
        x[i] = (double)(rng.at(2 * (uint64_t)i) >> 11) * (1.0 / 9007199254740992.0);
        y[i] = (double)(rng.at(2 * (uint64_t)i + 1) >> 11) * (1.0 / 9007199254740992.0);
    }
    uint32_t g = (uint32_t)(1.0 / radius);
    if (g < 1) g = 1;
    if (g > 4096) g = 4096;
    std::vector<std::vector<uint32_t>> cell((size_t)g * g);
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t cx = std::min(g - 1, (uint32_t)(x[i] * g)), cy = std::min(g - 1, (uint32_t)(y[i] * g));
        cell[(size_t)cy * g + cx].push_back(i);
    }
    const double r2 = radius * radius;
    std::vector<uint64_t> keys;
    for (uint32_t cy = 0; cy < g; ++cy)
        for (uint32_t cx = 0; cx < g; ++cx)
            for (uint32_t i : cell[(size_t)cy * g + cx])
                for (int dy = -1; dy <= 1; ++dy)
                    for (int dx = -1; dx <= 1; ++dx) {
                        int ny = (int)cy + dy, nx = (int)cx + dx;
                        if (ny < 0 || nx < 0 || ny >= (int)g || nx >= (int)g) continue;
                        for (uint32_t j : cell[(size_t)ny * g + nx]) {
                            if (j <= i) continue;
                            double ddx = x[i] - x[j], ddy = y[i] - y[j];
                            double sx = ddx * ddx, sy = ddy * ddy;
                            if (sx + sy < r2) keys.push_back(pack(i, j));
                        }
                    }
    return finish(keys, n, out);
}

int kt_plant_cliques(uint32_t num_nodes, const uint32_t* u, const uint32_t* v, uint64_t num_edges, uint32_t count,
                     uint32_t min_size, uint32_t max_size, uint64_t seed, kt_edges* out) {
    if (!out) return KT_ERR_INVALID_ARG;
    memset(out, 0, sizeof(*out));
    if ((num_edges && (!u || !v)) || min_size < 2 || max_size < min_size || max_size > num_nodes)
        return KT_ERR_INVALID_ARG;
    Rng rng(seed, 6);
    uint64_t ctr = 0;
    std::vector<uint64_t> extra;
    std::vector<uint32_t> members;
    for (uint32_t q = 0; q < count; ++q) {
        uint32_t s = min_size + bounded(rng.at(ctr++), max_size - min_size + 1);
        members.clear();
        while (members.size() < s) {
            uint32_t x = bounded(rng.at(ctr++), num_nodes);
            if (std::find(members.begin(), members.end(), x) == members.end()) members.push_back(x);
        }
        for (size_t i = 0; i < members.size(); ++i)
            for (size_t j = i + 1; j < members.size(); ++j) extra.push_back(pack(members[i], members[j]));
    }
    // Is the input canonical already (u < v, (u, v) strictly increasing, ids in range)?  Then only
    // the clique edges are sorted and merged into it.
    std::atomic<bool> canonical{true};
    parallel_for(num_edges, [&](size_t lo, size_t hi) {
        for (size_t i = lo; i < hi; ++i) {
            if (u[i] >= v[i] || v[i] >= num_nodes || (i > 0 && pack(u[i - 1], v[i - 1]) >= pack(u[i], v[i]))) {
                canonical = false;
                return;
            }
        }
    });
    if (!canonical) {
        std::vector<uint64_t> keys(num_edges);
        for (uint64_t i = 0; i < num_edges; ++i) {
            if (u[i] >= num_nodes || v[i] >= num_nodes) return KT_ERR_INVALID_ARG;
            keys[i] = pack(u[i], v[i]);
        }
        keys.insert(keys.end(), extra.begin(), extra.end());
        return finish(keys, num_nodes, out);
    }
    std::sort(extra.begin(), extra.end());
    extra.erase(std::unique(extra.begin(), extra.end()), extra.end());
    const uint64_t cap = num_edges + extra.size();
    out->num_nodes = num_nodes;
    out->u = (uint32_t*)malloc(sizeof(uint32_t) * (cap ? cap : 1));
    out->v = (uint32_t*)malloc(sizeof(uint32_t) * (cap ? cap : 1));
    if (!out->u || !out->v) { free(out->u); free(out->v); out->u = out->v = nullptr; return KT_ERR_HOST_ALLOC; }
    uint64_t i = 0, j = 0, w = 0;
    while (i < num_edges || j < extra.size()) {
        const uint64_t a = i < num_edges ? pack(u[i], v[i]) : UINT64_MAX;
        const uint64_t b = j < extra.size() ? extra[j] : UINT64_MAX;
        const uint64_t k = a <= b ? a : b;
        if (a <= b) ++i;
        if (b <= a) ++j;
        out->u[w] = (uint32_t)(k >> 32);
        out->v[w] = (uint32_t)k;
        ++w;
    }
    out->num_edges = w;
    return KT_OK;
}

int kt_gen_batch(uint32_t num_graphs, uint32_t n_min, uint32_t n_max, uint64_t seed, kt_edges* out,
                 uint32_t* vertex_offsets) {
    if (!out || !vertex_offsets || num_graphs == 0 || n_min < 64 || n_max < n_min) return KT_ERR_INVALID_ARG;
    memset(out, 0, sizeof(*out));
    // per graph: size log-uniform in [n_min, n_max] (libm exp/log), even graphs Barabasi-Albert with
    // m in {2,4,8,16}, odd graphs Watts-Strogatz with k in {6,10,20} and p = 0.1; then 0-3 cliques
    // of 8-64 vertices (capped at the graph size)
    std::vector<uint32_t> sizes(num_graphs);
    Rng rng(seed, 7);
    const double lr = std::log((double)n_max / (double)n_min);
    uint64_t total_n = 0;
    for (uint32_t g = 0; g < num_graphs; ++g) {
        const double u = (double)(rng.at(4ull * g) >> 11) * (1.0 / 9007199254740992.0);
        uint32_t n = (uint32_t)std::llround((double)n_min * std::exp(u * lr));
        if (n < n_min) n = n_min;
        if (n > n_max) n = n_max;
        sizes[g] = n;
        vertex_offsets[g] = (uint32_t)total_n;
        total_n += n;
        if (total_n > 0xffffffffull) return KT_ERR_TOO_LARGE;
    }
    vertex_offsets[num_graphs] = (uint32_t)total_n;
    std::vector<kt_edges> parts(num_graphs);
    std::atomic<uint32_t> next{0};
    std::atomic<int> status{KT_OK};
    auto work = [&] {
        for (uint32_t g; (g = next.fetch_add(1)) < num_graphs;) {
            const uint64_t gs = mix64(seed ^ mix64(0x6a09e667f3bcc909ull + g));
            const uint32_t n = sizes[g];
            kt_edges base{};
            int rc;
            if ((g & 1) == 0) {
                static const uint32_t ms[4] = {2, 4, 8, 16};
                rc = kt_gen_ba(n, ms[rng.at(4ull * g + 1) & 3], gs, &base);
            } else {
                static const uint32_t ks[3] = {6, 10, 20};
                rc = kt_gen_ws(n, ks[bounded(rng.at(4ull * g + 1), 3)], 0.1, gs, &base);
            }
            if (rc == KT_OK) {
                const uint32_t cliques = bounded(rng.at(4ull * g + 2), 4);
                const uint32_t hi = std::min<uint32_t>(64, n);
                if (cliques) {
                    kt_edges with{};
                    rc = kt_plant_cliques(n, base.u, base.v, base.num_edges, cliques, std::min<uint32_t>(8, hi), hi,
                                          gs ^ 0x3c6ef372fe94f82bull, &with);
                    kt_edges_free(&base);
                    base = with;
                }
            }
            if (rc != KT_OK) status.store(rc);
            parts[g] = base;
        }
    };
    std::vector<std::thread> th;
    for (unsigned t = 0; t < worker_count(); ++t) th.emplace_back(work);
    for (auto& x : th) x.join();
    if (status.load() != KT_OK) {
        for (auto& p : parts) kt_edges_free(&p);
        return status.load();
    }
    uint64_t m = 0;
    for (auto& p : parts) m += p.num_edges;
    out->num_nodes = (uint32_t)total_n;
    out->num_edges = m;
    out->u = (uint32_t*)malloc(sizeof(uint32_t) * (m ? m : 1));
    out->v = (uint32_t*)malloc(sizeof(uint32_t) * (m ? m : 1));
    if (!out->u || !out->v) {
        kt_edges_free(out);
        for (auto& p : parts) kt_edges_free(&p);
        return KT_ERR_HOST_ALLOC;
    }
    uint64_t w = 0;
    for (uint32_t g = 0; g < num_graphs; ++g) {
        const uint32_t off = vertex_offsets[g];
        for (uint64_t i = 0; i < parts[g].num_edges; ++i, ++w) {
            out->u[w] = parts[g].u[i] + off;
            out->v[w] = parts[g].v[i] + off;
        }
        kt_edges_free(&parts[g]);
    }
    return KT_OK;
}

void kt_edges_free(kt_edges* g) {
    if (!g) return;
    free(g->u);
    free(g->v);
    g->u = g->v = nullptr;
    g->num_edges = 0;
}

}  // extern "C"
