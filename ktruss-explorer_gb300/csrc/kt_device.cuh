// Device-side helpers shared by the CUDA translation units of libktruss_gb300.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "kt_internal.h"

namespace kt {

constexpr uint32_t kFullMask = 0xffffffffu;

// Bits of the device error word (Engine::ctrl[kCtrlError]).
enum : uint32_t {
    kErrBadVertex = 1u << 0,   // an entry names a vertex >= num_nodes
    kErrSelfLoop = 1u << 1,    // src == dst
    kErrDuplicate = 1u << 2,   // the same (src, dst) entry twice
    kErrAsymmetric = 1u << 3,  // (u, v) present without (v, u)
    kErrTimeout = 1u << 4,     // a bounded grid-barrier wait expired
    kErrRunaway = 1u << 5,     // the peel loop exceeded its round or level bound
    kErrCrossGraph = 1u << 6,  // a batch entry joins two different graphs
};

// Layout of the device control block (uint32 words unless noted).
enum : uint32_t {
    kCtrlError = 0,
    // words 1-9, 12, 13 and 26-27 are unused; 21-24 hold the support plan during the count
    kCtrlVariantChanged = 25,  // a variant pass deleted an edge
    kCtrlTriLo = 10,      // 64-bit triangle counter (lo, hi)
    kCtrlTriHi = 11,
    kCtrlBigRow = 14,     // first rank whose symmetric row is long (block-wide compaction)
    kCtrlTinyRow = 15,    // first rank whose symmetric row is not tiny (thread-wise compaction below)
    // Persistent peel kernel: barrier, outputs, and rings of per-round / per-level counters
    // (slot r % 4 belongs to round r; slot (r+2) % 4 is cleared during round r).
    kPBarCount = 16,   // u64 (words 16..17): grid-barrier arrivals since the launch
    kPKmax = 18,
    kPRounds = 19,
    kPLevels = 20,
    kPBigCount = 28,   // [4] long-row slots of the round
    kPLAlive = 32,     // [4] alive edges after the level scan
    kPLMin = 36,       // [4] minimum support over them
    kPLMinId = 40,     // [4] smallest alive edge id at the level scan (later scans start there)
    kPCompactions = 44,
    kPPhaseNs = 48,    // [6] u64 nanoseconds per phase kind (init, level scan, collect,
                       //     compaction, mark, process), measured by block 0 barrier to barrier
    kPEdges = 60,      // [4] edges queued for the round (chunked or long-row)
    kPChunks = 64,     // [4] u64 (words 64..71): work chunks claimed for the round; 64 bits
                       //     because a frontier of most edges can need more than 2^32 chunks
    kPWalk = 72,       // u64 (words 72..73): row entries queued for walks over the whole peel
    kPSched = 76,      // [4] schedule chosen on the device by the learned selector: support group,
                       //     chunk width, compaction and recount percentages (kept by the peel's init)
    kCtrlWords = 80,
};

// Schedule i of the autotuner's grid (kt_schedule_grid): support group {4, 8, 16} x chunk width
// {8, 16, 32} x compaction {0, 85} x recount {0, 50}, the last varying fastest.  Shared by the host
// grid and the selector's on-device choice.
__host__ __device__ __forceinline__ void grid_schedule(uint32_t i, uint32_t* group, uint32_t* width,
                                                       uint32_t* compact, uint32_t* recount) {
    *recount = (i & 1u) ? 50u : 0u;
    *compact = (i & 2u) ? 85u : 0u;
    const uint32_t gw = i >> 2;  // group index * 3 + width index
    *width = 8u << (gw % 3u);
    *group = 4u << (gw / 3u);
}

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Read-only load: the non-coherent cache path on the device, a plain load in host builds of the
// search helpers below (their unit test runs them on the CPU).
__host__ __device__ __forceinline__ uint32_t ld_ro(const uint32_t* p) {
#ifdef __CUDA_ARCH__
    return __ldg(p);
#else
    return *p;
#endif
}

// Index of the first element >= x in sorted a[0, n) (lower bound).
__host__ __device__ __forceinline__ uint32_t lower_bound_u32(const uint32_t* __restrict__ a, uint32_t n,
                                                             uint32_t x) {
    uint32_t lo = 0;
    while (n > 0) {
        uint32_t half = n >> 1;
        if (ld_ro(a + lo + half) < x) {
            lo += half + 1;
            n -= half + 1;
        } else {
            n = half;
        }
    }
    return lo;
}

// Lower bound of t in the sorted row a[lo, hi) of an array whose every 32nd element is copied to
// fence[] (fence[f] = a[32 f]).  Rows longer than 32 entries are first searched in their fences,
// which lie in a 32x smaller array, then in one block of at most 32 entries (one or two 128-byte
// lines), so a search reads at most two lines of `a` instead of one per halving.
__host__ __device__ __forceinline__ uint32_t fenced_lower_bound(const uint32_t* __restrict__ a,
                                                                const uint32_t* __restrict__ fence, uint32_t lo,
                                                                uint32_t hi, uint32_t t) {
    if (hi - lo > 32) {
        const uint32_t f0 = (lo + 31) >> 5, f1 = (hi - 1) >> 5;  // fences inside the row
        uint32_t f = f0, n = f1 - f0 + 1;                         // first fence >= t
        while (n > 0) {
            const uint32_t half = n >> 1;
            if (ld_ro(fence + f + half) < t) {
                f += half + 1;
                n -= half + 1;
            } else {
                n = half;
            }
        }
        // the answer lies in (32 (f-1), 32 f] (or [lo, 32 f0] when no fence is below t)
        const uint32_t s = f == f0 ? lo : 32 * (f - 1) + 1;
        const uint32_t e = 32 * f + 1 < hi ? 32 * f + 1 : hi;
        lo = s;
        hi = e;
    }
    return lo + lower_bound_u32(a + lo, hi - lo, t);
}

inline uint32_t ceil_div(uint64_t a, uint64_t b) { return (uint32_t)((a + b - 1) / b); }

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(uint32_t* p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned long long atom_add_acq_rel_u64(unsigned long long* p, unsigned long long v) {
    unsigned long long old;
    asm volatile("atom.add.acq_rel.gpu.global.u64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(v) : "memory");
    return old;
}

// Grid-wide barrier for a cooperative launch whose `expected` blocks are all resident.
// One 64-bit arrival counter, never reset during a launch: after the block's threads meet at
// __syncthreads, thread 0 adds 1 with acquire-release semantics (its block's writes become
// visible to whoever acquires the counter) and, unless it completed the barrier, polls the
// counter with acquire loads until it reaches the next multiple of `expected`.  No generation
// word, no reset and no fences: the last arriver has nothing to publish.  Every wait is bounded:
// a block that waits longer than timeout_ns sets kErrTimeout in ctrl[kCtrlError] and returns
// false; blocks see the bit while they poll and return false too, so the kernel ends instead of
// hanging.  Returns true when all blocks arrived.  The counter (ctrl words kPBarCount) must be
// zero at launch.
__device__ __forceinline__ bool grid_barrier(uint32_t* ctrl, uint32_t expected, uint64_t timeout_ns) {
    __shared__ uint32_t s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t ok = 1;
        unsigned long long* count = reinterpret_cast<unsigned long long*>(ctrl + kPBarCount);
        const unsigned long long old = atom_add_acq_rel_u64(count, 1ull);
        const unsigned long long target = (old / expected + 1) * expected;
        if (old + 1 != target) {
            const uint64_t t0 = global_ns();
            uint32_t spins = 0;
            while (ld_acquire_u64(count) < target) {
                if ((++spins & 31u) == 0) {
                    if (ld_acquire(ctrl + kCtrlError) & kErrTimeout) { ok = 0; break; }
                    if (global_ns() - t0 > timeout_ns) {
                        atomicOr(ctrl + kCtrlError, kErrTimeout);
                        ok = 0;
                        break;
                    }
                    if (spins > 256) __nanosleep(64);
                }
            }
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

}  // namespace kt
