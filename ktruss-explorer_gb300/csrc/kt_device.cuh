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
};

// Layout of the device control block (uint32 words unless noted).
enum : uint32_t {
    kCtrlError = 0,
    kCtrlCount0 = 1,      // frontier / compaction counters
    kCtrlCount1 = 2,
    kCtrlMin = 3,         // minimum support over alive edges
    kCtrlKmax = 4,
    kCtrlRound = 5,
    kCtrlLevel = 6,
    kCtrlAlive = 7,
    kCtrlBarrier = 8,     // grid barrier arrival counter
    kCtrlBarrierGen = 9,  // grid barrier generation
    kCtrlTriLo = 10,      // 64-bit triangle counter (lo, hi)
    kCtrlTriHi = 11,
    kCtrlItems0 = 12,     // work-item queue counters
    kCtrlItems1 = 13,
    kCtrlBigRow = 14,     // first rank whose symmetric row is long (block-wide compaction)
    kCtrlWords = 16,
};

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Index of the first element >= x in sorted a[0, n) (lower bound).
__device__ __forceinline__ uint32_t lower_bound_u32(const uint32_t* __restrict__ a, uint32_t n, uint32_t x) {
    uint32_t lo = 0;
    while (n > 0) {
        uint32_t half = n >> 1;
        if (__ldg(a + lo + half) < x) {
            lo += half + 1;
            n -= half + 1;
        } else {
            n = half;
        }
    }
    return lo;
}

inline uint32_t ceil_div(uint64_t a, uint64_t b) { return (uint32_t)((a + b - 1) / b); }

}  // namespace kt
