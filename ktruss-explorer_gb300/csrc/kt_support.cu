// Edge support (triangle count per edge) on the degree-oriented CSR.
//
// Replaces count_triangles_kernel of the reference (kernel_ddc.cu:11-54): there one thread
// merges the two out-lists of its edge and issues three atomics per triangle.  Here each
// oriented edge (u,v), u < v in rank order, is handled by a group of G lanes (G = 4, 8, 16 or
// 32, the schedule's support_group).  Only the part
// of N+(u) above v can hold a common neighbour, and it starts right after the edge itself in
// u's row, so the intersection is  S = o_col[j+1 .. o_ptr[u+1])  with  L = N+(v).  Lanes stride
// over the shorter list and binary-search the longer one; for a triangle (u,v,w) found at
// positions x (in u's row) and y (in v's row), the edges (u,w) = x and (v,w) = y gain one
// support each, and (u,v) gains the group's match count once.
//
// Bound: the oriented CSR (o_ptr, o_col) is L2-resident at RMAT scale 20 (63 MB < 129 MB),
// so the kernel is bound by L1/L2 probe latency and atomic throughput, not HBM.

#include "kt_device.cuh"
#include "kt_engine.h"

namespace kt {

namespace {

constexpr int kThreads = 256;

template <int G>
__global__ void __launch_bounds__(kThreads) k_support(const uint32_t* __restrict__ o_ptr,
                                                      const uint32_t* __restrict__ o_col,
                                                      const uint32_t* __restrict__ e_src, uint32_t m,
                                                      uint32_t* __restrict__ sup) {
    const uint32_t lane = lane_id();
    const uint32_t glane = lane & (G - 1);
    const uint32_t gmask = (G == 32) ? kFullMask : (((1u << G) - 1) << (lane & ~(uint32_t)(G - 1)));
    const uint64_t gid = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
    const uint64_t ngroups = ((uint64_t)gridDim.x * blockDim.x) / G;
    for (uint64_t j64 = gid; j64 < m; j64 += ngroups) {
        const uint32_t j = (uint32_t)j64;
        const uint32_t u = e_src[j], v = o_col[j];
        const uint32_t a0 = j + 1, a1 = o_ptr[u + 1];
        const uint32_t b0 = o_ptr[v], b1 = o_ptr[v + 1];
        const uint32_t na = a1 - a0, nb = b1 - b0;
        uint32_t cnt = 0;
        if (na && nb) {
            // iterate the shorter list, search the longer
            const bool iter_a = na <= nb;
            const uint32_t i0 = iter_a ? a0 : b0, ni = iter_a ? na : nb;
            const uint32_t s0 = iter_a ? b0 : a0, ns = iter_a ? nb : na;
            for (uint32_t t = glane; t < ni; t += G) {
                const uint32_t x = i0 + t;
                const uint32_t w = o_col[x];
                const uint32_t idx = lower_bound_u32(o_col + s0, ns, w);
                if (idx < ns && o_col[s0 + idx] == w) {
                    ++cnt;
                    atomicAdd(&sup[x], 1u);
                    atomicAdd(&sup[s0 + idx], 1u);
                }
            }
        }
        __syncwarp(gmask);
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) cnt += __shfl_xor_sync(gmask, cnt, o);
        if (glane == 0 && cnt) atomicAdd(&sup[j], cnt);
    }
}

}  // namespace

int count_support(kt_engine* e) {
    if (e->m == 0) return KT_OK;
    int rc = check_cuda(cudaMemsetAsync(e->sup, 0, sizeof(uint32_t) * e->m, e->stream), "clear support");
    if (rc) return rc;
    const uint32_t G = e->sched.support_group;
    uint64_t blocks = ((uint64_t)e->m * G + kThreads - 1) / kThreads;
    const uint64_t max_blocks = (uint64_t)e->num_sms * 16;
    if (blocks > max_blocks) blocks = max_blocks;
    switch (G) {
        case 4: k_support<4><<<(uint32_t)blocks, kThreads, 0, e->stream>>>(e->o_ptr, e->o_col, e->e_src, e->m, e->sup); break;
        case 16: k_support<16><<<(uint32_t)blocks, kThreads, 0, e->stream>>>(e->o_ptr, e->o_col, e->e_src, e->m, e->sup); break;
        case 32: k_support<32><<<(uint32_t)blocks, kThreads, 0, e->stream>>>(e->o_ptr, e->o_col, e->e_src, e->m, e->sup); break;
        default: k_support<8><<<(uint32_t)blocks, kThreads, 0, e->stream>>>(e->o_ptr, e->o_col, e->e_src, e->m, e->sup); break;
    }
    count_launch(e);
    return check_launch(e, "k_support");
}

}  // namespace kt
