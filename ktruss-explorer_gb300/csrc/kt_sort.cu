// Device primitives for the CSR build: exclusive scan and a stable LSD radix sort.
//
// These replace the Thrust scan and the per-row CPU quicksort of the reference build
// (graph.cu:457 thrust::exclusive_scan, graph.cu:462-476 "Sort outgoing edges ... on CPU").

#include "kt_device.cuh"
#include "kt_engine.h"

namespace kt {

namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr uint32_t kScanTile = kScanThreads * kScanItems;  // 4096

// Block-wide exclusive scan of one value per thread; returns the block total in *total.
template <class T>
__device__ __forceinline__ T block_exclusive_scan(T v, T* warp_sums, T* total) {
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    T x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(kFullMask, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        T w = lane < nwarps ? warp_sums[lane] : T(0);
        T s = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            T y = __shfl_up_sync(kFullMask, s, o);
            if (lane >= (uint32_t)o) s += y;
        }
        if (lane < nwarps) warp_sums[lane] = s - w;
        if (lane == 31) warp_sums[32] = s;
    }
    __syncthreads();
    T r = warp_sums[warp] + x - v;
    *total = warp_sums[32];
    __syncthreads();
    return r;
}

template <class T>
__global__ void __launch_bounds__(kScanThreads) k_scan_tile_sums(const T* __restrict__ in, uint64_t n,
                                                                   T* __restrict__ sums) {
    __shared__ T ws[33];
    const uint64_t base = (uint64_t)blockIdx.x * kScanTile;
    T s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        uint64_t idx = base + threadIdx.x + (uint64_t)i * kScanThreads;
        if (idx < n) s += in[idx];
    }
    T total;
    block_exclusive_scan<T>(s, ws, &total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// Exclusive scan of each tile, offset by the scanned tile sums (if given).
template <class T>
__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const T* in, T* out, uint64_t n,
                                                               const T* __restrict__ tile_offsets) {
    __shared__ T tile[kScanTile];
    __shared__ T ws[33];
    const uint64_t base = (uint64_t)blockIdx.x * kScanTile;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        uint64_t idx = base + threadIdx.x + (uint64_t)i * kScanThreads;
        tile[threadIdx.x + i * kScanThreads] = idx < n ? in[idx] : T(0);
    }
    __syncthreads();
    T v[kScanItems], s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        v[i] = tile[threadIdx.x * kScanItems + i];
        s += v[i];
    }
    T total;
    T run = block_exclusive_scan<T>(s, ws, &total) + (tile_offsets ? tile_offsets[blockIdx.x] : T(0));
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        tile[threadIdx.x * kScanItems + i] = run;
        run += v[i];
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        uint64_t idx = base + threadIdx.x + (uint64_t)i * kScanThreads;
        if (idx < n) out[idx] = tile[threadIdx.x + i * kScanThreads];
    }
}

constexpr uint32_t kSortTile = 2048;  // keys per tile (one histogram column per tile and digit)
constexpr int kDigits = 256;          // 8-bit digits
constexpr int kSortThreads = kDigits; // the histogram kernel: one digit per thread
// The scatter: kScatterThreads threads a block, each warp ranking kScatterSteps 32-key steps.
// 512 threads of 4 steps hold 32 registers a thread (4 blocks, all 64 warps of a SM); 256
// threads of 8 steps needed 64 (32 warps a SM) and ran at 40 % of DRAM bandwidth.  Measured on
// GB300: batch4096 build 69.7 -> 69.1 ms, R-MAT 24 build 128.7 -> 128.3 ms.
constexpr int kScatterThreads = 512;
constexpr int kScatterWarps = kScatterThreads / 32;
constexpr int kScatterSteps = 4;
constexpr uint32_t kScatterWarpKeys = 32 * kScatterSteps;
static_assert(kScatterWarps * kScatterWarpKeys == kSortTile, "a scatter block covers one tile");
static_assert(kScatterThreads >= kDigits, "the first kDigits threads own one digit each");

__global__ void __launch_bounds__(kSortThreads) k_radix_hist(const uint64_t* __restrict__ keys, uint64_t n,
                                                               unsigned shift, uint32_t* __restrict__ hist,
                                                               uint32_t num_blocks) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const uint64_t base = (uint64_t)blockIdx.x * kSortTile;
    for (uint32_t i = threadIdx.x; i < kSortTile; i += kSortThreads) {
        uint64_t idx = base + i;
        if (idx < n) atomicAdd(&h[(uint32_t)(keys[idx] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[(uint64_t)threadIdx.x * num_blocks + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter of one 2048-key tile: each warp ranks its kScatterWarpKeys consecutive keys in
// 32-key steps with __match_any_sync; warps are then offset by the counts of earlier warps (the
// first kDigits threads own one digit each for the tile's counts and offsets).  The tile is first
// arranged in digit order in shared memory, then written out so that consecutive threads store
// consecutive positions of each digit's run (coalesced stores).
__global__ void __launch_bounds__(kScatterThreads) k_radix_scatter(const uint64_t* __restrict__ kin,
                                                                  const uint32_t* __restrict__ vin,
                                                                  uint64_t* __restrict__ kout,
                                                                  uint32_t* __restrict__ vout, uint64_t n,
                                                                  unsigned shift,
                                                                  const uint32_t* __restrict__ hist,
                                                                  uint32_t num_blocks) {
    __shared__ uint32_t wh[kScatterWarps][kDigits];
    __shared__ uint32_t goff[kDigits];   // global start of each digit's run for this tile
    __shared__ uint32_t toff[kDigits];   // start of each digit's run inside the tile
    __shared__ uint32_t ws[33];
    __shared__ uint64_t skey[kSortTile];
    __shared__ uint32_t sval[kSortTile];
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    const bool owner = threadIdx.x < (uint32_t)kDigits;  // digit threadIdx.x (whole warps)
    for (uint32_t i = threadIdx.x; i < kScatterWarps * kDigits; i += kScatterThreads) (&wh[0][0])[i] = 0;
    if (owner) goff[threadIdx.x] = hist[(uint64_t)threadIdx.x * num_blocks + blockIdx.x];
    __syncthreads();
    const uint64_t tbase = (uint64_t)blockIdx.x * kSortTile;
    const uint64_t wbase = tbase + (uint64_t)warp * kScatterWarpKeys;
    uint64_t key[kScatterSteps];
    uint32_t val[kScatterSteps], dig[kScatterSteps], rk[kScatterSteps];
#pragma unroll
    for (int s = 0; s < kScatterSteps; ++s) {
        uint64_t idx = wbase + (uint32_t)s * 32 + lane;
        bool valid = idx < n;
        key[s] = valid ? kin[idx] : 0ull;
        val[s] = (valid && vin) ? vin[idx] : 0u;
        uint32_t d = valid ? ((uint32_t)(key[s] >> shift) & 255u) : 256u;
        dig[s] = d;
        uint32_t peers = __match_any_sync(kFullMask, d);
        uint32_t base = d < 256 ? wh[warp][d] : 0u;
        __syncwarp();
        if (d < 256 && lane == (uint32_t)(__ffs(peers) - 1)) wh[warp][d] = base + __popc(peers);
        __syncwarp();
        rk[s] = base + __popc(peers & lanemask_lt());
    }
    __syncthreads();
    uint32_t count = 0;  // keys of digit threadIdx.x in the tile
    if (owner) {
        uint32_t run = 0;
#pragma unroll
        for (int w = 0; w < kScatterWarps; ++w) {
            uint32_t c = wh[w][threadIdx.x];
            wh[w][threadIdx.x] = run;
            run += c;
        }
        count = run;
    }
    // exclusive scan of the tile's digit counts (one digit per owner thread)
    {
        constexpr int kDigitWarps = kDigits / 32;
        uint32_t x = count;
        if (owner) {
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(kFullMask, x, o);
                if (lane >= (uint32_t)o) x += y;
            }
            if (lane == 31) ws[warp] = x;
        }
        __syncthreads();
        if (warp == 0) {
            const uint32_t w = lane < kDigitWarps ? ws[lane] : 0u;
            uint32_t t = w;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(kFullMask, t, o);
                if (lane >= (uint32_t)o) t += y;
            }
            if (lane < kDigitWarps) ws[lane] = t - w;
        }
        __syncthreads();
        if (owner) toff[threadIdx.x] = ws[warp] + x - count;
    }
    __syncthreads();
#pragma unroll
    for (int s = 0; s < kScatterSteps; ++s) {
        const uint32_t d = dig[s];
        if (d < 256) {
            const uint32_t lp = toff[d] + wh[warp][d] + rk[s];
            skey[lp] = key[s];
            sval[lp] = val[s];
        }
    }
    __syncthreads();
    const uint32_t valid = (uint32_t)min((uint64_t)kSortTile, n - tbase);
    for (uint32_t i = threadIdx.x; i < valid; i += kScatterThreads) {
        const uint64_t k = skey[i];
        const uint32_t d = (uint32_t)(k >> shift) & 255u;
        const uint32_t pos = goff[d] + (i - toff[d]);
        kout[pos] = k;
        if (vin) vout[pos] = sval[i];
    }
}

}  // namespace

// Hierarchical scan: tile sums are scanned recursively in scratch (used as a stack from
// word `tmp_off` on), then every tile is rescanned with its offset.
template <class T>
static int scan_level(kt_engine* e, const T* in, T* out, uint64_t n, T* tmp, uint64_t tmp_words, uint64_t tmp_off) {
    if (n == 0) return KT_OK;
    if (n <= kScanTile) {
        k_scan_tiles<T><<<1, kScanThreads, 0, e->stream>>>(in, out, n, nullptr);
        count_launch(e);
        return check_launch(e, "k_scan_tiles");
    }
    const uint64_t nb = (n + kScanTile - 1) / kScanTile;
    const uint64_t words = (nb + 63) & ~63ull;
    if (tmp_off + words > tmp_words)
        return fail(KT_ERR_INVALID_ARG, "scan scratch too small (%llu elements)", (unsigned long long)tmp_words);
    T* sums = tmp + tmp_off;
    k_scan_tile_sums<T><<<(uint32_t)nb, kScanThreads, 0, e->stream>>>(in, n, sums);
    count_launch(e);
    int rc = check_launch(e, "k_scan_tile_sums");
    if (rc) return rc;
    rc = scan_level<T>(e, sums, sums, nb, tmp, tmp_words, tmp_off + words);
    if (rc) return rc;
    k_scan_tiles<T><<<(uint32_t)nb, kScanThreads, 0, e->stream>>>(in, out, n, sums);
    count_launch(e);
    return check_launch(e, "k_scan_tiles");
}

int exclusive_scan(kt_engine* e, const uint32_t* in, uint32_t* out, uint64_t n) {
    return scan_level<uint32_t>(e, in, out, n, e->scan_tmp, e->scan_tmp_words, 0);
}

int exclusive_scan_u64(kt_engine* e, const uint64_t* in, uint64_t* out, uint64_t n) {
    return scan_level<uint64_t>(e, in, out, n, reinterpret_cast<uint64_t*>(e->scan_tmp), e->scan_tmp_words / 2, 0);
}

int radix_sort(kt_engine* e, uint64_t* key_a, uint32_t* val_a, uint64_t* key_b, uint32_t* val_b, uint64_t n,
               unsigned bits, int* result_in_b) {
    *result_in_b = 0;
    if (n <= 1 || bits == 0) return KT_OK;
    const uint64_t nb64 = (n + kSortTile - 1) / kSortTile;
    if (nb64 * 256 > e->hist_words) return fail(KT_ERR_INVALID_ARG, "sort histogram scratch too small");
    const uint32_t nb = (uint32_t)nb64;
    uint64_t *kin = key_a, *kout = key_b;
    uint32_t *vin = val_a, *vout = val_b;
    for (unsigned shift = 0; shift < bits; shift += 8) {
        k_radix_hist<<<nb, kSortThreads, 0, e->stream>>>(kin, n, shift, e->hist, nb);
        count_launch(e);
        int rc = check_launch(e, "k_radix_hist");
        if (rc) return rc;
        rc = exclusive_scan(e, e->hist, e->hist, (uint64_t)nb * 256);
        if (rc) return rc;
        k_radix_scatter<<<nb, kScatterThreads, 0, e->stream>>>(kin, vin, kout, vout, n, shift, e->hist, nb);
        count_launch(e);
        rc = check_launch(e, "k_radix_scatter");
        if (rc) return rc;
        uint64_t* tk = kin; kin = kout; kout = tk;
        uint32_t* tv = vin; vin = vout; vout = tv;
        *result_in_b ^= 1;
    }
    return KT_OK;
}

}  // namespace kt
