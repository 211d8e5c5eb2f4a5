// Device-side TSV ingest: the graph file parsed in HBM instead of by fscanf on the host.
//
// Replaces createCOOFromFile (graph.cu:37-79), which reads "dst src x" triples of unsigned
// decimal numbers separated by any whitespace, 1-based ids, x ignored, rejecting self loops.
// Here the text is split into 32 KB tiles, one block each, staged in shared memory with 16-byte
// loads.  Pass 1 counts the tokens of every tile (a token starts at a digit that follows a
// non-digit) and flags bytes that are neither digits nor whitespace; the host turns the tile counts
// into token offsets (one small copy each way) and checks the triple count against the caller's
// capacity.  Pass 2 numbers the tokens in file order (warp ballots and a block scan per 256-byte
// step) and parses each: token t is field t % 3 of entry t / 3; a number of more than 10 digits or
// above 2^32-1 is an error.  Pass 3 checks each entry (no zero id, no self loop), converts it to
// 0-based and takes the largest id as the vertex count.  Errors carry the position of the first
// offending byte or entry, and the call returns the same statuses as the host reader
// (KT_ERR_IO, KT_ERR_SELF_LOOP) plus KT_ERR_CAPACITY when the output buffers are too small.
//
// Bound: HBM and the byte-wise work in shared memory: the text is read twice, the entries written
// once (8 B each).

#include <cerrno>
#include <cstdio>
#include <cstring>
#include <vector>

#include "kt_device.cuh"
#include "kt_engine.h"

namespace kt {

namespace {

constexpr uint32_t kTile = 32768;  // bytes per block
constexpr int kIngestThreads = 256;
constexpr uint32_t kMaxDigits = 10;

enum : uint32_t { kErrChar = 0, kErrOverflow = 1, kErrZero = 2, kErrLoop = 3, kErrKinds = 4 };

__device__ __forceinline__ bool is_digit(unsigned char c) { return c >= '0' && c <= '9'; }
__device__ __forceinline__ bool is_space(unsigned char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r'; }

// Tile [t0, t0 + len) into shared memory; 16-byte loads when the source is 16-byte aligned.
__device__ uint32_t load_tile(const unsigned char* __restrict__ text, uint64_t bytes, uint64_t t0, unsigned char* sm) {
    const uint32_t len = (uint32_t)min((uint64_t)kTile, bytes - t0);
    const unsigned char* src = text + t0;
    uint32_t done = 0;
    if ((reinterpret_cast<uintptr_t>(src) & 15) == 0) {
        const uint32_t n16 = len / 16;
        for (uint32_t i = threadIdx.x; i < n16; i += blockDim.x)
            reinterpret_cast<uint4*>(sm)[i] = reinterpret_cast<const uint4*>(src)[i];
        done = n16 * 16;
    }
    for (uint32_t i = done + threadIdx.x; i < len; i += blockDim.x) sm[i] = src[i];
    __syncthreads();
    return len;
}

__device__ __forceinline__ unsigned char byte_at(const unsigned char* __restrict__ text, uint64_t t0, uint32_t len,
                                                 const unsigned char* sm, int64_t i) {
    // i relative to the tile; outside the tile, read global memory (callers keep 0 <= t0 + i)
    return (i >= 0 && i < (int64_t)len) ? sm[i] : text[t0 + i];
}

// Pass 1: tokens per tile, and the first byte that is neither a digit nor whitespace.
__global__ void __launch_bounds__(kIngestThreads) k_tsv_count(const unsigned char* __restrict__ text, uint64_t bytes,
                                                              uint32_t* __restrict__ tile_tokens,
                                                              unsigned long long* __restrict__ err) {
    __shared__ __align__(16) unsigned char sm[kTile];
    __shared__ uint32_t wsum[kIngestThreads / 32];
    const uint64_t t0 = (uint64_t)blockIdx.x * kTile;
    const uint32_t len = load_tile(text, bytes, t0, sm);
    uint32_t count = 0;
    unsigned long long bad = ~0ull;
    for (uint32_t i = threadIdx.x; i < len; i += blockDim.x) {
        const unsigned char c = sm[i];
        if (is_digit(c)) {
            const bool prev_digit = (i > 0) ? is_digit(sm[i - 1]) : (t0 > 0 && is_digit(text[t0 - 1]));
            count += prev_digit ? 0u : 1u;
        } else if (!is_space(c)) {
            bad = min(bad, (unsigned long long)(t0 + i));
        }
    }
    count = __reduce_add_sync(kFullMask, count);
    if (bad != ~0ull) atomicMin(err + kErrChar, bad);  // rare: one atomic per offending thread
    if (lane_id() == 0) wsum[threadIdx.x >> 5] = count;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t s = 0;
        for (int w = 0; w < kIngestThreads / 32; ++w) s += wsum[w];
        tile_tokens[blockIdx.x] = s;
    }
}

// Pass 2: number the tokens in file order and parse them into the raw (1-based) entry fields.
__global__ void __launch_bounds__(kIngestThreads) k_tsv_parse(const unsigned char* __restrict__ text, uint64_t bytes,
                                                              const unsigned long long* __restrict__ tile_base,
                                                              uint32_t* __restrict__ dst, uint32_t* __restrict__ src,
                                                              unsigned long long* __restrict__ err) {
    __shared__ __align__(16) unsigned char sm[kTile];
    __shared__ uint32_t wcount[kIngestThreads / 32];
    const uint64_t t0 = (uint64_t)blockIdx.x * kTile;
    const uint32_t len = load_tile(text, bytes, t0, sm);
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    unsigned long long token = tile_base[blockIdx.x];
    for (uint32_t step = 0; step < len; step += blockDim.x) {
        const uint32_t i = step + threadIdx.x;
        bool start = false;
        if (i < len && is_digit(sm[i])) {
            const bool prev_digit = (i > 0) ? is_digit(sm[i - 1]) : (t0 > 0 && is_digit(text[t0 - 1]));
            start = !prev_digit;
        }
        const uint32_t ballot = __ballot_sync(kFullMask, start);
        if (lane == 0) wcount[warp] = __popc(ballot);
        __syncthreads();
        uint32_t before = 0, total = 0;
        for (int w = 0; w < kIngestThreads / 32; ++w) {
            before += w < (int)warp ? wcount[w] : 0u;
            total += wcount[w];
        }
        if (start) {
            const unsigned long long t = token + before + __popc(ballot & lanemask_lt());
            uint64_t v = 0;
            uint32_t digits = 0;
            for (int64_t p = i; t0 + p < bytes; ++p) {
                const unsigned char c = byte_at(text, t0, len, sm, p);
                if (!is_digit(c)) break;
                if (++digits > kMaxDigits) break;
                v = v * 10 + (c - '0');
            }
            if (digits > kMaxDigits || v > 0xffffffffull) {
                atomicMin(err + kErrOverflow, (unsigned long long)(t0 + i));
            } else {
                const unsigned long long e = t / 3;
                const uint32_t f = (uint32_t)(t % 3);
                if (f == 0) dst[e] = (uint32_t)v;
                else if (f == 1) src[e] = (uint32_t)v;
            }
        }
        token += total;
        __syncthreads();
    }
}

// Pass 3: validate and convert the entries; the largest 1-based id is the vertex count.
__global__ void k_tsv_finish(uint32_t* __restrict__ dst, uint32_t* __restrict__ src, uint64_t entries,
                             unsigned long long* __restrict__ err, uint32_t* __restrict__ max_id) {
    uint32_t mx = 0;
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < entries; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t a = dst[e], b = src[e];
        if (a == 0 || b == 0) {
            atomicMin(err + kErrZero, (unsigned long long)e);
        } else if (a == b) {
            atomicMin(err + kErrLoop, (unsigned long long)e);
        } else {
            dst[e] = a - 1;
            src[e] = b - 1;
            mx = max(mx, max(a, b));
        }
    }
    mx = __reduce_max_sync(kFullMask, mx);
    if (lane_id() == 0 && mx) atomicMax(max_id, mx);
}

// Scratch of one parse: per-tile token counts / offsets, error positions, the vertex count.
struct IngestScratch {
    uint32_t* tiles = nullptr;
    unsigned long long* base = nullptr;
    unsigned long long* err = nullptr;  // kErrKinds positions, then the max id (as u64 slot)
    ~IngestScratch() {
        if (tiles) cudaFree(tiles);
        if (base) cudaFree(base);
        if (err) cudaFree(err);
    }
};

}  // namespace

int parse_tsv(kt_engine* e, const char* d_text, uint64_t bytes, uint32_t* d_src, uint32_t* d_dst, uint64_t capacity,
              uint64_t* num_entries, uint32_t* num_nodes) {
    *num_entries = 0;
    *num_nodes = 0;
    if (bytes == 0) return KT_OK;
    const unsigned char* text = reinterpret_cast<const unsigned char*>(d_text);
    const uint64_t tiles = (bytes + kTile - 1) / kTile;
    if (tiles > 0x7fffffffull) return fail(KT_ERR_TOO_LARGE, "text of %llu bytes is too large", (unsigned long long)bytes);
    IngestScratch s;
    int rc;
    if ((rc = check_cuda(cudaMalloc(&s.tiles, sizeof(uint32_t) * tiles), "allocate ingest scratch")) ||
        (rc = check_cuda(cudaMalloc(&s.base, sizeof(unsigned long long) * tiles), "allocate ingest scratch")) ||
        (rc = check_cuda(cudaMalloc(&s.err, sizeof(unsigned long long) * (kErrKinds + 1)), "allocate ingest scratch")) ||
        (rc = check_cuda(cudaMemsetAsync(s.err, 0xff, sizeof(unsigned long long) * kErrKinds, e->stream), "clear")) ||
        (rc = check_cuda(cudaMemsetAsync(s.err + kErrKinds, 0, sizeof(unsigned long long), e->stream), "clear")))
        return rc;
    k_tsv_count<<<(uint32_t)tiles, kIngestThreads, 0, e->stream>>>(text, bytes, s.tiles, s.err);
    count_launch(e);
    if ((rc = check_launch(e, "k_tsv_count"))) return rc;
    std::vector<uint32_t> counts(tiles);
    std::vector<unsigned long long> base(tiles), errs(kErrKinds + 1);
    if ((rc = check_cuda(cudaMemcpyAsync(counts.data(), s.tiles, sizeof(uint32_t) * tiles, cudaMemcpyDeviceToHost,
                                         e->stream), "read tile counts")) ||
        (rc = check_cuda(cudaMemcpyAsync(errs.data(), s.err, sizeof(unsigned long long) * (kErrKinds + 1),
                                         cudaMemcpyDeviceToHost, e->stream), "read errors")) ||
        (rc = check_cuda(cudaStreamSynchronize(e->stream), "synchronize")))
        return rc;
    if (errs[kErrChar] != ~0ull)
        return fail(KT_ERR_IO, "byte %llu is neither a digit nor whitespace", (unsigned long long)errs[kErrChar]);
    unsigned long long tokens = 0;
    for (uint64_t t = 0; t < tiles; ++t) {
        base[t] = tokens;
        tokens += counts[t];
    }
    if (tokens % 3 != 0)
        return fail(KT_ERR_IO, "entry %llu is not a 'dst src x' triple", (unsigned long long)(tokens / 3 + 1));
    const uint64_t entries = tokens / 3;
    if (entries >= 0xffffffffull) return fail(KT_ERR_TOO_LARGE, "more than 2^32-2 entries");
    if (entries > capacity)
        return fail(KT_ERR_CAPACITY, "the text holds %llu entries, the output buffers %llu",
                    (unsigned long long)entries, (unsigned long long)capacity);
    if (entries && (!d_src || !d_dst)) return fail(KT_ERR_INVALID_ARG, "null output buffer");
    if ((rc = check_cuda(cudaMemcpyAsync(s.base, base.data(), sizeof(unsigned long long) * tiles,
                                         cudaMemcpyHostToDevice, e->stream), "upload token offsets")))
        return rc;
    k_tsv_parse<<<(uint32_t)tiles, kIngestThreads, 0, e->stream>>>(text, bytes, s.base, d_dst, d_src, s.err);
    count_launch(e);
    if ((rc = check_launch(e, "k_tsv_parse"))) return rc;
    if (entries) {
        uint64_t blocks = (entries + 255) / 256;
        if (blocks > (uint64_t)e->num_sms * 32) blocks = (uint64_t)e->num_sms * 32;
        k_tsv_finish<<<(uint32_t)blocks, 256, 0, e->stream>>>(d_dst, d_src, entries, s.err,
                                                             reinterpret_cast<uint32_t*>(s.err + kErrKinds));
        count_launch(e);
        if ((rc = check_launch(e, "k_tsv_finish"))) return rc;
    }
    if ((rc = check_cuda(cudaMemcpyAsync(errs.data(), s.err, sizeof(unsigned long long) * (kErrKinds + 1),
                                         cudaMemcpyDeviceToHost, e->stream), "read errors")) ||
        (rc = check_cuda(cudaStreamSynchronize(e->stream), "synchronize")))
        return rc;
    if (errs[kErrOverflow] != ~0ull)
        return fail(KT_ERR_IO, "the number at byte %llu does not fit 32 bits", (unsigned long long)errs[kErrOverflow]);
    const unsigned long long zero = errs[kErrZero], loop = errs[kErrLoop];
    if (zero != ~0ull && zero < loop)
        return fail(KT_ERR_IO, "entry %llu has a 0 vertex id (ids are 1-based)", zero + 1);
    if (loop != ~0ull)
        return fail(KT_ERR_SELF_LOOP, "entry %llu: Edges from a vertex to itself are not allowed!", loop + 1);
    *num_entries = entries;
    *num_nodes = (uint32_t)errs[kErrKinds];
    return KT_OK;
}

}  // namespace kt

using kt::check_cuda;
using kt::fail;

extern "C" {

int kt_engine_parse_tsv(kt_engine* e, const char* d_text, uint64_t bytes, uint32_t* d_src, uint32_t* d_dst,
                        uint64_t capacity, uint64_t* num_entries, uint32_t* num_nodes) {
    kt::clear_error();
    if (!e || !num_entries || !num_nodes || (bytes && !d_text))
        return fail(KT_ERR_INVALID_ARG, "kt_engine_parse_tsv: null argument");
    int rc = check_cuda(cudaSetDevice(e->device), "cudaSetDevice");
    if (rc) return rc;
    return kt::parse_tsv(e, d_text, bytes, d_src, d_dst, capacity, num_entries, num_nodes);
}

int kt_engine_read_tsv(kt_engine* e, const char* path, uint32_t* d_src, uint32_t* d_dst, uint64_t capacity,
                       uint64_t* num_entries, uint32_t* num_nodes) {
    kt::clear_error();
    if (!e || !path || !num_entries || !num_nodes) return fail(KT_ERR_INVALID_ARG, "kt_engine_read_tsv: null argument");
    FILE* fp = fopen(path, "rb");
    if (!fp) return fail(KT_ERR_IO, "cannot open %s: %s", path, strerror(errno));
    fseek(fp, 0, SEEK_END);
    const long sz = ftell(fp);
    fseek(fp, 0, SEEK_SET);
    if (sz < 0) {
        fclose(fp);
        return fail(KT_ERR_IO, "cannot size %s", path);
    }
    int rc = check_cuda(cudaSetDevice(e->device), "cudaSetDevice");
    char* h = nullptr;
    char* d = nullptr;
    if (!rc && sz > 0) {
        if (!(rc = check_cuda(cudaMallocHost(&h, (size_t)sz), "allocate pinned staging")) &&
            !(rc = check_cuda(cudaMalloc(&d, (size_t)sz), "allocate device text"))) {
            if (fread(h, 1, (size_t)sz, fp) != (size_t)sz) rc = fail(KT_ERR_IO, "short read on %s", path);
            if (!rc) rc = check_cuda(cudaMemcpyAsync(d, h, (size_t)sz, cudaMemcpyHostToDevice, e->stream), "H2D");
        }
    }
    fclose(fp);
    if (!rc) rc = kt::parse_tsv(e, d, (uint64_t)sz, d_src, d_dst, capacity, num_entries, num_nodes);
    if (d) cudaFree(d);
    if (h) cudaFreeHost(h);
    return rc;
}

}  // extern "C"
