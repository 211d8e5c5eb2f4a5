// Truss decomposition that allocates nothing: kt_decompose_noalloc.
//
// Some callers cannot let a library allocate device memory: programs whose device memory is
// owned by one memory manager with a fixed budget (a database or graph engine that hands out
// every byte itself), and latency-sensitive loops that cannot afford cudaMalloc/cudaFree, which
// may synchronize the whole device and take the driver's allocator lock.  For them this entry
// point runs the same device pipeline as kt_engine_decompose (CSR build, support count, peel,
// per-entry output) with all of its scratch - CSR arrays, sort buffers, queues, counters - carved
// from one statically sized device array declared below.  The caller passes device buffers for
// the input entries and the outputs.
//
// The array costs kNoAllocScratchBytes of device memory on every GPU where it is loaded, until
// the process exits.  CUDA loads modules lazily by default, so the array is usually backed when
// the first call on a device takes its address (or when the context is created, under
// CUDA_MODULE_LOADING=EAGER): that first call can fail with a CUDA error when device memory is
// short.  Later calls allocate nothing.
//
// Set-up: the first call on a device (with that device current) takes the array's device address
// with cudaGetSymbolAddress and lays the workspace out in it; that first call should happen before
// any stream capture.  Every later call looks the address up again (a host-side lookup): if the
// context was torn down and made again (cudaDeviceReset), the module is reloaded and the array may
// have moved, and the workspace is laid out again at the new address.  All calls on a device share
// the array, which keeps the previous call's contents; the pipeline clears what must start at zero
// (control words, degrees, supports, round stamps).  Calls on one device are serialized by a lock,
// and each call synchronizes its stream before it returns: two calls whose GPU work overlapped
// would race on the shared scratch.

#include <mutex>

#include "kt_device.cuh"
#include "kt_engine.h"

namespace {

constexpr uint32_t kNoAllocMaxNodes = 1u << 17;       // 131,072 vertices
constexpr uint64_t kNoAllocMaxEntries = 1ull << 19;   // 524,288 entries = 262,144 undirected edges
constexpr size_t kNoAllocScratchBytes = 40ull << 20;  // 40 MiB, checked against the layout at set-up
constexpr size_t kCtrlBytes = 512;                    // control words at the start of the array
static_assert(kCtrlBytes >= sizeof(uint32_t) * kt::kCtrlWords, "control block does not fit");
constexpr int kMaxDevices = 64;

// File-scope scratch.  In host code this name is only a stand-in; its device address comes from
// cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

struct NoAllocDevice {
    std::mutex mu;
    bool ready = false;
    void* base = nullptr;               // the array's device address at the last set-up
    kt_engine engine;                   // pointers carved from g_noalloc_scratch; no events, no arena
    uint32_t h_ctrl[kt::kCtrlWords];    // host copy of the control words (static, not pinned)
};

NoAllocDevice g_devices[kMaxDevices];

// With the device current: the workspace layout inside the array at device address `ptr`.
int set_up(int device, NoAllocDevice& d, void* ptr) {
    int rc;
    kt_engine& e = d.engine;
    e.device = device;
    if ((rc = kt::check_cuda(cudaDeviceGetAttribute(&e.num_sms, cudaDevAttrMultiProcessorCount, device),
                             "SM count")))
        return rc;
    const size_t need = kt::carve(&e, nullptr, kNoAllocMaxNodes, kNoAllocMaxEntries, false);
    if (need + kCtrlBytes > kNoAllocScratchBytes)
        return kt::fail(KT_ERR_INTERNAL, "no-allocation scratch too small: %zu bytes needed", need + kCtrlBytes);
    char* base = static_cast<char*>(ptr);
    e.ctrl = reinterpret_cast<uint32_t*>(base);
    kt::carve(&e, base + kCtrlBytes, kNoAllocMaxNodes, kNoAllocMaxEntries, false);
    e.cap_nodes = kNoAllocMaxNodes;
    e.cap_entries = kNoAllocMaxEntries;
    e.h_ctrl = d.h_ctrl;
    d.base = ptr;
    d.ready = true;
    return KT_OK;
}

}  // namespace

extern "C" int kt_decompose_noalloc(const uint32_t* d_src, const uint32_t* d_dst, uint64_t num_entries,
                                    uint32_t num_nodes, uint32_t* d_truss_per_entry, uint32_t* d_k_max,
                                    void* stream) {
    kt::clear_error();
    if (num_entries && (!d_src || !d_dst || !d_truss_per_entry))
        return kt::fail(KT_ERR_INVALID_ARG, "kt_decompose_noalloc: null device buffer");
    if (num_entries > kNoAllocMaxEntries || num_nodes > kNoAllocMaxNodes)
        return kt::fail(KT_ERR_TOO_LARGE,
                        "kt_decompose_noalloc: %llu entries and %u vertices exceed its fixed scratch "
                        "(at most %llu entries and %u vertices); use kt_engine_decompose",
                        (unsigned long long)num_entries, num_nodes, (unsigned long long)kNoAllocMaxEntries,
                        kNoAllocMaxNodes);
    int device = 0;
    int rc = kt::check_cuda(cudaGetDevice(&device), "cudaGetDevice");
    if (rc) return rc;
    if (device < 0 || device >= kMaxDevices) return kt::fail(KT_ERR_NO_DEVICE, "device %d out of range", device);
    NoAllocDevice& d = g_devices[device];
    std::lock_guard<std::mutex> lock(d.mu);
    // the array's address on every call: a context made again after a reset may have moved it
    void* ptr = nullptr;
    if ((rc = kt::check_cuda(cudaGetSymbolAddress(&ptr, g_noalloc_scratch),
                             "cudaGetSymbolAddress of the no-allocation scratch")))
        return rc;
    if ((!d.ready || ptr != d.base) && (rc = set_up(device, d, ptr))) return rc;
    kt_engine& e = d.engine;
    e.stream = static_cast<cudaStream_t>(stream);
    e.stats_ready = false;
    if ((rc = kt::build_graph(&e, d_src, d_dst, num_entries, num_nodes)) || (rc = kt::count_support(&e)) ||
        (rc = kt::peel_decompose(&e)) || (rc = kt::emit_truss_per_entry(&e, d_truss_per_entry, d_k_max)))
        return rc;
    // the call ends only when its GPU work has: then a peel wait that ran out is reported
    if ((rc = kt::check_cuda(cudaMemcpyAsync(d.h_ctrl, e.ctrl, sizeof(uint32_t), cudaMemcpyDeviceToHost, e.stream),
                             "read control word")) ||
        (rc = kt::check_cuda(cudaStreamSynchronize(e.stream), "synchronize")))
        return rc;
    if (d.h_ctrl[kt::kCtrlError] & kt::kErrTimeout)
        return kt::fail(KT_ERR_TIMEOUT, "a grid barrier wait of the peel kernel expired");
    if (d.h_ctrl[kt::kCtrlError] & kt::kErrRunaway)
        return kt::fail(KT_ERR_INTERNAL, "the peel kernel exceeded its round or level bound");
    return KT_OK;
}
