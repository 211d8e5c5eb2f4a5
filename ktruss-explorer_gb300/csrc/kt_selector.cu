// Learned schedule selector: a small FP32 MLP that picks the kernel schedule of a graph.
//
// No counterpart in the reference, whose variants (-d, -f, -r, -b, -t) are chosen by hand on the
// command line.  The network reads 16 statistics of the built graph (size, degree moments, the
// walk lengths min(deg u, deg v) of its edges, density) and predicts, from the autotuner's grid,
// the variant - support group x chunk width x compaction (18 classes, softmax) - and the recount
// switch (one logit: recount a round's survivors once its frontier holds half of the alive
// edges, or always decrement).  Layers 16 -> 64 -> 64 -> 19, ReLU, inputs standardized with the
// training set's mean and scale.
//
// Everything runs in hand-written FP32 kernels: the graph statistics and features, inference
// (one block of 64 threads per graph), and training - per-sample forward and backward through
// the activations, per-parameter weight gradients summed over the batch in a fixed order (no
// float atomics, so a gradient is reproducible bit for bit), and Adam.  Labels come from the
// autotuner's timings: the variant whose better recount setting is fastest, and whether the
// fastest recount-on schedule beats the fastest recount-off one.  Every schedule computes the
// same truss numbers, so a wrong prediction costs time, never correctness.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "kt_device.cuh"
#include "kt_engine.h"

struct kt_selector {
    int device = 0;
    cudaStream_t stream = nullptr;
    float* d_params = nullptr;          // kt::sel::kAll floats: weights, biases, mean, scale
    std::vector<float> h_params;        // host copy
};

namespace kt {

namespace sel {

constexpr int F = KT_SELECTOR_FEATURES, H = 64, V = KT_SELECTOR_VARIANTS, O = V + 1;
constexpr int kW1 = 0, kB1 = kW1 + H * F, kW2 = kB1 + H, kB2 = kW2 + H * H, kW3 = kB2 + H, kB3 = kW3 + O * H;
constexpr int kParams = kB3 + O;
constexpr int kMean = kParams, kScale = kParams + F, kAll = kParams + 2 * F;
static_assert(kParams == KT_SELECTOR_PARAMS, "parameter count");

// Forward pass of one sample by the first H threads of a block (all its threads call it: it holds
// block barriers); xs: standardized input in shared memory.
__device__ void forward(const float* __restrict__ P, const float* xs, float* h1s, float* h2s, float* os) {
    const int j = threadIdx.x;
    float a;
    if (j < H) {
        a = P[kB1 + j];
        for (int i = 0; i < F; ++i) a += P[kW1 + j * F + i] * xs[i];
        h1s[j] = a > 0.f ? a : 0.f;
    }
    __syncthreads();
    if (j < H) {
        a = P[kB2 + j];
        for (int i = 0; i < H; ++i) a += P[kW2 + j * H + i] * h1s[i];
        h2s[j] = a > 0.f ? a : 0.f;
    }
    __syncthreads();
    if (j < O) {
        a = P[kB3 + j];
        for (int i = 0; i < H; ++i) a += P[kW3 + j * H + i] * h2s[i];
        os[j] = a;
    }
    __syncthreads();
}

// Schedule index in the autotuner's grid order: variant * 2 + recount.
__device__ uint32_t choose(const float* os) {
    int best = 0;
    for (int v = 1; v < V; ++v)
        if (os[v] > os[best]) best = v;
    return (uint32_t)best * 2u + (os[V] > 0.f ? 1u : 0u);
}

__device__ __forceinline__ float warp_sum(float a) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(kFullMask, a, o);
    return a;
}

// Dense layer for inference, one unit per warp at a time: the lanes read the unit's weight row
// coalesced (K <= 64 inputs, two per lane) and sum by shuffles; each warp issues the loads of kU
// units before it reduces any, so the weights cost a few L2 round trips instead of one per input.
template <int K, int N, bool kRelu>
__device__ __forceinline__ void infer_layer(const float* __restrict__ W, const float* __restrict__ bias,
                                            const float* in, float* out) {
    static_assert(K <= 64, "two inputs per lane");
    constexpr int kU = 8;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j0 = warp * kU; j0 < N; j0 += nw * kU) {
        float a[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const int j = j0 + u;
            a[u] = 0.f;
            if (j < N) {
                if (lane < K) a[u] = W[j * K + lane] * in[lane];
                if (lane + 32 < K) a[u] += W[j * K + lane + 32] * in[lane + 32];
            }
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const float t = warp_sum(a[u]) + (j0 + u < N ? bias[j0 + u] : 0.f);
            if (lane == 0 && j0 + u < N) out[j0 + u] = kRelu ? (t > 0.f ? t : 0.f) : t;
        }
    }
}

// Forward pass of one sample for inference by all threads of a block (whole warps; it holds block
// barriers).  Same network as `forward`; the sums run in another order, so logits may differ from
// it in the last bits.
__device__ void infer(const float* __restrict__ P, const float* xs, float* h1s, float* h2s, float* os) {
    infer_layer<F, H, true>(P + kW1, P + kB1, xs, h1s);
    __syncthreads();
    infer_layer<H, H, true>(P + kW2, P + kB2, h1s, h2s);
    __syncthreads();
    infer_layer<H, O, false>(P + kW3, P + kB3, h2s, os);
    __syncthreads();
}

// One block per training sample: forward, loss, and the gradients of the pre-activations
// (D3 = d loss / d logits, D2, D1), all divided by the batch size.  Also stores the sample's
// standardized input and activations for the weight gradients.
__global__ void __launch_bounds__(H) k_train_step(const float* __restrict__ P, const float* __restrict__ X_all,
                                                  const uint32_t* __restrict__ labels_all,
                                                  const uint32_t* __restrict__ order, uint32_t B,
                                                  float* __restrict__ Xb, float* __restrict__ H1, float* __restrict__ H2,
                                                  float* __restrict__ D1, float* __restrict__ D2, float* __restrict__ D3,
                                                  float* __restrict__ loss) {
    __shared__ float xs[F], h1s[H], h2s[H], os[O], d3s[O], d2s[H];
    const uint32_t b = blockIdx.x, j = threadIdx.x;
    const uint32_t s = order[b];
    if (j < F) {
        xs[j] = X_all[(size_t)s * F + j];
        Xb[(size_t)b * F + j] = xs[j];
    }
    __syncthreads();
    forward(P, xs, h1s, h2s, os);
    H1[(size_t)b * H + j] = h1s[j];
    H2[(size_t)b * H + j] = h2s[j];
    const uint32_t yv = labels_all[2 * s], yr = labels_all[2 * s + 1];
    const float inv_b = 1.f / (float)B;
    if (j < V) {
        float mx = os[0];
        for (int v = 1; v < V; ++v) mx = fmaxf(mx, os[v]);
        float sum = 0.f;
        for (int v = 0; v < V; ++v) sum += expf(os[v] - mx);
        const float p = expf(os[j] - mx) / sum;
        d3s[j] = (p - (j == yv ? 1.f : 0.f)) * inv_b;
        if (j == 0) {
            const float z = os[V], r = (float)yr;
            const float bce = fmaxf(z, 0.f) - z * r + log1pf(expf(-fabsf(z)));
            loss[b] = logf(sum) + mx - os[yv] + bce;
        }
    } else if (j == V) {
        const float z = os[V];
        d3s[V] = (1.f / (1.f + expf(-z)) - (float)yr) * inv_b;
    }
    __syncthreads();
    if (j < O) D3[(size_t)b * O + j] = d3s[j];
    float g = 0.f;
    for (int o = 0; o < O; ++o) g += P[kW3 + o * H + j] * d3s[o];
    g = h2s[j] > 0.f ? g : 0.f;
    d2s[j] = g;
    D2[(size_t)b * H + j] = g;
    __syncthreads();
    g = 0.f;
    for (int k = 0; k < H; ++k) g += P[kW2 + k * H + j] * d2s[k];
    D1[(size_t)b * H + j] = h1s[j] > 0.f ? g : 0.f;
}

// Gradient of every parameter, summed over the batch in sample order.
__global__ void k_weight_grad(const float* __restrict__ Xb, const float* __restrict__ H1, const float* __restrict__ H2,
                              const float* __restrict__ D1, const float* __restrict__ D2,
                              const float* __restrict__ D3, uint32_t B, float* __restrict__ G) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= kParams) return;
    const float* dv;
    const float* av = nullptr;
    int dstride, astride = 0, row, col = 0;
    if (p < kB1) {
        row = p / F, col = p % F, dv = D1, dstride = H, av = Xb, astride = F;
    } else if (p < kW2) {
        row = p - kB1, dv = D1, dstride = H;
    } else if (p < kB2) {
        row = (p - kW2) / H, col = (p - kW2) % H, dv = D2, dstride = H, av = H1, astride = H;
    } else if (p < kW3) {
        row = p - kB2, dv = D2, dstride = H;
    } else if (p < kB3) {
        row = (p - kW3) / H, col = (p - kW3) % H, dv = D3, dstride = O, av = H2, astride = H;
    } else {
        row = p - kB3, dv = D3, dstride = O;
    }
    float g = 0.f;
    for (uint32_t b = 0; b < B; ++b) {
        const float d = dv[(size_t)b * dstride + row];
        g += av ? d * av[(size_t)b * astride + col] : d;
    }
    G[p] = g;
}

__global__ void k_adam(float* __restrict__ P, const float* __restrict__ G, float* __restrict__ M,
                       float* __restrict__ Vv, float lr, float beta1, float beta2, float eps, float bc1, float bc2) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= kParams) return;
    const float g = G[p];
    const float m = beta1 * M[p] + (1.f - beta1) * g;
    const float v = beta2 * Vv[p] + (1.f - beta2) * g * g;
    M[p] = m;
    Vv[p] = v;
    P[p] -= lr * (m / bc1) / (sqrtf(v / bc2) + eps);
}

// Inference on raw features: one block per sample.
__global__ void __launch_bounds__(H) k_predict(const float* __restrict__ P, const float* __restrict__ X, uint32_t* choice) {
    __shared__ float xs[F], h1s[H], h2s[H], os[O];
    const uint32_t b = blockIdx.x, j = threadIdx.x;
    if (j < F) xs[j] = (X[(size_t)b * F + j] - P[kMean + j]) / P[kScale + j];
    __syncthreads();
    infer(P, xs, h1s, h2s, os);
    if (j == 0) choice[b] = choose(os);
}

// Graph statistics (integers, exact): per vertex (rank space) degree d and oriented out-degree
// od; per edge the walk length min(d_u, d_v).  Sums except kMaxD and kMaxOd (maxima).
enum : int {
    kSumD2 = 0, kMaxD, kLowD, kHighD, kMaxOd, kSumOd2, kSumMin, kSumMin2, kShortMin, kLongMin, kNumStat,
    kTicket = 15, kStats = 16
};
constexpr int kSelThreads = 256;                  // statistics block (its first H threads run the network)
constexpr int kSelWarps = kSelThreads / 32;
static_assert(kSelThreads >= H && H >= F && H >= O, "the network runs on the first H threads");

__device__ __forceinline__ bool stat_is_max(int s) { return s == kMaxD || s == kMaxOd; }

// Statistics, features and choice in one launch: every block reduces its share of the vertex and
// edge statistics to one partial per statistic (part[block * kNumStat + s], plain stores - no
// contended atomics); the last block to finish (an atomic ticket in st[kTicket], after a fence)
// reduces the partials, turns them into the 16 features and, with P, runs the network and writes
// the choice and its schedule.  st[kTicket] must be zero on entry; gridDim.x <= kSelMaxBlocks.
__global__ void __launch_bounds__(kSelThreads) k_select(const uint32_t* __restrict__ s_ptr,
                                                        const uint32_t* __restrict__ o_ptr,
                                                        const uint32_t* __restrict__ e_src,
                                                        const uint32_t* __restrict__ o_col, uint32_t n, uint32_t m,
                                                        unsigned long long* __restrict__ st,
                                                        unsigned long long* __restrict__ part,
                                                        const float* __restrict__ P, float* __restrict__ feat,
                                                        uint32_t* __restrict__ choice, uint32_t* __restrict__ sched) {
    __shared__ float fs[F], xs[F], h1s[H], h2s[H], os[O];
    __shared__ unsigned long long ws[kSelWarps][kNumStat], tot[kNumStat];
    __shared__ uint32_t last;
    unsigned long long v[kNumStat] = {};
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < n; x += stride) {
        const uint32_t d = s_ptr[x + 1] - s_ptr[x], od = o_ptr[x + 1] - o_ptr[x];
        v[kSumD2] += (unsigned long long)d * d;
        v[kSumOd2] += (unsigned long long)od * od;
        v[kLowD] += d <= 2;
        v[kHighD] += d >= 64;
        v[kMaxD] = max(v[kMaxD], (unsigned long long)d);
        v[kMaxOd] = max(v[kMaxOd], (unsigned long long)od);
    }
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < m; j += stride) {
        const uint32_t a = e_src[j], b = o_col[j];
        const uint32_t w = min(s_ptr[a + 1] - s_ptr[a], s_ptr[b + 1] - s_ptr[b]);
        v[kSumMin] += w;
        v[kSumMin2] += (unsigned long long)w * w;
        v[kShortMin] += w <= 8;
        v[kLongMin] += w >= 32;
    }
#pragma unroll
    for (int q = 0; q < kNumStat; ++q) {
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long t = __shfl_xor_sync(kFullMask, v[q], o);
            v[q] = stat_is_max(q) ? max(v[q], t) : v[q] + t;
        }
    }
    const uint32_t warp = threadIdx.x >> 5;
    if (lane_id() == 0)
#pragma unroll
        for (int q = 0; q < kNumStat; ++q) ws[warp][q] = v[q];
    __syncthreads();
    if (threadIdx.x < kNumStat) {
        const int q = threadIdx.x;
        unsigned long long r = 0;
        for (int w = 0; w < kSelWarps; ++w) r = stat_is_max(q) ? max(r, ws[w][q]) : r + ws[w][q];
        part[(size_t)blockIdx.x * kNumStat + q] = r;
        __threadfence();
    }
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(st + kTicket, 1ull) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    // last block: partials of all blocks, kNumStat groups of kSelThreads / kNumStat threads
    if (threadIdx.x < kNumStat) tot[threadIdx.x] = 0;
    __syncthreads();
    constexpr uint32_t kGroup = kSelThreads / kNumStat;
    if (threadIdx.x < kGroup * kNumStat) {
        const int q = threadIdx.x / kGroup;
        unsigned long long r = 0;
        for (uint32_t blk = threadIdx.x % kGroup; blk < gridDim.x; blk += kGroup) {
            const unsigned long long t = __ldcg(part + (size_t)blk * kNumStat + q);
            r = stat_is_max(q) ? max(r, t) : r + t;
        }
        if (stat_is_max(q))
            atomicMax(&tot[q], r);
        else
            atomicAdd(&tot[q], r);
    }
    __syncthreads();
    const int j = threadIdx.x;
    if (j == 0) st[kTicket] = 0;  // ready for the next call
    if (j < F) {  // one feature per thread
        const double dn = n > 0 ? (double)n : 1.0, dm = m > 0 ? (double)m : 1.0;
        const double avg = 2.0 * m / dn;
        double f = 0.0;
        switch (j) {
            case 0: f = log2(dn); break;
            case 1: f = log2(dm + 1.0); break;
            case 2: f = avg; break;
            case 3: f = log2((double)tot[kMaxD] + 1.0); break;
            case 4: f = avg > 0 ? sqrt(fmax((double)tot[kSumD2] / dn - avg * avg, 0.0)) / avg : 0.0; break;
            case 5: f = log2((double)tot[kSumD2] / (2.0 * dm) + 1.0); break;
            case 6: f = (double)tot[kLowD] / dn; break;
            case 7: f = (double)tot[kHighD] / dn; break;
            case 8: f = log2((double)tot[kMaxOd] + 1.0); break;
            case 9: f = m > 0 ? sqrt((double)tot[kSumOd2] / dn) / (m / dn) : 0.0; break;
            case 10: f = log2((double)tot[kSumMin] / dm + 1.0); break;
            case 11: f = (double)tot[kShortMin] / dm; break;
            case 12: f = (double)tot[kLongMin] / dm; break;
            case 13: f = n > 1 ? log2(2.0 * m / (dn * (dn - 1.0)) + 1e-12) : 0.0; break;
            case 14: f = log2(sqrt((double)tot[kSumMin2] / dm) + 1.0); break;
            default: f = avg > 0 ? log2((double)tot[kMaxD] / avg + 1.0) : 0.0; break;
        }
        fs[j] = (float)f;
    }
    __syncthreads();
    if (j < F) {
        feat[j] = fs[j];
        if (P) xs[j] = (fs[j] - P[kMean + j]) / P[kScale + j];
    }
    __syncthreads();
    if (!P) return;
    infer(P, xs, h1s, h2s, os);
    if (j == 0) {
        const uint32_t c = choose(os);
        *choice = c;
        // the chosen schedule for the support and peel kernels of this call (ctrl[kPSched..+3])
        grid_schedule(c, sched, sched + 1, sched + 2, sched + 3);
    }
}

// Labels from one graph's timings (kt_schedule_grid order, index = variant * 2 + recount).
void labels_of(const float* t, uint32_t* yv, uint32_t* yr) {
    uint32_t best_v = 0;
    float best_t = 0;
    float best_r[2] = {0, 0};
    for (uint32_t v = 0; v < (uint32_t)V; ++v) {
        const float tv = std::min(t[2 * v], t[2 * v + 1]);
        if (v == 0 || tv < best_t) {
            best_t = tv;
            best_v = v;
        }
        for (int r = 0; r < 2; ++r)
            if (v == 0 || t[2 * v + r] < best_r[r]) best_r[r] = t[2 * v + r];
    }
    *yv = best_v;
    *yr = best_r[1] < best_r[0] ? 1u : 0u;
}

// SplitMix64 for the initial weights and the minibatch order.
struct Mix {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

int upload(kt_selector* s) {
    return check_cuda(cudaMemcpyAsync(s->d_params, s->h_params.data(), sizeof(float) * kAll, cudaMemcpyHostToDevice,
                                      s->stream),
                      "upload selector parameters");
}

// Device buffers of one training call.
struct TrainBuffers {
    float *X = nullptr, *Xb = nullptr, *H1 = nullptr, *H2 = nullptr, *D1 = nullptr, *D2 = nullptr, *D3 = nullptr;
    float *loss = nullptr, *G = nullptr, *M = nullptr, *Vv = nullptr;
    uint32_t *labels = nullptr, *order = nullptr;
    ~TrainBuffers() {
        for (void* p : {(void*)X, (void*)Xb, (void*)H1, (void*)H2, (void*)D1, (void*)D2, (void*)D3, (void*)loss,
                        (void*)G, (void*)M, (void*)Vv, (void*)labels, (void*)order})
            if (p) cudaFree(p);
    }
    int alloc(uint32_t n, uint32_t B) {
        int rc;
        if ((rc = check_cuda(cudaMalloc(&X, sizeof(float) * n * F), "selector buffers")) ||
            (rc = check_cuda(cudaMalloc(&Xb, sizeof(float) * B * F), "selector buffers")) ||
            (rc = check_cuda(cudaMalloc(&H1, sizeof(float) * B * H), "selector buffers")) ||
            (rc = check_cuda(cudaMalloc(&H2, sizeof(float) * B * H), "selector buffers")) ||
            (rc = check_cuda(cudaMalloc(&D1, sizeof(float) * B * H), "selector buffers")) ||
            (rc = check_cuda(cudaMalloc(&D2, sizeof(float) * B * H), "selector buffers")) ||
            (rc = check_cuda(cudaMalloc(&D3, sizeof(float) * B * O), "selector buffers")) ||
            (rc = check_cuda(cudaMalloc(&loss, sizeof(float) * n), "selector buffers")) ||
            (rc = check_cuda(cudaMalloc(&G, sizeof(float) * kParams), "selector buffers")) ||
            (rc = check_cuda(cudaMalloc(&M, sizeof(float) * kParams), "selector buffers")) ||
            (rc = check_cuda(cudaMalloc(&Vv, sizeof(float) * kParams), "selector buffers")) ||
            (rc = check_cuda(cudaMalloc(&labels, sizeof(uint32_t) * 2 * n), "selector buffers")) ||
            (rc = check_cuda(cudaMalloc(&order, sizeof(uint32_t) * n), "selector buffers")))
            return rc;
        return KT_OK;
    }
};

// Standardized features and labels of a data set, uploaded.
int load_data(kt_selector* s, TrainBuffers& tb, const float* features, const float* times, uint32_t n) {
    std::vector<float> x((size_t)n * F);
    std::vector<uint32_t> y(2 * (size_t)n);
    for (uint32_t i = 0; i < n; ++i) {
        for (int f = 0; f < F; ++f)
            x[(size_t)i * F + f] = (features[(size_t)i * F + f] - s->h_params[kMean + f]) / s->h_params[kScale + f];
        labels_of(times + (size_t)i * KT_SELECTOR_SCHEDULES, &y[2 * i], &y[2 * i + 1]);
    }
    int rc;
    if ((rc = check_cuda(cudaMemcpyAsync(tb.X, x.data(), sizeof(float) * x.size(), cudaMemcpyHostToDevice, s->stream),
                         "upload features")) ||
        (rc = check_cuda(cudaMemcpyAsync(tb.labels, y.data(), sizeof(uint32_t) * y.size(), cudaMemcpyHostToDevice,
                                         s->stream), "upload labels")) ||
        (rc = check_cuda(cudaStreamSynchronize(s->stream), "synchronize")))
        return rc;
    return KT_OK;
}

int batch_gradient(kt_selector* s, TrainBuffers& tb, const uint32_t* order, uint32_t B) {
    k_train_step<<<B, H, 0, s->stream>>>(s->d_params, tb.X, tb.labels, order, B, tb.Xb, tb.H1, tb.H2, tb.D1, tb.D2,
                                         tb.D3, tb.loss);
    int rc = check_cuda(cudaGetLastError(), "k_train_step");
    if (rc) return rc;
    k_weight_grad<<<(kParams + 255) / 256, 256, 0, s->stream>>>(tb.Xb, tb.H1, tb.H2, tb.D1, tb.D2, tb.D3, B, tb.G);
    return check_cuda(cudaGetLastError(), "k_weight_grad");
}

}  // namespace sel

// With a selector attached: the features and the network's choice are computed on the device, and
// the choice is written to the control block, where the support count and the peel read it - the
// call enqueues its whole pipeline without waiting for the choice (no host read).  The host learns
// the chosen schedule when the statistics are read (finish_stats).
int select_schedule(kt_engine* e) {
    e->sched_on_device = false;
    kt_selector* s = e->selector;
    if (!s || e->m == 0) return KT_OK;
    if (s->device != e->device) return fail(KT_ERR_INVALID_ARG, "the selector lives on another device");
    int rc;
    if ((rc = graph_features(e, s->d_params))) return rc;
    e->sched_on_device = true;
    return KT_OK;
}

int graph_features(kt_engine* e, const float* d_params) {
    unsigned long long* st = reinterpret_cast<unsigned long long*>(e->sel_stats);
    // no clearing launch: the ticket is zeroed with the workspace and the last block of every
    // launch clears it again (a launch either runs all its blocks or, if it fails, none)
    // one launch: blocks for at least four vertices or edges per thread, at most eight per SM and
    // kSelMaxBlocks (the partials buffer)
    const uint64_t work = std::max<uint64_t>(e->n, e->m);
    const uint64_t cap = std::min<uint64_t>((uint64_t)e->num_sms * 8, kSelMaxBlocks);
    const uint32_t blocks =
        (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((work + 4 * sel::kSelThreads - 1) / (4 * sel::kSelThreads), cap));
    sel::k_select<<<blocks, sel::kSelThreads, 0, e->stream>>>(
        e->s_ptr, e->o_ptr, e->e_src, e->o_col, e->n, e->m, st, reinterpret_cast<unsigned long long*>(e->sel_part),
        d_params, e->sel_feat, e->sel_choice, e->ctrl + kPSched);
    count_launch(e);
    return check_launch(e, "k_select");
}

}  // namespace kt

using kt::check_cuda;
using kt::fail;

extern "C" {

int kt_selector_create(int device, uint64_t seed, kt_selector** out) {
    kt::clear_error();
    if (!out) return fail(KT_ERR_INVALID_ARG, "kt_selector_create: null output");
    *out = nullptr;
    int rc = check_cuda(cudaSetDevice(device), "cudaSetDevice");
    if (rc) return rc;
    kt_selector* s = new kt_selector();
    s->device = device;
    s->h_params.assign(kt::sel::kAll, 0.f);
    // He-uniform weights, zero biases, identity standardization
    kt::sel::Mix rng{seed};
    auto init = [&](int off, int rows, int cols) {
        const double lim = std::sqrt(6.0 / cols);
        for (int i = 0; i < rows * cols; ++i) s->h_params[off + i] = (float)((2.0 * rng.uniform() - 1.0) * lim);
    };
    init(kt::sel::kW1, kt::sel::H, kt::sel::F);
    init(kt::sel::kW2, kt::sel::H, kt::sel::H);
    init(kt::sel::kW3, kt::sel::O, kt::sel::H);
    for (int f = 0; f < kt::sel::F; ++f) s->h_params[kt::sel::kScale + f] = 1.f;
    if ((rc = check_cuda(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking), "create stream")) ||
        (rc = check_cuda(cudaMalloc(&s->d_params, sizeof(float) * kt::sel::kAll), "allocate selector")) ||
        (rc = kt::sel::upload(s)) || (rc = check_cuda(cudaStreamSynchronize(s->stream), "synchronize"))) {
        kt_selector_destroy(s);
        return rc;
    }
    *out = s;
    return KT_OK;
}

int kt_selector_destroy(kt_selector* s) {
    if (!s) return KT_OK;
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    if (s->d_params) cudaFree(s->d_params);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return KT_OK;
}

int kt_selector_get_params(kt_selector* s, float* params, float* mean, float* scale) {
    kt::clear_error();
    if (!s) return fail(KT_ERR_INVALID_ARG, "kt_selector_get_params: null selector");
    if (params) std::memcpy(params, s->h_params.data(), sizeof(float) * kt::sel::kParams);
    if (mean) std::memcpy(mean, s->h_params.data() + kt::sel::kMean, sizeof(float) * kt::sel::F);
    if (scale) std::memcpy(scale, s->h_params.data() + kt::sel::kScale, sizeof(float) * kt::sel::F);
    return KT_OK;
}

int kt_selector_set_params(kt_selector* s, const float* params, const float* mean, const float* scale) {
    kt::clear_error();
    if (!s) return fail(KT_ERR_INVALID_ARG, "kt_selector_set_params: null selector");
    if (scale)
        for (int f = 0; f < kt::sel::F; ++f)
            if (!(scale[f] > 0.f)) return fail(KT_ERR_INVALID_ARG, "scale[%d] must be positive", f);
    if (params) std::memcpy(s->h_params.data(), params, sizeof(float) * kt::sel::kParams);
    if (mean) std::memcpy(s->h_params.data() + kt::sel::kMean, mean, sizeof(float) * kt::sel::F);
    if (scale) std::memcpy(s->h_params.data() + kt::sel::kScale, scale, sizeof(float) * kt::sel::F);
    int rc = check_cuda(cudaSetDevice(s->device), "cudaSetDevice");
    if (rc || (rc = kt::sel::upload(s))) return rc;
    return check_cuda(cudaStreamSynchronize(s->stream), "synchronize");
}

int kt_selector_gradient(kt_selector* s, const float* features, const float* times, uint32_t n, float* grad,
                         float* loss) {
    kt::clear_error();
    if (!s || !features || !times || n == 0) return fail(KT_ERR_INVALID_ARG, "kt_selector_gradient: empty input");
    int rc = check_cuda(cudaSetDevice(s->device), "cudaSetDevice");
    if (rc) return rc;
    kt::sel::TrainBuffers tb;
    if ((rc = tb.alloc(n, n)) || (rc = kt::sel::load_data(s, tb, features, times, n))) return rc;
    std::vector<uint32_t> order(n);
    std::iota(order.begin(), order.end(), 0u);
    if ((rc = check_cuda(cudaMemcpyAsync(tb.order, order.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice,
                                         s->stream), "upload order")) ||
        (rc = kt::sel::batch_gradient(s, tb, tb.order, n)))
        return rc;
    std::vector<float> l(n);
    if ((grad && (rc = check_cuda(cudaMemcpyAsync(grad, tb.G, sizeof(float) * kt::sel::kParams, cudaMemcpyDeviceToHost,
                                                  s->stream), "read gradient"))) ||
        (rc = check_cuda(cudaMemcpyAsync(l.data(), tb.loss, sizeof(float) * n, cudaMemcpyDeviceToHost, s->stream),
                         "read loss")) ||
        (rc = check_cuda(cudaStreamSynchronize(s->stream), "synchronize")))
        return rc;
    if (loss) {
        double sum = 0;
        for (float v : l) sum += v;
        *loss = (float)(sum / n);
    }
    return KT_OK;
}

int kt_selector_train(kt_selector* s, const float* features, const float* times, uint32_t n, uint32_t epochs,
                      uint32_t batch, float lr, uint64_t seed, float* epoch_loss) {
    kt::clear_error();
    if (!s || !features || !times || n == 0 || batch == 0 || !(lr > 0.f))
        return fail(KT_ERR_INVALID_ARG, "kt_selector_train: empty input, zero batch or non-positive rate");
    int rc = check_cuda(cudaSetDevice(s->device), "cudaSetDevice");
    if (rc) return rc;
    // standardization from the training set
    for (int f = 0; f < kt::sel::F; ++f) {
        double mu = 0, sq = 0;
        for (uint32_t i = 0; i < n; ++i) mu += features[(size_t)i * kt::sel::F + f];
        mu /= n;
        for (uint32_t i = 0; i < n; ++i) {
            const double d = features[(size_t)i * kt::sel::F + f] - mu;
            sq += d * d;
        }
        const double sd = std::sqrt(sq / n);
        s->h_params[kt::sel::kMean + f] = (float)mu;
        s->h_params[kt::sel::kScale + f] = sd > 1e-6 ? (float)sd : 1.f;
    }
    if ((rc = kt::sel::upload(s))) return rc;
    const uint32_t B = batch < n ? batch : n;
    kt::sel::TrainBuffers tb;
    if ((rc = tb.alloc(n, B)) || (rc = kt::sel::load_data(s, tb, features, times, n))) return rc;
    if ((rc = check_cuda(cudaMemsetAsync(tb.M, 0, sizeof(float) * kt::sel::kParams, s->stream), "clear moments")) ||
        (rc = check_cuda(cudaMemsetAsync(tb.Vv, 0, sizeof(float) * kt::sel::kParams, s->stream), "clear moments")))
        return rc;
    kt::sel::Mix rng{seed};
    std::vector<uint32_t> order(n);
    std::vector<float> l(n);
    const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
    uint64_t t = 0;
    for (uint32_t ep = 0; ep < epochs; ++ep) {
        std::iota(order.begin(), order.end(), 0u);
        for (uint32_t i = n - 1; i > 0; --i) std::swap(order[i], order[rng.next() % (i + 1)]);
        if ((rc = check_cuda(cudaMemcpyAsync(tb.order, order.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice,
                                             s->stream), "upload order")))
            return rc;
        double sum = 0;
        for (uint32_t off = 0; off < n; off += B) {
            const uint32_t b = std::min(B, n - off);
            if ((rc = kt::sel::batch_gradient(s, tb, tb.order + off, b))) return rc;
            ++t;
            const float bc1 = (float)(1.0 - std::pow((double)beta1, (double)t));
            const float bc2 = (float)(1.0 - std::pow((double)beta2, (double)t));
            kt::sel::k_adam<<<(kt::sel::kParams + 255) / 256, 256, 0, s->stream>>>(s->d_params, tb.G, tb.M, tb.Vv, lr,
                                                                                  beta1, beta2, eps, bc1, bc2);
            if ((rc = check_cuda(cudaGetLastError(), "k_adam")) ||
                (rc = check_cuda(cudaMemcpyAsync(l.data() + off, tb.loss, sizeof(float) * b, cudaMemcpyDeviceToHost,
                                                 s->stream), "read loss")))
                return rc;
        }
        if ((rc = check_cuda(cudaStreamSynchronize(s->stream), "synchronize"))) return rc;
        for (uint32_t i = 0; i < n; ++i) sum += l[i];
        if (epoch_loss) epoch_loss[ep] = (float)(sum / n);
    }
    if ((rc = check_cuda(cudaMemcpyAsync(s->h_params.data(), s->d_params, sizeof(float) * kt::sel::kParams,
                                         cudaMemcpyDeviceToHost, s->stream), "read parameters")))
        return rc;
    return check_cuda(cudaStreamSynchronize(s->stream), "synchronize");
}

int kt_selector_predict(kt_selector* s, const float* features, uint32_t n, kt_schedule* out) {
    kt::clear_error();
    if (!s || (n && (!features || !out))) return fail(KT_ERR_INVALID_ARG, "kt_selector_predict: null argument");
    if (n == 0) return KT_OK;
    int rc = check_cuda(cudaSetDevice(s->device), "cudaSetDevice");
    if (rc) return rc;
    float* d_x = nullptr;
    uint32_t* d_c = nullptr;
    std::vector<uint32_t> c(n);
    if ((rc = check_cuda(cudaMalloc(&d_x, sizeof(float) * n * kt::sel::F), "allocate")) ||
        (rc = check_cuda(cudaMalloc(&d_c, sizeof(uint32_t) * n), "allocate")) ||
        (rc = check_cuda(cudaMemcpyAsync(d_x, features, sizeof(float) * n * kt::sel::F, cudaMemcpyHostToDevice,
                                         s->stream), "upload features"))) {
        cudaFree(d_x);
        cudaFree(d_c);
        return rc;
    }
    kt::sel::k_predict<<<n, kt::sel::H, 0, s->stream>>>(s->d_params, d_x, d_c);
    rc = check_cuda(cudaGetLastError(), "k_predict");
    if (!rc)
        rc = check_cuda(cudaMemcpyAsync(c.data(), d_c, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, s->stream),
                        "read choices");
    if (!rc) rc = check_cuda(cudaStreamSynchronize(s->stream), "synchronize");
    cudaFree(d_x);
    cudaFree(d_c);
    if (rc) return rc;
    kt_schedule grid[KT_SELECTOR_SCHEDULES];
    kt_schedule_grid(grid, KT_SELECTOR_SCHEDULES);
    for (uint32_t i = 0; i < n; ++i) out[i] = grid[c[i] < KT_SELECTOR_SCHEDULES ? c[i] : 0];
    return KT_OK;
}

}  // extern "C"
