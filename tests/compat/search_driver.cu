// Host build of the engine's row-search helpers (kt_device.cuh), for tests/test_search.py: reads
// an array, its queries (lo hi t) and prints fenced_lower_bound and lower_bound_u32 for each.
#include <cstdint>
#include <cstdio>
#include <vector>

#include "kt_device.cuh"

int main() {
    unsigned long long m = 0, q = 0;
    if (scanf("%llu", &m) != 1) return 1;
    std::vector<uint32_t> a(m + 1), fence(m / 32 + 2);
    for (unsigned long long i = 0; i < m; ++i)
        if (scanf("%u", &a[i]) != 1) return 1;
    for (unsigned long long f = 0; f * 32 < m; ++f) fence[f] = a[f * 32];  // as k_fences
    if (scanf("%llu", &q) != 1) return 1;
    for (unsigned long long i = 0; i < q; ++i) {
        uint32_t lo, hi, t;
        if (scanf("%u %u %u", &lo, &hi, &t) != 3) return 1;
        printf("%u %u\n", kt::fenced_lower_bound(a.data(), fence.data(), lo, hi, t),
               lo + kt::lower_bound_u32(a.data() + lo, hi - lo, t));
    }
    return 0;
}
