// Checks pma::ordered_sort against std::sort on inputs with many equal keys (the pore stage's
// maximum-ball order): the permutations must be identical. Built and run by
// tests/test_ordered_sort.py.
#include "ordered_sort.h"
#include <random>
#include <vector>
#include <cstdio>
int main() {
    std::mt19937_64 rng(1);
    for (int t = 0; t < 40; ++t) {
        size_t n = (t % 4 == 0) ? (rng() % 100) : (rng() % 3000000);
        int distinct = 1 + rng() % (t % 3 == 0 ? 3 : 1000);
        std::vector<unsigned long long> a(n);
        for (size_t i = 0; i < n; ++i) a[i] = ((rng() % distinct) << 32) | i;
        if (t % 5 == 1) std::sort(a.begin(), a.end());  // sorted input
        if (t % 5 == 2) std::reverse(a.begin(), a.end());
        auto b = a;
        auto less = [](unsigned long long x, unsigned long long y) { return (x >> 32) > (y >> 32); };
        std::sort(a.begin(), a.end(), less);
        auto c = b;
        pma::ordered_sort(b.begin(), b.end(), less, 1 + t % 4);
        if (a != b) { printf("MISMATCH t=%d n=%zu\n", t, n); return 1; }
        // raw pointers, as the pore stage sorts a page-locked buffer; level 0 is std::sort's own steps
        pma::ordered_sort(c.data(), c.data() + c.size(), less, t % 5);
        if (a != c) { printf("MISMATCH (pointers) t=%d n=%zu\n", t, n); return 1; }
    }
    printf("ok\n");
    return 0;
}
