// The team sort of csrc/stdsort.h against std::sort on seeded random inputs:
// the permutations must be identical (ties included), and the pass it runs
// on its threads after sorting (a gather by the permutation, as the FASTA
// readers use it) must see the final permutation and cover every position
// once.  Built and run by tests/test_stdsort.py; prints the number of
// mismatches and exits non-zero on any.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <numeric>
#include <random>
#include <vector>

#include "stdsort.h"

int main(int argc, char** argv) {
    const int trials = argc > 1 ? std::atoi(argv[1]) : 160;
    std::mt19937_64 rng(argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 20261203ull);
    int bad = 0;
    for (int trial = 0; trial < trials; trial++) {
        const int n = 65536 + (int)(rng() % 250000);
        std::vector<int32_t> key(n);
        const int mode = trial % 8;
        std::lognormal_distribution<double> ln(std::log(1500.0), 0.5);
        for (int i = 0; i < n; i++) {
            switch (mode) {
                case 0: key[i] = (int32_t)std::min(10000.0, std::max(300.0, ln(rng))); break;
                case 1: key[i] = 150; break;                          // all equal
                case 2: key[i] = (int32_t)(rng() % 2); break;         // two values
                case 3: key[i] = 140 + (int32_t)(rng() % 12); break;  // a few values
                case 4: key[i] = (int32_t)(rng() % 1000000); break;   // nearly distinct
                case 5: key[i] = n - i; break;                        // already in order
                case 6: key[i] = i / 3; break;                        // reversed, with ties
                default: key[i] = i < n / 2 ? i : n - i; break;       // organ pipe
            }
        }
        std::vector<int32_t> a(n), b(n);
        std::iota(a.begin(), a.end(), 0);
        std::iota(b.begin(), b.end(), 0);
        const int32_t* k = key.data();
        auto longer_first = [k](const int32_t& x, const int32_t& y) { return k[x] > k[y]; };
        std::sort(a.begin(), a.end(), longer_first);
        const int threads = 2 + (int)(rng() % 15);
        std::vector<int32_t> gathered(n, -1);
        std::vector<int> visits(n, 0);
        const int32_t* pb = b.data();
        int32_t* pg = gathered.data();
        int* pv = visits.data();
        const std::function<void(int, int)> gather = [=](int t, int T) {
            const int lo = (int)((int64_t)n * t / T), hi = (int)((int64_t)n * (t + 1) / T);
            for (int i = lo; i < hi; i++) {
                pg[i] = k[pb[i]];
                pv[i]++;
            }
        };
        gsdr::std_sort_threaded(b.begin(), b.end(), longer_first, threads,
                                trial % 2 ? gather : std::function<void(int, int)>());
        bool gather_ok = true;
        if (trial % 2)
            for (int i = 0; i < n; i++)
                if (visits[i] != 1 || gathered[i] != key[a[i]]) gather_ok = false;
        if (a != b || !gather_ok) {
            bad++;
            std::printf("mismatch: trial %d n %d mode %d threads %d gather %d\n", trial, n, mode,
                        threads, (int)gather_ok);
        }
    }
    std::printf("mismatches %d of %d\n", bad, trials);
    return bad != 0;
}
