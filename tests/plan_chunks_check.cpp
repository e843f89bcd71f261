// The job layout computed in parts by the sort's threads (csrc/plan_chunks.h,
// as the FASTA path runs it in the sort's gather: plan_chunk per part, the
// threads meet, plan_shift by the parts before, plan_join in order) against a
// plain serial restatement of the layout: per read round4(L / 16 + 1) words
// and round4(entries) k-mer entries, entries = L - k + 1 clamped to [0, 4^k]
// (0 in drop mode).  Prints "mismatches M of C".
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <numeric>
#include <random>
#include <thread>
#include <vector>

#include "plan_chunks.h"
#include "stdsort.h"

namespace {

struct Serial {
    std::vector<int64_t> pack_off, kmer_off;
    int64_t ents_sum = 0, ents_max = 0, max_len = 0;
    bool sorted = true, valid = true;
};

Serial serial(const std::vector<int64_t>& off, const std::vector<int32_t>& len, int64_t n_bytes,
              int k, bool drop) {
    const int n = (int)len.size();
    Serial s;
    s.pack_off.assign(n + 1, 0);
    s.kmer_off.assign(n + 1, 0);
    const int64_t kcap = (int64_t)1 << (2 * (k > 0 ? k : 1));
    for (int i = 0; i < n; i++) {
        const int64_t L = len[i];
        if (L < 0 || off[i] < 0 || off[i] + L > n_bytes) s.valid = false;
        if (L > s.max_len) s.max_len = L;
        if (i > 0 && L > len[i - 1]) s.sorted = false;
        s.pack_off[i + 1] = s.pack_off[i] + ((L / 16 + 1 + 3) / 4) * 4;
        int64_t e = drop ? 0 : L - k + 1;
        if (e < 0) e = 0;
        if (e > kcap) e = kcap;
        s.ents_sum += e;
        if (e > s.ents_max) s.ents_max = e;
        s.kmer_off[i + 1] = s.kmer_off[i] + ((e + 3) / 4) * 4;
    }
    return s;
}

// One case: records with lengths `rec_len` at offsets `rec_off`, sorted by
// length (descending) by the team sort, laid out in its gather.
bool run_case(const std::vector<int64_t>& rec_off, const std::vector<int64_t>& rec_len,
              int64_t n_bytes, int k, bool drop, int threads) {
    const int32_t nr = (int32_t)rec_len.size();
    std::vector<int32_t> order(nr);
    std::iota(order.begin(), order.end(), 0);
    std::vector<int64_t> s_off(nr);
    std::vector<int32_t> s_len(nr);
    gsdr::PlanPreset preset;
    preset.pack_off.assign((size_t)nr + 1, -7);
    preset.kmer_off.assign((size_t)nr + 1, -7);
    preset.pack_off[0] = 0;
    preset.kmer_off[0] = 0;
    std::vector<gsdr::PlanChunk> parts((size_t)std::max(threads, 1));
    std::atomic<int> arrived{0};
    int used = 0;
    const int32_t* ord = order.data();
    const int64_t* doff = rec_off.data();
    const int64_t* dlp = rec_len.data();
    int64_t* soff = s_off.data();
    int32_t* slen = s_len.data();
    int64_t* pk = preset.pack_off.data();
    int64_t* km = preset.kmer_off.data();
    gsdr::PlanChunk* pp = parts.data();
    std::atomic<int>* arr = &arrived;
    int* usedp = &used;
    const std::function<void(int, int)> gather = [=](int t, int T) {
        const int32_t lo = (int32_t)((int64_t)nr * t / T), hi = (int32_t)((int64_t)nr * (t + 1) / T);
        for (int32_t i = lo; i < hi; i++) {
            soff[i] = doff[ord[i]];
            slen[i] = (int32_t)dlp[ord[i]];
        }
        pp[t] = gsdr::plan_chunk(soff, slen, n_bytes, lo, hi, k, drop, pk, km);
        arr->fetch_add(1, std::memory_order_acq_rel);
        while (arr->load(std::memory_order_acquire) < T) std::this_thread::yield();
        int64_t pb = 0, kb = 0;
        for (int u = 0; u < t; u++) {
            pb += pp[u].pack;
            kb += pp[u].kmer;
        }
        gsdr::plan_shift(lo, hi, pb, kb, pk, km);
        if (t == 0) *usedp = T;
    };
    gsdr::std_sort_threaded(order.begin(), order.end(),
                            [dlp](const int32_t& a, const int32_t& c) { return dlp[a] > dlp[c]; },
                            threads, gather);
    if (used < 1 || used > (int)parts.size()) return false;
    gsdr::PlanChunk all = parts[0];
    for (int u = 1; u < used; u++) {
        const int32_t lo = (int32_t)((int64_t)nr * u / used);
        const int32_t hi = (int32_t)((int64_t)nr * (u + 1) / used);
        const bool follows = lo >= hi || lo == 0 || slen[lo] <= slen[lo - 1];
        all = gsdr::plan_join(all, parts[u], follows);
    }
    const Serial ref = serial(s_off, s_len, n_bytes, k, drop);
    return preset.pack_off == ref.pack_off && preset.kmer_off == ref.kmer_off &&
           all.pack == ref.pack_off[nr] && all.kmer == ref.kmer_off[nr] &&
           all.ents_sum == ref.ents_sum && all.ents_max == ref.ents_max &&
           all.max_len == ref.max_len && all.sorted == ref.sorted && all.valid == ref.valid;
}

}  // namespace

int main(int argc, char** argv) {
    const int cases = argc > 1 ? std::atoi(argv[1]) : 60;
    std::mt19937_64 rng(20251204);
    const int sizes[] = {0, 1, 2, 3, 17, 1000, 65535, 65536, 70001, 200000};
    const int ks[] = {1, 4, 5, 6, 7, 8, 12};
    int bad = 0, run = 0;
    for (int c = 0; c < cases; c++) {
        const int n = sizes[c % (int)(sizeof(sizes) / sizeof(sizes[0]))];
        const int k = ks[(c / 3) % (int)(sizeof(ks) / sizeof(ks[0]))];
        const bool drop = (c % 7) == 3;
        const int threads = 1 + (int)(rng() % 16);
        std::vector<int64_t> off(n), len(n);
        int64_t pos = 0;
        for (int i = 0; i < n; i++) {
            // lengths: zeros, below k, ties, up to past 4^k + k for small k
            const int kind = (int)(rng() % 8);
            int64_t L = kind == 0 ? 0
                        : kind == 1 ? (int64_t)(rng() % 4)
                        : kind == 2 ? 150
                        : kind == 3 ? 4096 + 12 + (int64_t)(rng() % 100)
                                    : 300 + (int64_t)(rng() % 9700);
            off[i] = pos;
            len[i] = L;
            pos += L + 1 + (int64_t)(rng() % 40);
        }
        int64_t n_bytes = pos + 16;
        // every tenth case: one read reaching past the byte buffer (not valid)
        if (n > 0 && c % 10 == 9) n_bytes = off[n - 1] + len[n - 1] - 1;
        run++;
        if (!run_case(off, len, n_bytes, k, drop, threads)) {
            bad++;
            std::printf("mismatch: n %d k %d drop %d threads %d\n", n, k, (int)drop, threads);
        }
    }
    std::printf("mismatches %d of %d\n", bad, run);
    return bad == 0 ? 0 : 1;
}
