// Per-read layout of a job's packed reads and k-mer lists: read i's words
// start at pack_off[i] and its k-mer entries at kmer_off[i]; each read takes
// round4(L / 16 + 1) words and round4(entries) entries, where entries =
// L - k + 1 clamped to [0, 4^k] (0 in drop mode).
//
// plan_chunk computes a range of reads' offsets as sums within the range;
// plan_shift then adds the sums of the ranges before it.  One range equals
// the serial pass; T ranges let T threads compute the offsets of their own
// parts of the reads (the FASTA path does it in the sort's gather, on the
// threads that wrote those reads' offsets and lengths).
#pragma once

#include <cstdint>
#include <vector>

namespace gsdr {

inline int64_t round4(int64_t v) { return (v + 3) & ~(int64_t)3; }

// k-mer entries of a read of L bases
inline int64_t plan_entries(int64_t L, int k, bool drop) {
    if (drop) return 0;
    const int64_t kcap = (int64_t)1 << (2 * (k > 0 ? k : 1));
    int64_t e = L - k + 1;
    if (e < 0) e = 0;
    return e > kcap ? kcap : e;
}

// What a range of reads adds to the layout.
struct PlanChunk {
    int64_t pack = 0, kmer = 0;  // words and entries of the range
    int64_t ents_sum = 0;        // k-mer entries before rounding
    int64_t ents_max = 0;
    int64_t max_len = 0;
    bool sorted = true;  // lengths non-increasing within the range
    bool valid = true;   // no negative length, every read inside the byte buffer
};

// Reads lo .. hi-1: pack_off[i + 1] and kmer_off[i + 1] = the words and
// entries of reads lo .. i.
inline PlanChunk plan_chunk(const int64_t* offset, const int32_t* length, int64_t n_bytes, int lo,
                            int hi, int k, bool drop, int64_t* pack_off, int64_t* kmer_off) {
    PlanChunk c;
    // (the running sums stay in registers: reading back the entry just
    // stored would chain every iteration on a store-to-load forward)
    int64_t pack = 0, kmer = 0, ents_sum = 0, ents_max = 0, max_len = 0;
    bool sorted = true, valid = true;
    for (int i = lo; i < hi; i++) {
        const int64_t L = length[i];
        valid = valid && L >= 0 && offset[i] >= 0 && offset[i] + L <= n_bytes;
        if (L > max_len) max_len = L;
        if (i > lo && L > length[i - 1]) sorted = false;
        pack += round4(L / 16 + 1);
        pack_off[i + 1] = pack;
        const int64_t e = plan_entries(L, k, drop);
        ents_sum += e;
        if (e > ents_max) ents_max = e;
        kmer += round4(e);
        kmer_off[i + 1] = kmer;
    }
    c.pack = pack;
    c.kmer = kmer;
    c.ents_sum = ents_sum;
    c.ents_max = ents_max;
    c.max_len = max_len;
    c.sorted = sorted;
    c.valid = valid;
    return c;
}

inline void plan_shift(int lo, int hi, int64_t pack_base, int64_t kmer_base, int64_t* pack_off,
                       int64_t* kmer_off) {
    if (pack_base == 0 && kmer_base == 0) return;
    for (int i = lo; i < hi; i++) {
        pack_off[i + 1] += pack_base;
        kmer_off[i + 1] += kmer_base;
    }
}

// Ranges combined in order: the first range's fields, then each next one's.
inline PlanChunk plan_join(const PlanChunk& a, const PlanChunk& b, bool b_follows_a_sorted) {
    PlanChunk c;
    c.pack = a.pack + b.pack;
    c.kmer = a.kmer + b.kmer;
    c.ents_sum = a.ents_sum + b.ents_sum;
    c.ents_max = a.ents_max > b.ents_max ? a.ents_max : b.ents_max;
    c.max_len = a.max_len > b.max_len ? a.max_len : b.max_len;
    c.sorted = a.sorted && b.sorted && b_follows_a_sorted;
    c.valid = a.valid && b.valid;
    return c;
}

// The layout of a job's reads computed by the caller (PlanChunk over all
// reads and the offsets), for Job::init to take instead of its own pass.
// Used only for the word length and drop mode it was computed with.
struct PlanPreset {
    int k = -1;
    bool drop = false;
    PlanChunk sums;
    std::vector<int64_t> pack_off, kmer_off;  // n + 1 entries each
};

}  // namespace gsdr
