// gsdr_oracle.cpp -- CPU restatement of the reference clustering path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle: the parity tests, the
// smoke check and bench.py's CPU-baseline / reference leg run it as the
// checker.  Nothing in the product (the CUDA library or the `cluster` CLI)
// links, loads or calls it.
//
// It restates, step by step and with the same integer / float / double types,
// the `cuda-version` variant of JuZhenCS/gene-sequences-de-redundancy:
//   options          cuda-version/func.cu:10-92   (checkOption)
//   FASTA read+sort  cuda-version/func.cu:94-117  (readFile)
//   padded layout    cuda-version/func.cu:119-137 (copyData; 64-bit offsets)
//   base codes       cuda-version/func.cu:139-179 (kernel_baseToNumber)
//   pigeon index     cuda-version/func.cu:188-250 (kernel_createPigeon1/2)
//   2-bit packing    cuda-version/func.cu:272-299 (kernel_compressData)
//   cutoffs          cuda-version/func.cu:312-337 (kernel_createCutoff)
//   composition      cuda-version/func.cu:351-394 (kernel_createPrefix)
//   k-mers           cuda-version/func.cu:522-558, 591-644 (createWords/sort/merge)
//   greedy loop      cuda-version/func.cu:655-710, 1001-1097
//   filters          cuda-version/func.cu:712-826 (makeTable/preFilter/pigeon/filter)
//   alignment        cuda-version/func.cu:828-999 (kernel_align: LCS >= cutoff)
//   FASTA write      cuda-version/func.cu:1099-1111 (saveFile)
//
// The alignment of the reference is a full dynamic-programming longest common
// subsequence over the gap-free (ACGT-only) sequences, accepted iff
// LCS >= baseCutoff[query].  Two interchangeable forms are provided: the
// cell-by-cell DP (mode 0) and Hyyro's bit-parallel LCS over 64-bit words
// (mode 1, the default); tests check that they agree.
//
// Behaviour on reads with no A/C/G/T base at all: the reference loops without
// end in createPrefix/createWords (func.cu:362-389, 421-435) when filters are on,
// and kernel_align never returns a decision when such a read is the
// representative (func.cu:863-999).  This oracle gives such reads an empty
// composition and no k-mers (so the word filter rejects them both ways) and
// rejects every candidate of a representative with no A/C/G/T base, which is
// what the reference's drop mode does.
//
// Variant 1 restates the top-level SYCL program of the same repository
// (func.cpp, a different clustering of the same inputs), selected by
// `variant`:
//   options          func.cpp:6-56   (checkOption: k rises with t, w 4..8,
//                                     keys i o t w only; no drop, no pigeon)
//   k-mers           func.cpp:238-326 (createWords/sortWords/mergeWords: every
//                                     window of k raw bytes without a non-ACGT
//                                     byte, u16 words, u16 multiplicities)
//   composition      func.cpp:197-236 (raw codes 0..3: the gap-free counts)
//   cutoffs          func.cpp:339-373 (createCutoff: float arithmetic, the
//                                     offset forced to 1)
//   alignment        func.cpp:572-676 (kernel_dynamic: bit-parallel LCS over
//                                     the gap-free sequences, accept iff
//                                     LCS > baseCutoff, strictly)
//   loop, filters    func.cpp:447-799 (the same round structure and filters)
// Its reader (func.cpp:70-117) gives the same reads as readFile above on a
// file whose every line ends with '\n' (on a last line without one it does
// not terminate), so the same reader serves both.  Parity of variant 1 is
// pinned only by the SYCL program's own output file (the repository's
// top-level result.fasta): no SYCL compiler is available to run it.
//
// Compile with -ffp-contract=off so that the cutoff arithmetic stays exact.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

struct Read {
    std::string name;
    std::string data;
};

struct Options {
    std::string inputFile = "testData.fasta";
    std::string outputFile = "result.fasta";
    float threshold = 0.95f;
    int wordLength = 0;
    int drop = 3;
    int pigeon = 0;
    int variant = 0;  // 0 cuda-version, 1 the SYCL program (func.cpp)
};

// checkOption (cuda-version/func.cu:10-92).  Returns 0 on success and 1 where
// the reference prints its usage text and exits.  Only the first character of
// a key is looked at (func.cu:19).  Comparisons of the float threshold with
// decimal literals happen in double, as in C++.
int check_option(int argc, char** argv, Options& o) {
    if (argc % 2 != 1) return 1;
    o = Options();
    for (int i = 1; i < argc; i += 2) {
        try {
            switch (argv[i][0]) {
                case 'i': o.inputFile = argv[i + 1]; break;
                case 'o': o.outputFile = argv[i + 1]; break;
                case 't': o.threshold = std::stof(argv[i + 1]); break;
                case 'w': o.wordLength = std::stoi(argv[i + 1]); break;
                case 'd': o.drop = std::stoi(argv[i + 1]); break;
                case 'p': o.pigeon = std::stoi(argv[i + 1]); break;
                default: return 1;
            }
        } catch (...) {
            return 1;
        }
    }
    if (o.threshold < 0.8 || o.threshold >= 1) return 1;
    if (o.wordLength == 0) {
        if (o.threshold < 0.88) o.wordLength = 4;
        else if (o.threshold < 0.94) o.wordLength = 7;
        else if (o.threshold < 0.97) o.wordLength = 6;
        else o.wordLength = 5;
    } else if (o.wordLength < 4 || o.wordLength > 12) {
        return 1;
    }
    if (o.drop == 3) {
        o.drop = (o.threshold <= 0.879) ? 1 : 0;
    } else if (o.drop != 0 && o.drop != 1) {
        return 1;
    }
    if (o.pigeon != 1 && o.pigeon != 0) return 1;
    return 0;
}

// checkOption of the SYCL program (func.cpp:6-56): keys i o t w only.
int check_option_sycl(int argc, char** argv, Options& o) {
    if (argc % 2 != 1) return 1;
    o = Options();
    o.variant = 1;
    for (int i = 1; i < argc; i += 2) {
        try {
            switch (argv[i][0]) {
                case 'i': o.inputFile = argv[i + 1]; break;
                case 'o': o.outputFile = argv[i + 1]; break;
                case 't': o.threshold = std::stof(argv[i + 1]); break;
                case 'w': o.wordLength = std::stoi(argv[i + 1]); break;
                default: return 1;
            }
        } catch (...) {
            return 1;
        }
    }
    if (o.threshold < 0.8 || o.threshold >= 1) return 1;
    if (o.wordLength == 0) {
        if (o.threshold < 0.88) o.wordLength = 4;
        else if (o.threshold < 0.94) o.wordLength = 5;
        else if (o.threshold < 0.97) o.wordLength = 6;
        else o.wordLength = 7;
    } else if (o.wordLength < 4 || o.wordLength > 8) {
        return 1;
    }
    o.drop = 0;
    o.pigeon = 0;
    return 0;
}

int g_keep_order = 0;

// readFile (cuda-version/func.cu:94-117): the first line is a name whatever
// it holds; a line starting with '>' starts the next record; every other line
// is appended verbatim (including any '\r').  Then std::sort, longest first.
void read_file(const std::string& path, std::vector<Read>& reads) {
    std::ifstream file(path);
    Read read;
    std::string line;
    std::getline(file, line);
    read.name = line;
    while (std::getline(file, line)) {
        if (line[0] == '>') {
            reads.push_back(read);
            read.name = line;
            read.data = "";
            continue;
        }
        read.data += line;
    }
    reads.push_back(read);
    if (g_keep_order) {
        // test hook: a file already in length order keeps its tie order
        std::stable_sort(reads.begin(), reads.end(),
                         [](const Read& a, const Read& b) { return a.data.size() > b.data.size(); });
        return;
    }
    std::sort(reads.begin(), reads.end(),
              [](Read& a, Read& b) { return a.data.size() > b.data.size(); });
}

// kernel_baseToNumber (cuda-version/func.cu:139-179)
inline int base_code(unsigned char c) {
    switch (c) {
        case 'A': case 'a': return 0;
        case 'C': case 'c': return 1;
        case 'G': case 'g': return 2;
        case 'T': case 't': case 'U': case 'u': return 3;
        default: return 4;
    }
}

// Per-read derived data, as the reference keeps it in `Data` (func.h:21-41).
struct Prep {
    int n = 0;
    int k = 0;
    std::vector<int> lengths;                  // raw length
    std::vector<long long> offsets;            // padded byte offsets (copyData)
    std::vector<int> gaps;                     // non-ACGT count
    std::vector<std::vector<uint8_t>> gf;      // gap-free codes 0..3
    std::vector<std::vector<uint32_t>> packed; // kernel_compressData words
    std::vector<int> prefix;                   // 4 per read
    std::vector<int> wordCutoff, baseCutoff, pigeonCutoff;
    std::vector<int> wordCounts;               // gap-free length - k + 1
    std::vector<std::vector<uint32_t>> kmer;   // distinct k-mers, sorted
    std::vector<std::vector<uint16_t>> kcnt;   // their multiplicities (u16)
    std::vector<std::vector<uint16_t>> pig;    // 256 inclusive prefix counts
    std::vector<std::vector<uint16_t>> pigIdx; // positions, counting-sorted
};

// kernel_compressData (cuda-version/func.cu:272-299): drop codes >= 4 and pack
// 16 bases per uint32, first base in the two most significant bits.  Always
// ends with a (possibly empty) partial word: gf/16 + 1 words.
void pack(const std::vector<uint8_t>& gf, std::vector<uint32_t>& out) {
    out.assign(gf.size() / 16 + 1, 0u);
    for (size_t i = 0; i < gf.size(); i++)
        out[i / 16] += (uint32_t)gf[i] << ((15 - (i % 16)) * 2);
}

// kernel_createCutoff (cuda-version/func.cu:312-337), same types.
void cutoffs(int length, float threshold, int wordLength, int& word, int& base, int& pigeon) {
    int required = length - wordLength + 1;
    int cutoff = (int)(std::ceil((double)(float)length * (1.0 - (double)threshold)) * wordLength);
    required -= cutoff;
    required = std::max(required, 1);
    float offset = 0;
    if ((double)threshold >= 0.9) {
        offset = (float)(1.1 - std::fabs((double)threshold - 0.95) * 2);
    } else {
        offset = 1;
    }
    required = (int)std::ceil((float)((float)required * offset));
    word = required;
    base = (int)std::ceil((float)((float)length * threshold));
    pigeon = (int)(std::ceil((double)(float)length * (1.0 - (double)threshold)) * 4);
}

// createCutoff of the SYCL program (func.cpp:339-373): float throughout and
// the offset factor overwritten with 1.
void cutoffs_sycl(int length, float threshold, int wordLength, int& word, int& base) {
    int required = length - wordLength + 1;
    float slack = std::ceil((float)((float)length * (float)(1.0f - threshold)));
    int cutoff = (int)(float)(slack * (float)wordLength);
    required -= cutoff;
    required = std::max(required, 1);
    required = (int)std::ceil((float)((float)required * 1.0f));
    word = required;
    base = (int)std::ceil((float)((float)length * threshold));
}

// createWords / sortWords / mergeWords of the SYCL program
// (func.cpp:238-326): the window of k raw codes ending at each position,
// skipped when it holds a code 4 (non-ACGT byte); the word puts the window's
// last base in the low bits.  Sorted multiset with u16 multiplicities.
void kmers_raw(const std::vector<uint8_t>& codes, int k, std::vector<uint32_t>& w,
               std::vector<uint16_t>& c) {
    w.clear();
    c.clear();
    std::vector<uint32_t> all;
    for (int i = k - 1; i < (int)codes.size(); i++) {
        uint32_t word = 0;
        bool skip = false;
        for (int j = 0; j < k; j++) {
            uint8_t b = codes[i - j];
            if (b == 4) skip = true;
            word += (uint32_t)(b & 3) << (2 * j);
        }
        if (!skip) all.push_back(word & 0xffffu);
    }
    std::sort(all.begin(), all.end());
    for (size_t i = 0; i < all.size();) {
        size_t j = i;
        while (j < all.size() && all[j] == all[i]) j++;
        w.push_back(all[i]);
        c.push_back((uint16_t)(j - i));
        i = j;
    }
}

// kernel_createWords / sortWords / mergeWords (cuda-version/func.cu:522-644):
// every k-mer of the gap-free sequence (first base most significant), as a
// sorted multiset; multiplicities are unsigned short (they wrap at 65536).
void kmers(const std::vector<uint8_t>& gf, int k, std::vector<uint32_t>& w,
           std::vector<uint16_t>& c) {
    w.clear();
    c.clear();
    int n = (int)gf.size() - k + 1;
    if (n <= 0) return;
    uint32_t mask = (k >= 16) ? 0xffffffffu : ((1u << (2 * k)) - 1u);
    std::vector<uint32_t> all;
    all.reserve(n);
    uint32_t word = 0;
    for (size_t i = 0; i < gf.size(); i++) {
        word = ((word << 2) + gf[i]) & mask;
        if ((int)i >= k - 1) all.push_back(word);
    }
    std::sort(all.begin(), all.end());
    for (size_t i = 0; i < all.size();) {
        size_t j = i;
        while (j < all.size() && all[j] == all[i]) j++;
        w.push_back(all[i]);
        c.push_back((uint16_t)(j - i));
        i = j;
    }
}

// kernel_createPigeon1 / kernel_createPigeon2 (cuda-version/func.cu:188-250).
// Runs over the raw codes (before gap removal).  A 4-mer window that holds a
// non-ACGT code is skipped.  pig = inclusive prefix of the 256-bucket
// histogram (u16).  pigIdx[slot] = (u16) absolute padded offset of the window's
// last base; within a bucket the slots are filled from the top down, so
// ascending slots hold descending positions.
void pigeon_index(const std::vector<uint8_t>& codes, long long offset,
                  std::vector<uint16_t>& pig, std::vector<uint16_t>& idx) {
    pig.assign(256, 0);
    idx.assign(codes.size() + 1, 0);
    auto scan = [&](bool fill) {
        int b[4] = {4, 4, 4, 4};
        for (size_t p = 0; p < codes.size(); p++) {
            b[0] = b[1]; b[1] = b[2]; b[2] = b[3]; b[3] = codes[p];
            unsigned short v = 0;
            int flag = 0;
            for (int j = 0; j < 4; j++) {
                v = (unsigned short)(v + ((b[j] & 3) << (3 - j) * 2));
                flag += std::max(b[j] - 3, 0);
            }
            if (flag) continue;
            if (!fill) {
                pig[v] = (uint16_t)(pig[v] + 1);
            } else {
                pig[v] = (uint16_t)(pig[v] - 1);
                int slot = pig[v];
                int absolute = (int)(offset + (long long)p);
                if ((size_t)slot < idx.size()) idx[slot] = (uint16_t)absolute;
            }
        }
    };
    auto prefix = [&]() {
        for (int i = 1; i < 256; i++) pig[i] = (uint16_t)(pig[i] + pig[i - 1]);
    };
    scan(false);
    prefix();
    scan(true);
    std::fill(pig.begin(), pig.end(), 0);
    scan(false);
    prefix();
}

void prepare(const std::vector<Read>& reads, const Options& opt, Prep& P, bool want_pigeon) {
    int n = (int)reads.size();
    P.n = n;
    P.k = opt.wordLength;
    P.lengths.resize(n);
    P.offsets.assign(n + 1, 0);
    P.gaps.resize(n);
    P.gf.resize(n);
    P.packed.resize(n);
    P.prefix.assign(4 * (size_t)n, 0);
    P.wordCutoff.resize(n);
    P.baseCutoff.resize(n);
    P.pigeonCutoff.resize(n);
    P.wordCounts.resize(n);
    P.kmer.resize(n);
    P.kcnt.resize(n);
    if (want_pigeon) {
        P.pig.resize(n);
        P.pigIdx.resize(n);
    }
    for (int i = 0; i < n; i++) {
        int L = (int)reads[i].data.size();
        P.lengths[i] = L;
        P.offsets[i + 1] = P.offsets[i] + L / 16 * 16 + 16;
    }
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < n; i++) {
        const std::string& s = reads[i].data;
        std::vector<uint8_t> codes(s.size());
        std::vector<uint8_t>& gf = P.gf[i];
        gf.clear();
        gf.reserve(s.size());
        for (size_t p = 0; p < s.size(); p++) {
            codes[p] = (uint8_t)base_code((unsigned char)s[p]);
            if (codes[p] < 4) gf.push_back(codes[p]);
        }
        P.gaps[i] = (int)(s.size() - gf.size());
        pack(gf, P.packed[i]);
        for (uint8_t b : gf) P.prefix[4 * (size_t)i + b]++;
        if (opt.variant == 1) {
            cutoffs_sycl(P.lengths[i], opt.threshold, opt.wordLength, P.wordCutoff[i],
                         P.baseCutoff[i]);
            P.pigeonCutoff[i] = 0;
            kmers_raw(codes, opt.wordLength, P.kmer[i], P.kcnt[i]);
            continue;
        }
        cutoffs(P.lengths[i], opt.threshold, opt.wordLength, P.wordCutoff[i], P.baseCutoff[i],
                P.pigeonCutoff[i]);
        P.wordCounts[i] = (int)gf.size() - opt.wordLength + 1;
        if (opt.drop == 0) kmers(gf, opt.wordLength, P.kmer[i], P.kcnt[i]);
        if (want_pigeon) pigeon_index(codes, P.offsets[i], P.pig[i], P.pigIdx[i]);
    }
}

// Cell-by-cell LCS, the recurrence kernel_align evaluates
// (cuda-version/func.cu:863-999): C[m][t] = max(C[m-1][t-1] + [q==T], C[m-1][t], C[m][t-1]).
int lcs_dp(const uint8_t* a, int na, const uint8_t* b, int nb) {
    std::vector<int> prev(nb + 1, 0), cur(nb + 1, 0);
    for (int i = 1; i <= na; i++) {
        cur[0] = 0;
        for (int j = 1; j <= nb; j++) {
            int v = prev[j - 1] + (a[i - 1] == b[j - 1]);
            v = std::max(v, prev[j]);
            v = std::max(v, cur[j - 1]);
            cur[j] = v;
        }
        std::swap(prev, cur);
    }
    return prev[nb];
}

// Bit-parallel LCS (Hyyro 2004): V' = (V + (V & M[c])) | (V & ~M[c]);
// LCS = number of zero bits of V over the pattern.
int lcs_bits(const uint8_t* a, int na, const uint8_t* b, int nb) {
    if (na == 0 || nb == 0) return 0;
    int W = (na + 63) / 64;
    std::vector<uint64_t> M(4 * (size_t)W, 0), V(W, ~0ull);
    for (int i = 0; i < na; i++) M[(size_t)a[i] * W + i / 64] |= 1ull << (i % 64);
    for (int j = 0; j < nb; j++) {
        const uint64_t* m = &M[(size_t)b[j] * W];
        uint64_t carry = 0;
        for (int w = 0; w < W; w++) {
            uint64_t v = V[w], u = v & m[w];
            uint64_t s = v + u;
            uint64_t c1 = s < v;
            uint64_t s2 = s + carry;
            uint64_t c2 = s2 < s;
            carry = c1 | c2;
            V[w] = s2 | (v & ~m[w]);
        }
    }
    int zeros = 0;
    for (int w = 0; w < W; w++) {
        uint64_t v = V[w];
        if (w == W - 1 && (na % 64)) v |= ~0ull << (na % 64);
        zeros += 64 - __builtin_popcountll(v);
    }
    return zeros;
}

int g_lcs_mode = 1;

inline int lcs(const std::vector<uint8_t>& a, const std::vector<uint8_t>& b) {
    return g_lcs_mode == 0 ? lcs_dp(a.data(), (int)a.size(), b.data(), (int)b.size())
                           : lcs_bits(a.data(), (int)a.size(), b.data(), (int)b.size());
}

// kernel_preFilter (cuda-version/func.cu:738-754): keep iff the base-composition
// bound reaches the query's base cutoff.
inline bool prefilter(const Prep& P, int r, int q) {
    int sum = 0;
    for (int b = 0; b < 4; b++)
        sum += std::min(P.prefix[4 * (size_t)r + b], P.prefix[4 * (size_t)q + b]);
    return !(sum < P.baseCutoff[q]);
}

// kernel_pigeon (cuda-version/func.cu:756-801).
inline bool pigeon_filter(const Prep& P, float threshold, int r, int q) {
    int lengthOne = P.lengths[r], lengthTwo = P.lengths[q];
    int gap = (int)((float)lengthOne - std::ceil((float)((float)lengthTwo * threshold)));
    int sum = 0;
    const std::vector<uint16_t>& pr = P.pig[r];
    const std::vector<uint16_t>& pq = P.pig[q];
    const std::vector<uint16_t>& ir = P.pigIdx[r];
    const std::vector<uint16_t>& iq = P.pigIdx[q];
    for (int t = 0; t < 256; t++) {
        int s1 = t > 0 ? pr[t - 1] : 0, e1 = pr[t];
        int s2 = t > 0 ? pq[t - 1] : 0, e2 = pq[t];
        while (s1 < e1 && s2 < e2) {
            int one = ir[s1], two = iq[s2];
            if (std::abs(one - two) >= gap) {
                s1++;
                s2++;
                sum++;
            } else if (one > two) {
                s1++;
            } else {
                s2++;
            }
        }
    }
    return !(sum < P.pigeonCutoff[q]);
}

// kernel_makeTable + kernel_filter (cuda-version/func.cu:712-723, 803-826):
// sum over distinct words of min(count in representative, count in query).
inline bool word_filter(const Prep& P, const std::vector<uint16_t>& table, int q) {
    int sum = 0;
    const std::vector<uint32_t>& w = P.kmer[q];
    const std::vector<uint16_t>& c = P.kcnt[q];
    for (size_t i = 0; i < w.size(); i++) sum += std::min(table[w[i]], c[i]);
    return !(sum < P.wordCutoff[q]);
}

// kernel_align decision (cuda-version/func.cu:885-886 and its twins); for the
// SYCL program kernel_dynamic's strict test (func.cpp:671).
int g_variant = 0;
inline bool align_accept(const Prep& P, int r, int q) {
    if (P.gf[r].empty()) return false;  // the reference never decides (see header)
    if (g_variant == 1) return lcs(P.gf[r], P.gf[q]) > P.baseCutoff[q];
    return lcs(P.gf[r], P.gf[q]) >= P.baseCutoff[q];
}

struct Stats {
    long long rounds = 0;
    long long prefilter_in = 0, prefilter_pass = 0;
    long long pigeon_pass = 0, word_pass = 0;
    long long aligned = 0, accepted = 0;
    long long cells = 0;  // sum over aligned pairs of q_gf * T_gf
};

// clustering / clusteringDrop (cuda-version/func.cu:1001-1097).  The round's
// candidates are the still-unclustered reads after the representative.
void clustering(const Options& opt, const Prep& P, std::vector<int>& cluster, Stats& st,
                int max_rounds) {
    int n = P.n;
    cluster.assign(n, -1);
    std::vector<int> remain(n);
    for (int i = 0; i < n; i++) remain[i] = i;
    size_t tsize = (opt.drop == 0) ? ((size_t)1 << (2 * opt.wordLength)) : 1;
    std::vector<uint16_t> table(tsize, 0);
    int rep = -1;
    while (true) {
        rep += 1;
        while (rep < n && cluster[rep] != -1) rep++;
        if (rep >= n) break;
        if (max_rounds >= 0 && st.rounds >= max_rounds) break;
        cluster[rep] = rep;
        st.rounds++;
        // updataRemain (func.cu:689-699)
        size_t cnt = 0;
        for (size_t i = 0; i < remain.size(); i++)
            if (cluster[remain[i]] == -1) remain[cnt++] = remain[i];
        remain.resize(cnt);
        if (opt.drop == 0)
            for (size_t i = 0; i < P.kmer[rep].size(); i++)
                if (P.kcnt[rep][i] > 0) table[P.kmer[rep][i]] = P.kcnt[rep][i];
        long long pf = 0, pg = 0, wp = 0, al = 0, ac = 0, cells = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : pf, pg, wp, al, ac, cells)
        for (long long i = 0; i < (long long)remain.size(); i++) {
            int q = remain[i];
            if (opt.drop == 0) {
                if (!prefilter(P, rep, q)) continue;
                pf++;
                if (opt.pigeon == 1) {
                    if (!pigeon_filter(P, opt.threshold, rep, q)) continue;
                    pg++;
                }
                if (!word_filter(P, table, q)) continue;
                wp++;
            }
            al++;
            cells += (long long)P.gf[rep].size() * (long long)P.gf[q].size();
            if (align_accept(P, rep, q)) {
                cluster[q] = rep;
                ac++;
            }
        }
        st.prefilter_in += (long long)remain.size();
        st.prefilter_pass += pf;
        st.pigeon_pass += pg;
        st.word_pass += wp;
        st.aligned += al;
        st.accepted += ac;
        st.cells += cells;
        if (opt.drop == 0)
            for (size_t i = 0; i < P.kmer[rep].size(); i++) table[P.kmer[rep][i]] = 0;
    }
}

// saveFile (cuda-version/func.cu:1099-1111): representatives in sorted order.
int save_file(const std::string& path, const std::vector<Read>& reads,
              const std::vector<int>& cluster) {
    std::ofstream file(path, std::ios::binary);
    int sum = 0;
    for (size_t i = 0; i < reads.size(); i++) {
        if (cluster[i] == (int)i) {
            file << reads[i].name << '\n';
            file << reads[i].data << '\n';
            sum++;
        }
    }
    return sum;
}

}  // namespace orc

// ---------------------------------------------------------------------------
// C interface for the tests (ctypes) and for bench.py's CPU legs.
// ---------------------------------------------------------------------------
extern "C" {

typedef struct {
    long long rounds, prefilter_in, prefilter_pass, pigeon_pass, word_pass, aligned, accepted,
        cells;
    double seconds;
    int k, drop, pigeon;
    float threshold;
} orc_stats;

// Parses argv like the reference CLI.  Returns 0, or 1 for the usage exit.
int orc_check_option(int argc, char** argv, float* t, int* k, int* drop, int* pigeon) {
    orc::Options o;
    int rc = orc::check_option(argc, argv, o);
    if (rc) return rc;
    *t = o.threshold;
    *k = o.wordLength;
    *drop = o.drop;
    *pigeon = o.pigeon;
    return 0;
}

void orc_cutoffs(const int* len, int n, float t, int k, int* word, int* base, int* pigeon) {
    for (int i = 0; i < n; i++) orc::cutoffs(len[i], t, k, word[i], base[i], pigeon[i]);
}

// LCS of two gap-free code sequences (values 0..3); -1 for any other value.
int orc_lcs(const uint8_t* a, int na, const uint8_t* b, int nb, int mode) {
    for (int i = 0; i < na; i++)
        if (a[i] > 3) return -1;
    for (int i = 0; i < nb; i++)
        if (b[i] > 3) return -1;
    return mode == 0 ? orc::lcs_dp(a, na, b, nb) : orc::lcs_bits(a, na, b, nb);
}

// Gap-free packing of one raw sequence; returns the number of words written
// (gf/16 + 1) and stores the gap count.
int orc_pack(const char* seq, int len, uint32_t* out, int* gaps) {
    std::vector<uint8_t> gf;
    for (int i = 0; i < len; i++) {
        int c = orc::base_code((unsigned char)seq[i]);
        if (c < 4) gf.push_back((uint8_t)c);
    }
    std::vector<uint32_t> w;
    orc::pack(gf, w);
    std::memcpy(out, w.data(), w.size() * 4);
    *gaps = len - (int)gf.size();
    return (int)w.size();
}

// Distinct k-mers of a gap-free code sequence (sorted) with u16 counts.
int orc_kmers(const uint8_t* gf, int n, int k, uint32_t* words, uint16_t* counts) {
    std::vector<uint8_t> v(gf, gf + n);
    std::vector<uint32_t> w;
    std::vector<uint16_t> c;
    orc::kmers(v, k, w, c);
    std::copy(w.begin(), w.end(), words);
    std::copy(c.begin(), c.end(), counts);
    return (int)w.size();
}

// Pigeon index of one raw sequence placed at padded offset `offset`.
void orc_pigeon_index(const char* seq, int len, long long offset, uint16_t* pig256,
                      uint16_t* idx) {
    std::vector<uint8_t> codes(len);
    for (int i = 0; i < len; i++) codes[i] = (uint8_t)orc::base_code((unsigned char)seq[i]);
    std::vector<uint16_t> p, x;
    orc::pigeon_index(codes, offset, p, x);
    std::copy(p.begin(), p.end(), pig256);
    std::copy(x.begin(), x.begin() + len, idx);
}

// The whole program on a FASTA file.  order_out[i] (optional) = index in file
// order of the i-th read after the sort; cluster_out[i] (optional) = cluster of
// sorted read i.  Returns the read count, or -1 for a usage error.
// max_rounds < 0 runs to the end; otherwise stops after that many
// representatives (for timing a bounded sample).
// variant 1: the SYCL program's semantics (d must be 0 or 3, p 0).
long long orc_run_v(const char* in, const char* out, float t, int w, int d, int p, int lcs_mode,
                    int threads, int max_rounds, int* order_out, int* cluster_out,
                    orc_stats* st_out, int variant) {
    orc::Options o;
    o.inputFile = in;
    o.outputFile = out ? out : "";
    o.threshold = t;
    o.wordLength = w;
    o.drop = d;
    o.pigeon = p;
    o.variant = variant;
    // Reuse check_option's derivations with the same rules.
    if (o.threshold < 0.8 || o.threshold >= 1) return -1;
    if (variant == 1) {
        if (o.wordLength == 0) {
            if (o.threshold < 0.88) o.wordLength = 4;
            else if (o.threshold < 0.94) o.wordLength = 5;
            else if (o.threshold < 0.97) o.wordLength = 6;
            else o.wordLength = 7;
        } else if (o.wordLength < 4 || o.wordLength > 8) {
            return -1;
        }
        if ((o.drop != 0 && o.drop != 3) || o.pigeon != 0) return -1;
        o.drop = 0;
    } else if (variant == 0) {
        if (o.wordLength == 0) {
            if (o.threshold < 0.88) o.wordLength = 4;
            else if (o.threshold < 0.94) o.wordLength = 7;
            else if (o.threshold < 0.97) o.wordLength = 6;
            else o.wordLength = 5;
        } else if (o.wordLength < 4 || o.wordLength > 12) {
            return -1;
        }
        if (o.drop == 3) o.drop = (o.threshold <= 0.879) ? 1 : 0;
        else if (o.drop != 0 && o.drop != 1) return -1;
        if (o.pigeon != 0 && o.pigeon != 1) return -1;
    } else {
        return -1;
    }
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
    orc::g_lcs_mode = lcs_mode;
    orc::g_variant = variant;
    std::vector<orc::Read> reads;
    {
        // Keep the file-order index beside each read through the sort: the
        // comparator looks at the length only, so the permutation is the one
        // the reference's std::sort produces.
        std::vector<orc::Read> raw;
        orc::read_file(o.inputFile, raw);
        reads.swap(raw);
    }
    if (order_out) {
        // Recover the permutation by re-sorting indices with the same comparator.
        std::vector<orc::Read> file_order;
        {
            std::ifstream file(o.inputFile);
            orc::Read read;
            std::string line;
            std::getline(file, line);
            read.name = line;
            while (std::getline(file, line)) {
                if (line[0] == '>') {
                    file_order.push_back(read);
                    read.name = line;
                    read.data = "";
                    continue;
                }
                read.data += line;
            }
            file_order.push_back(read);
        }
        struct Tagged {
            orc::Read r;
            int idx;
        };
        std::vector<Tagged> tg(file_order.size());
        for (size_t i = 0; i < file_order.size(); i++) tg[i] = {file_order[i], (int)i};
        auto longer = [](const Tagged& a, const Tagged& b) {
            return a.r.data.size() > b.r.data.size();
        };
        if (orc::g_keep_order) std::stable_sort(tg.begin(), tg.end(), longer);
        else std::sort(tg.begin(), tg.end(), longer);
        for (size_t i = 0; i < tg.size(); i++) order_out[i] = tg[i].idx;
    }
    double t0 = 0;
#ifdef _OPENMP
    t0 = omp_get_wtime();
#endif
    orc::Prep P;
    orc::prepare(reads, o, P, o.pigeon == 1 && o.drop == 0);
    std::vector<int> cluster;
    orc::Stats st;
    orc::clustering(o, P, cluster, st, max_rounds);
    double t1 = t0;
#ifdef _OPENMP
    t1 = omp_get_wtime();
#endif
    if (out && out[0]) orc::save_file(o.outputFile, reads, cluster);
    if (cluster_out) std::copy(cluster.begin(), cluster.end(), cluster_out);
    if (st_out) {
        st_out->rounds = st.rounds;
        st_out->prefilter_in = st.prefilter_in;
        st_out->prefilter_pass = st.prefilter_pass;
        st_out->pigeon_pass = st.pigeon_pass;
        st_out->word_pass = st.word_pass;
        st_out->aligned = st.aligned;
        st_out->accepted = st.accepted;
        st_out->cells = st.cells;
        st_out->seconds = t1 - t0;
        st_out->k = o.wordLength;
        st_out->drop = o.drop;
        st_out->pigeon = o.pigeon;
        st_out->threshold = o.threshold;
    }
    return (long long)reads.size();
}

long long orc_run(const char* in, const char* out, float t, int w, int d, int p, int lcs_mode,
                  int threads, int max_rounds, int* order_out, int* cluster_out,
                  orc_stats* st_out) {
    return orc_run_v(in, out, t, w, d, p, lcs_mode, threads, max_rounds, order_out, cluster_out,
                     st_out, 0);
}

// Test hook: 1 = read_file keeps the file's order of equal-length reads
// (std::stable_sort) instead of the reference's std::sort order.
void orc_set_keep_order(int keep) { orc::g_keep_order = keep; }

// checkOption of the SYCL program.  Returns 0, or 1 for its usage exit.
int orc_check_option_sycl(int argc, char** argv, float* t, int* k) {
    orc::Options o;
    int rc = orc::check_option_sycl(argc, argv, o);
    if (rc) return rc;
    *t = o.threshold;
    *k = o.wordLength;
    return 0;
}

void orc_cutoffs_sycl(const int* len, int n, float t, int k, int* word, int* base) {
    for (int i = 0; i < n; i++) orc::cutoffs_sycl(len[i], t, k, word[i], base[i]);
}

// The SYCL program's k-mers of one raw sequence (sorted) with u16 counts.
int orc_kmers_raw(const char* seq, int len, int k, uint32_t* words, uint16_t* counts) {
    std::vector<uint8_t> codes(len);
    for (int i = 0; i < len; i++) codes[i] = (uint8_t)orc::base_code((unsigned char)seq[i]);
    std::vector<uint32_t> w;
    std::vector<uint16_t> c;
    orc::kmers_raw(codes, k, w, c);
    std::copy(w.begin(), w.end(), words);
    std::copy(c.begin(), c.end(), counts);
    return (int)w.size();
}

// Pairwise decision on two raw sequences with the parameters of threshold t:
// bit 0 prefilter pass, bit 1 word-filter pass, bit 2 LCS >= cutoff.
// `rep` plays the representative.  Used by the known-answer test.
int orc_pair(const char* rep, int lr, const char* q, int lq, float t, int k) {
    std::vector<orc::Read> reads(2);
    reads[0].data.assign(rep, lr);
    reads[1].data.assign(q, lq);
    orc::Options o;
    o.threshold = t;
    o.wordLength = k;
    o.drop = 0;
    orc::g_variant = 0;
    orc::Prep P;
    orc::prepare(reads, o, P, false);
    std::vector<uint16_t> table((size_t)1 << (2 * k), 0);
    for (size_t i = 0; i < P.kmer[0].size(); i++) table[P.kmer[0][i]] = P.kcnt[0][i];
    int r = 0;
    if (orc::prefilter(P, 0, 1)) r |= 1;
    if (orc::word_filter(P, table, 1)) r |= 2;
    if (orc::align_accept(P, 0, 1)) r |= 4;
    return r;
}

}  // extern "C"

#ifdef ORC_MAIN
// Command-line form with the reference's argument rules (cuda-version/main.cu).
int main(int argc, char** argv) {
    orc::Options o;
    if (orc::check_option(argc, argv, o)) {
        std::cout << "Please check parameters." << std::endl;
        std::cout << "a.out i inputFile t threshold" << std::endl;
        return 0;
    }
    orc_stats st;
    long long n = orc_run(o.inputFile.c_str(), o.outputFile.c_str(), o.threshold, o.wordLength,
                          o.drop, o.pigeon, 1, 0, -1, nullptr, nullptr, &st);
    std::cout << "reads count:\t" << n << "\nrounds:\t" << st.rounds << "\nseconds:\t"
              << st.seconds << std::endl;
    return 0;
}
#endif
