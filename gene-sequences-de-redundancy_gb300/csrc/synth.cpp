// synth.cpp -- seeded synthetic FASTA workloads (seed sequences plus mutated
// copies, shuffled), used by the tests and the benchmark.  The output is the
// same byte for byte on x86-64 and AArch64: the random generator is integer
// (xoshiro256**), the only floating-point functions are written here with
// + - * / and sqrt (all correctly rounded), and the file is compiled with
// -ffp-contract=off.
#include "gsdr_synth.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

inline uint64_t splitmix64(uint64_t& x) {
    uint64_t z = (x += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

struct Rng {
    uint64_t s[4];
    explicit Rng(uint64_t seed) {
        uint64_t x = seed;
        for (int i = 0; i < 4; i++) s[i] = splitmix64(x);
    }
    static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {
        uint64_t r = rotl(s[1] * 5, 7) * 9;
        uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    // uniform double in [0, 1) with 53 random bits
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    // uniform integer in [lo, hi]
    int64_t range(int64_t lo, int64_t hi) {
        uint64_t span = (uint64_t)(hi - lo) + 1;
        return lo + (int64_t)(next() % span);
    }
};

const double kLn2 = 0.6931471805599453094;
const double kPi = 3.14159265358979323846;

// log(x) for x > 0: x = m 2^e with m in [sqrt(1/2), sqrt(2)), then
// log(m) = 2 atanh((m-1)/(m+1)) by its series.
double det_log(double x) {
    int e = 0;
    double m = std::frexp(x, &e);  // m in [0.5, 1)
    if (m < 0.70710678118654752) {
        m *= 2.0;
        e -= 1;
    }
    double s = (m - 1.0) / (m + 1.0);
    double s2 = s * s;
    double term = s, sum = 0.0;
    for (int k = 1; k < 40; k += 2) {
        sum += term / (double)k;
        term *= s2;
    }
    return 2.0 * sum + (double)e * kLn2;
}

// exp(x): x = n ln2 + r with |r| <= ln2/2, Taylor series of exp(r).
double det_exp(double x) {
    double n = std::floor(x / kLn2 + 0.5);
    double r = x - n * kLn2;
    double term = 1.0, sum = 1.0;
    for (int k = 1; k < 30; k++) {
        term = term * r / (double)k;
        sum += term;
    }
    return std::ldexp(sum, (int)n);
}

// cos(x) for x in [0, 2 pi): shift to [-pi, pi], Taylor series.
double det_cos(double x) {
    if (x > kPi) x -= 2.0 * kPi;
    double x2 = x * x, term = 1.0, sum = 1.0;
    for (int k = 2; k < 60; k += 2) {
        term = -term * x2 / (double)((k - 1) * k);
        sum += term;
    }
    return sum;
}

double normal(Rng& r) {
    double u1 = r.uniform();
    if (u1 < 1e-300) u1 = 1e-300;
    double u2 = r.uniform();
    return std::sqrt(-2.0 * det_log(u1)) * det_cos(2.0 * kPi * u2);
}

int draw_length(const gsdr_synth_cfg& c, Rng& r) {
    double L = 0;
    switch (c.len_dist) {
        case GSDR_LEN_UNIFORM: L = (double)r.range((int64_t)c.len_lo, (int64_t)c.len_hi); break;
        case GSDR_LEN_LOGNORMAL:
            L = c.len_median * det_exp(c.len_sigma * normal(r));
            break;
        case GSDR_LEN_FIXED: L = c.len_lo; break;
        case GSDR_LEN_LOGUNIFORM: {
            double a = det_log(c.len_lo), b = det_log(c.len_hi);
            L = det_exp(a + (b - a) * r.uniform());
            break;
        }
        default: L = c.len_lo;
    }
    L = std::floor(L + 0.5);
    if (L < c.len_lo) L = c.len_lo;
    if (L > c.len_hi) L = c.len_hi;
    return (int)L;
}

inline char draw_base(Rng& r, double gc) {
    double u = r.uniform();
    if (u < gc * 0.5) return 'G';
    if (u < gc) return 'C';
    if (u < gc + (1.0 - gc) * 0.5) return 'A';
    return 'T';
}

inline char other_base(Rng& r, char b) {
    static const char kB[4] = {'A', 'C', 'G', 'T'};
    for (;;) {
        char c = kB[r.next() & 3];
        if (c != b) return c;
    }
}

struct Event {
    int pos;
    int kind;  // 0 substitution, 1 insertion, 2 deletion
    int len;
};

std::string mutate(const std::string& src, const gsdr_synth_cfg& c, double gc, Rng& r) {
    double id = c.id_lo + (1.0 - c.id_lo) * r.uniform();
    int L = (int)src.size();
    int nev = (int)std::floor((1.0 - id) * (double)L + 0.5);
    std::vector<Event> ev;
    ev.reserve(nev + 1);
    bool sub_only = c.mode == GSDR_MODE_SUBST_FIXED;
    for (int e = 0; e < nev; e++) {
        Event x;
        x.pos = (int)r.range(0, L - 1);
        if (sub_only || r.uniform() < c.sub_frac) {
            x.kind = 0;
            x.len = 1;
        } else {
            x.kind = (r.next() & 1) ? 1 : 2;
            x.len = (int)r.range(c.indel_lo, c.indel_hi);
        }
        ev.push_back(x);
    }
    if (sub_only && r.uniform() < c.extra_indel_frac) {
        Event x;
        x.pos = (int)r.range(0, L - 1);
        x.kind = (r.next() & 1) ? 1 : 2;
        x.len = (int)r.range(c.indel_lo, c.indel_hi);
        ev.push_back(x);
    }
    std::stable_sort(ev.begin(), ev.end(), [](const Event& a, const Event& b) { return a.pos < b.pos; });
    std::string out;
    out.reserve(L + 64);
    size_t e = 0;
    int p = 0;
    while (p < L) {
        bool consumed = false;
        char base = src[p];
        while (e < ev.size() && ev[e].pos <= p) {
            const Event& x = ev[e++];
            if (x.pos < p) continue;  // its base was deleted earlier
            if (x.kind == 0) {
                base = other_base(r, base);
            } else if (x.kind == 1) {
                for (int i = 0; i < x.len; i++) out.push_back(draw_base(r, gc));
            } else {
                p += x.len;
                consumed = true;
                break;
            }
        }
        if (consumed) continue;
        out.push_back(base);
        p++;
    }
    if (sub_only) {
        while ((int)out.size() < L) out.push_back(draw_base(r, gc));
        out.resize(L);
    }
    if (out.empty()) out.push_back(draw_base(r, gc));
    return out;
}

}  // namespace

extern "C" {

void gsdr_synth_preset(int config, gsdr_synth_cfg* c) {
    std::memset(c, 0, sizeof(*c));
    c->sub_frac = 0.8;
    c->indel_lo = 1;
    c->indel_hi = 3;
    c->gc_lo = c->gc_hi = 0.5;
    c->mode = GSDR_MODE_GENERAL;
    c->seed = 20261203ull + (uint64_t)config;
    switch (config) {
        case 0:  // 10k reads, 2k seeds, 200-1000 bp, 90-100% identity
            c->n_reads = 10000; c->n_seeds = 2000;
            c->len_dist = GSDR_LEN_UNIFORM; c->len_lo = 200; c->len_hi = 1000;
            c->copies_max = 9; c->id_lo = 0.90;
            break;
        case 1:  // 200k reads, 40k seeds, lognormal(1500, 0.5) in 300-10k, 92-100%
            c->n_reads = 200000; c->n_seeds = 40000;
            c->len_dist = GSDR_LEN_LOGNORMAL; c->len_median = 1500; c->len_sigma = 0.5;
            c->len_lo = 300; c->len_hi = 10000;
            c->copies_max = 9; c->id_lo = 0.92;
            c->gc_lo = 0.4; c->gc_hi = 0.6;
            break;
        case 2:  // 2M reads of 150 bp, 300k seeds, 0-14 copies, 88-100%, substitutions
            c->n_reads = 2000000; c->n_seeds = 300000;
            c->len_dist = GSDR_LEN_FIXED; c->len_lo = 150; c->len_hi = 150;
            c->copies_max = 14; c->id_lo = 0.88;
            c->mode = GSDR_MODE_SUBST_FIXED; c->extra_indel_frac = 0.10;
            c->indel_lo = 1; c->indel_hi = 2;
            break;
        case 3:  // 300k reads, 60k seeds, log-uniform 2k-30k, 80-100%, subs:indel 3:1
            c->n_reads = 300000; c->n_seeds = 60000;
            c->len_dist = GSDR_LEN_LOGUNIFORM; c->len_lo = 2000; c->len_hi = 30000;
            c->copies_max = 9; c->id_lo = 0.80;
            c->sub_frac = 0.75; c->indel_lo = 1; c->indel_hi = 10;
            break;
        case 4:  // one serving job: config-0 recipe, lengths 150-5000 (size set by caller)
        default:
            c->n_reads = 1000; c->n_seeds = 200;
            c->len_dist = GSDR_LEN_UNIFORM; c->len_lo = 150; c->len_hi = 5000;
            c->copies_max = 9; c->id_lo = 0.90;
            break;
    }
}

int64_t gsdr_synth_generate(const gsdr_synth_cfg* cfg, char** out, int64_t* out_len) {
    const gsdr_synth_cfg& c = *cfg;
    *out = nullptr;
    *out_len = 0;
    if (c.n_reads <= 0 || c.n_seeds <= 0 || c.len_lo < 1 || c.len_hi < c.len_lo) return -1;
    int64_t S = std::min(c.n_seeds, c.n_reads);
    Rng master(c.seed);
    std::vector<int> copies(S);
    int64_t total = S;
    for (int64_t s = 0; s < S; s++) {
        copies[s] = (int)master.range(0, c.copies_max);
        total += copies[s];
    }
    while (total > c.n_reads) {
        int64_t s = master.range(0, S - 1);
        if (copies[s] > 0) {
            copies[s]--;
            total--;
        }
    }
    if (c.copies_max > 0) {
        while (total < c.n_reads) {
            int64_t s = master.range(0, S - 1);
            if (copies[s] < c.copies_max) {
                copies[s]++;
                total++;
            }
        }
    }
    std::vector<int64_t> first(S + 1, 0);
    for (int64_t s = 0; s < S; s++) first[s + 1] = first[s] + 1 + copies[s];
    int64_t N = first[S];
    std::vector<std::string> recs(N);
    uint64_t base_seed = master.next();
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t s = 0; s < S; s++) {
        uint64_t x = base_seed ^ ((uint64_t)s * 0xd1b54a32d192ed03ull);
        Rng r(splitmix64(x));
        double gc = c.gc_lo + (c.gc_hi - c.gc_lo) * r.uniform();
        int L = draw_length(c, r);
        std::string seq(L, 'A');
        for (int i = 0; i < L; i++) seq[i] = draw_base(r, gc);
        recs[first[s]] = seq;
        for (int k = 0; k < copies[s]; k++) recs[first[s] + 1 + k] = mutate(seq, c, gc, r);
    }
    std::vector<int64_t> perm(N);
    for (int64_t i = 0; i < N; i++) perm[i] = i;
    for (int64_t i = N - 1; i > 0; i--) {
        int64_t j = master.range(0, i);
        std::swap(perm[i], perm[j]);
    }
    int64_t bytes = 0;
    for (int64_t i = 0; i < N; i++) bytes += (int64_t)recs[i].size() + 24;
    char* buf = (char*)std::malloc((size_t)bytes + 1);
    if (!buf) return -2;
    int64_t pos = 0;
    for (int64_t i = 0; i < N; i++) {
        int64_t id = perm[i];
        pos += std::snprintf(buf + pos, 24, ">s%lld\n", (long long)id);
        std::memcpy(buf + pos, recs[id].data(), recs[id].size());
        pos += (int64_t)recs[id].size();
        buf[pos++] = '\n';
    }
    *out = buf;
    *out_len = pos;
    return N;
}

int64_t gsdr_synth_write(const gsdr_synth_cfg* cfg, const char* path) {
    char* buf = nullptr;
    int64_t len = 0;
    int64_t n = gsdr_synth_generate(cfg, &buf, &len);
    if (n < 0) return n;
    FILE* f = std::fopen(path, "wb");
    if (!f) {
        std::free(buf);
        return -3;
    }
    size_t w = std::fwrite(buf, 1, (size_t)len, f);
    std::fclose(f);
    std::free(buf);
    return w == (size_t)len ? n : -4;
}

void gsdr_synth_free(char* p) { std::free(p); }

}  // extern "C"
