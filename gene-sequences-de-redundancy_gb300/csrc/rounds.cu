// rounds.cu -- the greedy round loop on the device, plain and batched.
//
// Plain form: one representative per round, as the reference's clustering()
// (cuda-version/func.cu:1001-1066) and clusteringDrop() (func.cu:1068-1097).
// A round is a fixed sequence of kernels that read their sizes from a
// RoundState in device memory, so rounds run back to back (and inside a CUDA
// graph) with no host round trip:
//   k_filter      kernel_preFilter + kernel_makeTable/kernel_filter
//                 (func.cu:712-754, 803-826): one warp per candidate; the
//                 composition bound first, then the candidate's (k-mer, count)
//                 entries streamed with 16-byte loads against the
//                 representative's table staged in shared memory.  Survivors
//                 are queued for alignment in six length classes.
//   k_align       kernel_align (func.cu:828-999): bit-parallel LCS on a group
//                 of G warps with W pattern words per lane (lcs_sys.cuh).
//   k_compact     updataRemain (func.cu:689-699): drops clustered reads from
//                 the remain list and finds the smallest unclustered index.
//   k_advance     updateRepresentative (func.cu:677-687).
//
// Batched form: every decision is a pure function of (representative,
// candidate), so a pass takes the next R unclustered reads r_1 < ... < r_R as
// tentative representatives, computes accept(i, j) for every tentative i and
// every unclustered j > r_i at once, and then replays the reference's order:
// r_i survives iff no surviving r_h (h < i) accepted it, and each candidate
// joins the first surviving tentative that accepted it.  That is exactly what
// R consecutive reference rounds produce.
//   k_bselect     next R unclustered indices from a forward cursor
//   k_bfilter_tab / k_bfilter_idx / k_bfilter_bits / k_bfilter_mask (+ k_bexact_t)
//                 prefilter + word filter of (tentative group, candidate):
//                 transposed per-tentative tables, an inverted k-mer index,
//                 k-mer count bitmaps or per-k-mer tentative masks (the last
//                 two with exact sums for the pairs their bounds leave open);
//                 k_bprefilter in drop mode
//   k_align       as above, accepted pairs listed instead of applied
//   k_bsurvive    survival of the tentatives in order (one warp)
//   k_bclaim      first surviving tentative per candidate (keyed atomicMax)
//   k_bapply      writes the winners into cluster[]
//   k_compact, k_badvance
// R adapts per pass: it halves after a pass in which representatives absorbed
// many reads (tentatives there mostly repeat each other's work) and doubles
// otherwise (8x after a pass too small to fill the device), up to the
// caller's maximum.  The result does not depend on R.
#include <cuda_runtime.h>

#include "gsdr_device.cuh"
#include "lcs_band.cuh"
#include "lcs_bandg.cuh"
#include "lcs_sys.cuh"

namespace gsdr {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kFilterThreads = 256;
constexpr int kAlignThreads = 256;  // 8 warps: 8/G groups of G warps
constexpr int kAbsorbHigh = 64;     // absorbed reads per representative that shrink R
constexpr int kFewPairs = 16384;    // queued pairs below which R grows 8x, not 2x
// Largest band window (words) sent to the banded kernel: batched passes, plain
// rounds.  A plain round waits for its slowest pair, and a lane works through
// its pair alone, so the plain form keeps long pairs on the systolic kernels.
constexpr int kBandMaxW = 32;
constexpr int kPlainBandMaxW = 0;

__device__ __forceinline__ bool prefilter_pass(const int4 a, const int4 b, int cut) {
    const int s = min(a.x, b.x) + min(a.y, b.y) + min(a.z, b.z) + min(a.w, b.w);
    return !(s < cut);
}

// Alignment class of a pattern of `words` 32-base words; the classes hold the
// same word counts in both forms, as warps x words per lane:
//   class            0       1       2        3        4        5        6
//   words          <=32    <=64   <=128    <=256    <=512   <=1024   <=2048
//   plain form      1x1     1x2     2x2      4x2      8x2      8x4      8x8
//   batched form    1x1     1x2     1x4      1x8      2x8      4x8      8x8
// The plain form waits for every round's longest pair, so it spreads a pattern
// over more warps (shorter per-base chain); the batched form has many pairs in
// flight and packs each pattern into as few warps as it can (fewer
// instructions per DP cell, no hand-offs between warps).
__device__ __forceinline__ int align_class(int words) {
    return words <= 32 ? 0 : words <= 64 ? 1 : words <= 128 ? 2 : words <= 256 ? 3
                         : words <= 512 ? 4 : words <= 1024 ? 5
                         : words <= kMaxPatternWords ? 6 : kLongClass;
}

// Queue of a pair: a band class (kSysClasses + 0..3 for windows of 4, 8, 16,
// 32 words) when its band fits a window of at most band_max_w words, else the
// systolic length class of its pattern.  Pairs decided without alignment
// (trivial_decision) stay in the systolic classes, which decide them.
// A lane works through its pair alone, so only pairs whose serial work (text
// bases x window words) stays below R.band_serial go to the banded kernel; a
// longer one would hold up its pass.
__device__ __forceinline__ int pair_class(int T, int q, int c, int band_max_w,
                                          long long band_serial, int group_max_w) {
    if (band_max_w > 0 && T > 0 && c > 0 && q >= c && T >= c) {
        const int bw = band_words(T, q, c);
        if (bw <= band_max_w) {
            const int w = bw <= 4 ? 4 : bw <= 8 ? 8 : bw <= 16 ? 16 : 32;
            if ((long long)T * w <= band_serial)
                return kSysClasses + (w == 4 ? 0 : w == 8 ? 1 : w == 16 ? 2 : 3);
        }
        if (bw <= group_max_w) return group_class(bw);
    }
    return align_class((q + 31) >> 5);
}

__device__ __forceinline__ void queue_align(RoundState* st, Pair* pairs, int seg_cap,
                                            const DevReads& R, int rep, int q, int band_max_w) {
    const int cls =
        pair_class(R.len_gf[rep], R.len_gf[q], R.cut_base[q], band_max_w, R.band_serial,
                   R.group_max_w);
    const int slot = atomicAdd(&st->n_pairs[cls], 1);
    if (slot < seg_cap) pairs[(size_t)cls * seg_cap + slot] = Pair{rep, q};
    else st->pair_overflow = 1;
}

// A pair that passed the composition bound and the word filter: to the
// alignment queues, or with the pigeon filter on (p 1) to its queue first.
// The reference applies the pigeon filter between the two (func.cu:1030-1044);
// all three are pure functions of the pair, so the order does not change
// which pairs reach the alignment.
__device__ __forceinline__ void push_pair(RoundState* st, Pair* pairs, int seg_cap,
                                          const DevReads& R, int rep, int q, int band_max_w) {
    if (R.pig_q) {
        const int slot = atomicAdd(&st->n_pig, 1);
        if (slot < R.pig_cap) R.pig_q[slot] = Pair{rep, q};
        else st->pair_overflow = 1;
        return;
    }
    queue_align(st, pairs, seg_cap, R, rep, q, band_max_w);
}

// Input bytes of the filter stage (filter_bytes), per launch for every
// remaining candidate: its composition, cutoffs and index (28 bytes) and its
// (k-mer, count) list, or its k-mer bitmap in the bitmap form -- in the plain
// form only what the filter reads (no list behind a failed composition
// bound), in the batched forms once per launch.  Re-reads of the same bytes
// by other tentative groups are not counted.
constexpr unsigned long long kCandFixedBytes = 16 + 8 + 4;
__device__ __forceinline__ unsigned long long cand_bytes(const DevReads& R, int q, bool drop) {
    // (k >= 8: 4-byte k-mer ids and 2-byte counts)
    return kCandFixedBytes + (drop ? 0ull : (R.kcnt ? 6ull : 4ull) * (unsigned)R.n_kmer[q]);
}

// ---------------------------------------------------------------- plain form

// tent: null in the plain form.  In the batched form (table filter) this
// kernel takes the passes with a single tentative: that tentative is the
// smallest unclustered read, so every other remaining read is its candidate
// and the pass is a plain round; k_bfilter_tab takes the passes with more.
template <int K, bool DROP>
__global__ void __launch_bounds__(kFilterThreads, 6) k_filter(DevReads R, RoundState* st,
                                                           const int32_t* __restrict__ remain,
                                                           Pair* pairs, int seg_cap,
                                                           const int32_t* __restrict__ tent) {
    extern __shared__ __align__(16) uint16_t table[];
    constexpr bool BITS = !DROP && K <= kMaxBitsK;
    constexpr int NBW = BITS ? (1 << (2 * K)) / 32 : 4;
    __shared__ __align__(16) uint32_t rbits[NBW];
    if (st->done) return;
    if (tent && st->n_tent != 1) return;
    const int rep = tent ? tent[0] : st->rep;
    const int band_w = tent ? kBandMaxW : kPlainBandMaxW;
    const int n = st->n_remain;
    if (n <= 0) return;
    // a block with no candidate skips its copy of the representative's table
    if ((long long)blockIdx.x * (kFilterThreads / 32) >= n) return;
    if (!DROP) {
        constexpr int NB = 1 << (2 * K);
        uint32_t* t32 = reinterpret_cast<uint32_t*>(table);
        for (int i = threadIdx.x; i < NB / 2; i += blockDim.x) t32[i] = 0u;
        __syncthreads();
        const uint32_t* e = R.kmer + R.kmer_off[rep];
        const int ne = R.n_kmer[rep];
        for (int i = threadIdx.x; i < ne; i += blockDim.x) {
            const uint32_t v = __ldg(e + i);
            const uint32_t c = v & 0xffffu;
            if (c) table[v >> 16] = (uint16_t)c;  // kernel_makeTable: only order > 0
        }
        if (BITS)
            for (int i = threadIdx.x; i < NBW; i += blockDim.x) rbits[i] = R.kbits[(size_t)rep * NBW + i];
        __syncthreads();
    }
    const int rep_extra = BITS ? R.kextra[rep] : 0;
    const int lane = threadIdx.x & 31;
    const int4 crep = R.comp[rep];
    unsigned n_pf = 0, n_wf = 0, n_al = 0;
    unsigned long long bytes = 0;
    const int nwarps = gridDim.x * (kFilterThreads / 32);
    // Software pipeline over this warp's candidates: while candidate i is
    // decided, the composition and cutoff of candidate i+1 are already in
    // flight and the index of candidate i+2 too, so part of the chain of
    // dependent loads (remain -> scalars -> list) overlaps the previous
    // candidate's list stream.  (Prefetching the bitmap as well needs 48
    // registers, five CTAs per SM instead of six, and measured slower.)
    int idx = blockIdx.x * (kFilterThreads / 32) + (threadIdx.x >> 5);
    int q_nx = idx < n ? __ldg(remain + idx) : -1;
    int q_af = idx + nwarps < n ? __ldg(remain + idx + nwarps) : -1;
    int4 comp_nx = make_int4(0, 0, 0, 0);
    int cb_nx = 0;
    if (q_nx >= 0) {
        comp_nx = R.comp[q_nx];
        cb_nx = R.cut_base[q_nx];
    }
    for (; idx < n; idx += nwarps) {
        const int q = q_nx;
        const int4 comp_q = comp_nx;
        const int cb_q = cb_nx;
        // issue the next candidate's loads before this one's work
        q_nx = q_af;
        q_af = idx + 2 * nwarps < n ? __ldg(remain + idx + 2 * nwarps) : -1;
        if (q_nx >= 0) {
            comp_nx = R.comp[q_nx];
            cb_nx = R.cut_base[q_nx];
        }
        if (q == rep) continue;
        n_pf++;
        bytes += kCandFixedBytes;  // composition, cutoffs, index
        // kernel_preFilter (func.cu:738-754); lossless, so also used in drop mode.
        if (!prefilter_pass(crep, comp_q, cb_q - R.strict)) continue;
        if (!DROP) {
            // kernel_filter (func.cu:803-826): S = sum over distinct k-mers of
            // min(count in representative, count in candidate), compared with
            // the candidate's word cutoff.
            n_wf++;
            const int cw = R.cut_word[q];
            const int64_t koff = R.kmer_off[q];
            const int nk = R.n_kmer[q];
            bool decided = false, pass = false;
            if (BITS) {
                // D = shared k-mers (non-zero counts) bounds S: D <= S <= D + min(excesses)
                bytes += 4ull * NBW;
                const int q_extra = R.kextra[q];
                const uint4 cb = __ldcs(reinterpret_cast<const uint4*>(R.kbits + (size_t)q * NBW) + lane % (NBW / 4));
                int d = 0;
                if (lane < NBW / 4) {
                    const uint4 rb = reinterpret_cast<const uint4*>(rbits)[lane];
                    d = __popc(cb.x & rb.x) + __popc(cb.y & rb.y) + __popc(cb.z & rb.z) +
                        __popc(cb.w & rb.w);
                }
                d = warp_sum_i(d);
                if (d >= cw) decided = pass = true;
                else if (d + min(q_extra, rep_extra) < cw) decided = true;
            }
            if (!decided) {
                const int ne4 = (nk + 3) >> 2;
                const uint4* e4 = reinterpret_cast<const uint4*>(R.kmer + koff);
                bytes += 16ull * ne4;
                int sum = 0;
#pragma unroll 4
                for (int i = lane; i < ne4; i += 32) {
                    const uint4 v = __ldcs(e4 + i);
                    sum += min((uint32_t)table[v.x >> 16], v.x & 0xffffu);
                    sum += min((uint32_t)table[v.y >> 16], v.y & 0xffffu);
                    sum += min((uint32_t)table[v.z >> 16], v.z & 0xffffu);
                    sum += min((uint32_t)table[v.w >> 16], v.w & 0xffffu);
                }
                sum = warp_sum_i(sum);
                pass = !(sum < cw);
            }
            if (!pass) continue;
        }
        n_al++;
        if (lane == 0) push_pair(st, pairs, seg_cap, R, rep, q, band_w);
    }
    if (lane == 0) {
        if (n_pf) atomicAdd(&st->cnt_prefilter, (unsigned long long)n_pf);
        if (n_wf) atomicAdd(&st->cnt_word, (unsigned long long)n_wf);
        if (n_al) atomicAdd(&st->cnt_aligned, (unsigned long long)n_al);
        if (bytes) atomicAdd(&st->filter_bytes, bytes);
    }
}

// kernel_pigeon (cuda-version/func.cu:756-801) on the queued pairs, one warp
// per pair, lane = 8 of the 256 buckets: within a bucket the two position
// lists (descending) are walked together; a pair of positions at least
// `gap` apart counts and both lists advance, otherwise the larger position
// advances.  gap = raw length of the representative - ceil(raw length of
// the candidate * t), in float as the reference computes it; the pair passes
// when the count reaches the candidate's pigeon cutoff.
template <bool BATCH>
__global__ void __launch_bounds__(256) k_pigeon(DevReads R, RoundState* st, Pair* pairs,
                                                int seg_cap) {
    if (st->done) return;
    if (BATCH && st->n_tent == 0) return;
    const int np = min(st->n_pig, R.pig_cap);
    const int lane = threadIdx.x & 31;
    const int nwarps = gridDim.x * (blockDim.x >> 5);
    unsigned rejected = 0;
    for (int k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); k < np; k += nwarps) {
        const Pair p = R.pig_q[k];
        const float prod = ceilf(__fmul_rn((float)R.len[p.cand], R.threshold));
        const int gap = (int)__fsub_rn((float)R.len[p.rep], prod);
        const uint16_t* pr = R.pig + (size_t)p.rep * 256;
        const uint16_t* pc = R.pig + (size_t)p.cand * 256;
        const uint16_t* ir = R.pidx + R.off[p.rep];
        const uint16_t* ic = R.pidx + R.off[p.cand];
        int sum = 0;
        for (int t = lane; t < 256; t += 32) {
            int s1 = t > 0 ? pr[t - 1] : 0, s2 = t > 0 ? pc[t - 1] : 0;
            const int e1 = pr[t], e2 = pc[t];
            while (s1 < e1 && s2 < e2) {
                const int one = ir[s1], two = ic[s2];
                if (abs(one - two) >= gap) {
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
        sum = warp_sum_i(sum);
        if (!(sum < R.cut_pig[p.cand])) {
            if (lane == 0)
                queue_align(st, pairs, seg_cap, R, p.rep, p.cand,
                            BATCH ? kBandMaxW : kPlainBandMaxW);
        } else {
            rejected++;
        }
    }
    if (lane == 0 && rejected) atomicAdd(&st->cnt_pig_reject, (unsigned long long)rejected);
}

// ---- word lengths 8..12, plain form: the reference's global table ----------
//
// kernel_makeTable / kernel_filter / kernel_cleanTable (func.cu:712-736,
// 803-826): the representative's counts go into a 4^k-entry table in global
// memory (set before the filter, cleared after it), and one warp per
// candidate sums min(table[k-mer], count) over the candidate's entries.

__global__ void k_gtab(DevReads R, RoundState* st, int clear) {
    if (st->done) return;
    const int rep = st->rep;
    const uint32_t* e = R.kmer + R.kmer_off[rep];
    const uint16_t* c = R.kcnt + R.kmer_off[rep];
    const int ne = R.n_kmer[rep];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ne; i += gridDim.x * blockDim.x) {
        if (clear) R.gtab[e[i]] = 0;
        else if (c[i]) R.gtab[e[i]] = c[i];  // only order > 0
    }
}

__global__ void __launch_bounds__(kFilterThreads) k_filter_g(DevReads R, RoundState* st,
                                                             const int32_t* __restrict__ remain,
                                                             Pair* pairs, int seg_cap) {
    if (st->done) return;
    const int rep = st->rep;
    const int n = st->n_remain;
    if (n <= 0) return;
    const int lane = threadIdx.x & 31;
    const int4 crep = R.comp[rep];
    unsigned n_pf = 0, n_wf = 0, n_al = 0;
    unsigned long long bytes = 0;
    const int nwarps = gridDim.x * (kFilterThreads / 32);
    for (int idx = blockIdx.x * (kFilterThreads / 32) + (threadIdx.x >> 5); idx < n;
         idx += nwarps) {
        const int q = remain[idx];
        if (q == rep) continue;
        n_pf++;
        bytes += kCandFixedBytes;
        if (!prefilter_pass(crep, R.comp[q], R.cut_base[q] - R.strict)) continue;
        n_wf++;
        bytes += 6ull * (unsigned)R.n_kmer[q];  // k-mer ids and counts
        const uint32_t* e = R.kmer + R.kmer_off[q];
        const uint16_t* c = R.kcnt + R.kmer_off[q];
        const int ne = R.n_kmer[q];
        int sum = 0;
        for (int i = lane; i < ne; i += 32)
            sum += min((uint32_t)__ldg(R.gtab + __ldg(e + i)), (uint32_t)__ldg(c + i));
        sum = warp_sum_i(sum);
        if (sum < R.cut_word[q]) continue;
        n_al++;
        if (lane == 0) push_pair(st, pairs, seg_cap, R, rep, q, kPlainBandMaxW);
    }
    if (lane == 0) {
        if (n_pf) atomicAdd(&st->cnt_prefilter, (unsigned long long)n_pf);
        if (n_wf) atomicAdd(&st->cnt_word, (unsigned long long)n_wf);
        if (n_al) atomicAdd(&st->cnt_aligned, (unsigned long long)n_al);
        if (bytes) atomicAdd(&st->filter_bytes, bytes);
    }
}

// Decisions that need no alignment; -1 when the LCS must be computed.
__device__ __forceinline__ int trivial_decision(int T, int q, int c) {
    if (T == 0) return 0;  // the reference's kernel_align never decides such a pair
    if (c <= 0) return 1;  // LCS >= 0 >= cutoff
    if (q < c || T < c) return 0;
    return -1;
}

struct AlignArgs {
    const Pair* pairs;
    int seg_cap;
    int32_t* cluster;
    int* work;
    // batched form
    const uint32_t* tidx;
    uint32_t* tt;
    uint32_t* ttrow;
    Pair* acc;
    int acc_cap;
};

// An accepted pair: the plain form absorbs the candidate at once; the batched
// form lists the pair for the greedy-order resolution and records when a
// tentative accepted another tentative.
template <bool BATCH>
__device__ __forceinline__ void on_accept(RoundState* st, const AlignArgs& A, const Pair p,
                                          int pass) {
    if (!BATCH) {
        A.cluster[p.cand] = p.rep;
        return;
    }
    const int slot = atomicAdd(&st->n_acc, 1);
    if (slot < A.acc_cap) A.acc[slot] = p;
    else st->acc_overflow = 1;
    const uint32_t kc = A.tidx[p.cand];
    if ((int)(kc >> 12) == pass) {
        const int h = A.tidx[p.rep] & 0xfff, ci = kc & 0xfff;
        atomicOr(&A.tt[h * kTTWords + (ci >> 5)], 1u << (ci & 31));
        atomicOr(&A.ttrow[h >> 5], 1u << (h & 31));
    }
}

// Greedy embedding in front of the alignment, one thread per queued pair:
// walking the candidate base by base and taking, for each, the next
// occurrence in the representative after the previous match builds a common
// subsequence, so its length is a lower bound of the LCS.  When it reaches the
// cutoff the pair is accepted without the bit-parallel alignment and removed
// from its queue (rep = -1).  Any other pair is left to k_align.  Next
// occurrences come from the representative's base bit-planes.
template <bool BATCH>
__global__ void __launch_bounds__(256) k_greedy(DevReads R, RoundState* st, AlignArgs A) {
    if (st->done) return;
    if (BATCH && (st->pair_overflow || st->n_tent == 0)) return;
    const int pass = BATCH ? st->pass : 0;
    int counts[kAlignClasses], total = 0;
    for (int c = 0; c < kAlignClasses; c++) {
        counts[c] = min(st->n_pairs[c], A.seg_cap);
        total += counts[c];
    }
    unsigned acc = 0;
    unsigned long long cells = 0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x) {
        int cls = 0, kk = k;
        while (kk >= counts[cls]) kk -= counts[cls++];
        Pair* slot = const_cast<Pair*>(A.pairs) + (size_t)cls * A.seg_cap + kk;
        const Pair p = *slot;
        const int T = R.len_gf[p.rep], q = R.len_gf[p.cand], c = R.cut_base[p.cand];
        if (T == 0 || c <= 0 || q < c || T < c) continue;  // trivial: k_align decides
        // The walk is sequential, and the longest walk of a pass delays the
        // whole pass: long candidates go to the (lane-parallel) alignment
        // unless the representative is long enough for an embedding.
        if (q > 4096 || (q > 2048 && T < 3 * c)) continue;
        const int64_t po = R.pack_off[p.rep];
        const int stride = (int)((R.pack_off[p.rep + 1] - po) >> 1);
        const uint32_t* planes = R.bm + 2 * po;
        const int nw = (T + 31) >> 5;
        const uint32_t* pq = R.packed + R.pack_off[p.cand];
        // The four plane words of the current 32-base text word stay in
        // registers; a new word is loaded only when the match position
        // crosses into it.  The walk also stops when reaching the cutoff has
        // become impossible (too little text or candidate left) or, after
        // 256 matches, when the text used per match so far projects well
        // past the end: stopping only hands the pair to the alignment.
        int pos = 0, g = 0, wcur = -1;
        uint32_t p0 = 0, p1 = 0, p2 = 0, p3 = 0;
        uint32_t qw = 0;
        for (int i = 0; i < q; i++) {
            if ((i & 15) == 0) qw = __ldg(pq + (i >> 4));
            const uint32_t ch = (qw >> (30 - 2 * (i & 15))) & 3u;
            uint32_t m = 0;
            int w = pos >> 5;
            while (w < nw) {
                if (w != wcur) {
                    p0 = __ldg(planes + w);
                    p1 = __ldg(planes + stride + w);
                    p2 = __ldg(planes + 2 * stride + w);
                    p3 = __ldg(planes + 3 * stride + w);
                    wcur = w;
                }
                m = ch == 0 ? p0 : ch == 1 ? p1 : ch == 2 ? p2 : p3;
                if (32 * w < pos) m &= 0xffffffffu << (pos & 31);
                if (m) break;
                w++;
            }
            if (!m) break;
            pos = 32 * w + __ffs(m);  // one past the match
            if (++g >= c) break;
            const int need = c - g;
            if (g + (q - 1 - i) < c || T - pos < need) break;
            if (g >= 256 && (long long)pos * need > 5ll * (T - pos) * g / 4) break;
        }
        if (g >= c) {
            on_accept<BATCH>(st, A, p, pass);
            slot->rep = -1;
            acc++;
            cells += (unsigned long long)T * (unsigned long long)q;
        }
    }
    acc = warp_sum_i((int)acc);
    if ((threadIdx.x & 31) == 0 && acc) {
        if (!BATCH) atomicAdd(&st->cnt_accepted, (unsigned long long)acc);
    }
    // per-thread cell counts: one atomic per non-zero thread is rare enough
    if (cells) atomicAdd(&st->cells, cells);
}

template <int G, int W, bool BATCH>
__global__ void __launch_bounds__(kAlignThreads, 3) k_align(DevReads R, RoundState* st, AlignArgs A,
                                                         int cls) {
    constexpr int NG = (kAlignThreads / 32) / G;
    __shared__ SysGroupT<G> groups[NG];
    extern __shared__ __align__(16) uint32_t peq_all[];  // sys_peq_words(W) per warp
    if (st->done) return;
    if (BATCH && (st->pair_overflow || st->n_tent == 0)) return;
    const int np = min(st->n_pairs[cls], A.seg_cap);
    if (np <= 0) return;
    const int pass = BATCH ? st->pass : 0;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = warp / G, gw = warp % G;
    SysGroupT<G>& S = groups[g];
    const int bar_id = 1 + g, bar_n = G * 32;
    const Pair* list = A.pairs + (size_t)cls * A.seg_cap;
    if (gw == 0 && lane == 0) {
        for (int b = 0; b < G; b++) {
            S.ready[b] = 0;
            S.consumed[b] = 0;
        }
        S.stop = 0;
        S.result = 0;
        S.error = 0;
    }
    unsigned long long acc = 0, cells = 0, done = 0;
    while (true) {
        if (gw == 0 && lane == 0) S.idx = atomicAdd(A.work + cls, 1);
        group_bar(bar_id, bar_n);
        const int i = *(volatile int*)&S.idx;
        if (i >= np) break;
        const Pair p = list[i];
        if (p.rep < 0) {  // already accepted by k_greedy
            group_bar(bar_id, bar_n);
            continue;
        }
        const int T = R.len_gf[p.rep], q = R.len_gf[p.cand], c = R.cut_base[p.cand];
        const int trivial = trivial_decision(T, q, c);
        if (trivial < 0) {
            const int words = (q + 31) >> 5;
            const int B = (words + 32 * W - 1) / (32 * W);
            if (gw < B)
                done += (unsigned long long)lcs_sys_pair<W>(
                            S, peq_all + warp * sys_peq_words(W), R.packed + R.pack_off[p.cand],
                            q, R.packed + R.pack_off[p.rep], T, c, B, gw, lane, &st->error) *
                        (32ull * 32 * 32 * W);
        }
        group_bar(bar_id, bar_n);
        if (gw == 0 && lane == 0) {
            const int ok = trivial >= 0 ? trivial : (S.error ? 0 : *(volatile int*)&S.result);
            cells += (unsigned long long)T * (unsigned long long)q;
            if (ok) {
                acc++;
                on_accept<BATCH>(st, A, p, pass);
            }
            for (int b = 0; b < G; b++) {
                S.ready[b] = 0;
                S.consumed[b] = 0;
            }
            S.stop = 0;
            S.result = 0;
            S.error = 0;
        }
        group_bar(bar_id, bar_n);
    }
    if (gw == 0 && lane == 0 && cells) {
        if (!BATCH) atomicAdd(&st->cnt_accepted, acc);
        atomicAdd(&st->cells, cells);
    }
    if (lane == 0 && done) atomicAdd(&st->cells_done, done);
}

// The four single-warp classes of the batched grouping (1x1, 1x2, 1x4, 1x8)
// in one launch: a warp takes pairs from one queue that runs through classes
// 3, 2, 1, 0 in that order, so the longest pairs start first and the short
// ones fill in behind them (one kernel tail per pass instead of four).
__global__ void __launch_bounds__(kAlignThreads, 3) k_align_single(DevReads R, RoundState* st,
                                                                   AlignArgs A, int* work) {
    __shared__ SysGroupT<1> groups[kAlignThreads / 32];  // one single-warp group per warp
    extern __shared__ __align__(16) uint32_t peq_all[];  // sys_peq_words(8) per warp
    if (st->done) return;
    if (st->pair_overflow || st->n_tent == 0) return;
    int cnt[4], total = 0;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        cnt[c] = min(st->n_pairs[3 - c], A.seg_cap);
        total += cnt[c];
    }
    if (total <= 0) return;
    const int pass = st->pass;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    SysGroupT<1>& S = groups[warp];
    unsigned long long cells = 0;
    unsigned done = 0;  // blocks of 32 steps x words per lane this warp ran
    while (true) {
        int i = 0;
        if (lane == 0) i = atomicAdd(work, 1);
        i = __shfl_sync(kFull, i, 0);
        if (i >= total) break;
        int q4 = 0;
        while (i >= cnt[q4]) i -= cnt[q4++];
        const int cls = 3 - q4;
        const Pair p = A.pairs[(size_t)cls * A.seg_cap + i];
        if (p.rep < 0) continue;  // already accepted by k_greedy
        const int T = R.len_gf[p.rep], q = R.len_gf[p.cand], c = R.cut_base[p.cand];
        int ok = trivial_decision(T, q, c);
        if (ok < 0) {
            if (lane == 0) {
                S.ready[0] = 0;
                S.consumed[0] = 0;
                S.stop = 0;
                S.result = 0;
                S.error = 0;
            }
            __syncwarp();
            const uint32_t* pq = R.packed + R.pack_off[p.cand];
            const uint32_t* pt = R.packed + R.pack_off[p.rep];
            uint32_t* peq = peq_all + warp * sys_peq_words(8);
            // words per lane: the fewest that hold the pattern (1024 bases
            // each over the warp), not the class's power of two -- a step
            // costs about three integer ops per word plus three
            const int wl = (q + 1023) >> 10;  // 1..8 in these classes (q <= 8192)
            int blocks = 0;
            switch (wl) {
                case 1: blocks = lcs_sys_pair<1>(S, peq, pq, q, pt, T, c, 1, 0, lane, &st->error); break;
                case 2: blocks = lcs_sys_pair<2>(S, peq, pq, q, pt, T, c, 1, 0, lane, &st->error); break;
                case 3: blocks = lcs_sys_pair<3>(S, peq, pq, q, pt, T, c, 1, 0, lane, &st->error); break;
                case 4: blocks = lcs_sys_pair<4>(S, peq, pq, q, pt, T, c, 1, 0, lane, &st->error); break;
                case 5: blocks = lcs_sys_pair<5>(S, peq, pq, q, pt, T, c, 1, 0, lane, &st->error); break;
                case 6: blocks = lcs_sys_pair<6>(S, peq, pq, q, pt, T, c, 1, 0, lane, &st->error); break;
                case 7: blocks = lcs_sys_pair<7>(S, peq, pq, q, pt, T, c, 1, 0, lane, &st->error); break;
                default: blocks = lcs_sys_pair<8>(S, peq, pq, q, pt, T, c, 1, 0, lane, &st->error); break;
            }
            done += (unsigned)blocks * (unsigned)(wl > 8 ? 8 : wl);
            __syncwarp();
            ok = *(volatile int*)&S.error ? 0 : *(volatile int*)&S.result;
        }
        if (lane == 0) {
            cells += (unsigned long long)T * (unsigned long long)q;
            if (ok) on_accept<true>(st, A, p, pass);
        }
    }
    if (lane == 0 && cells) atomicAdd(&st->cells, cells);
    // cells: 32 steps x 32 lanes x words per lane x 32 bits per block
    if (lane == 0 && done) atomicAdd(&st->cells_done, (unsigned long long)done * (32ull * 32 * 32));
}

// Banded alignment (lcs_band.cuh) of the pairs of band class cls, whose band
// fits a window of W words: one pair per lane.  All lanes of a warp run the
// same blocks of 32 text bases, each on its own pair; a lane whose pair is
// decided takes the next one from the class queue at the next block.
template <int W, bool BATCH>
__global__ void __launch_bounds__(kAlignThreads) k_band(DevReads R, RoundState* st, AlignArgs A,
                                                        int cls) {
    // text bases per unrolled group: fewer for wide windows (code size)
    constexpr int G = W >= 16 ? 4 : 8;
    if (st->done) return;
    if (BATCH && (st->pair_overflow || st->n_tent == 0)) return;
    const int np = min(st->n_pairs[cls], A.seg_cap);
    if (np <= 0) return;
    const int pass = BATCH ? st->pass : 0;
    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    const Pair* list = A.pairs + (size_t)cls * A.seg_cap;
    int* work = A.work + cls;
    BandLane<W> L;
    L.clear();
    Pair p{-1, -1};
    bool busy = false, more = true;
    unsigned long long cells = 0;
    unsigned acc = 0, done = 0;  // done: blocks of 32 text bases this lane ran on a pair
    while (true) {
        // lanes without a pair take the next ones (one atomic per warp)
        unsigned need = __ballot_sync(kFull, !busy);
        while (need && more) {
            int base = 0;
            if (lane == 0) base = atomicAdd(work, __popc(need));
            base = __shfl_sync(kFull, base, 0);
            if (!busy) {
                const int i = base + __popc(need & lt_mask);
                if (i < np) {
                    const Pair pp = list[i];
                    if (pp.rep >= 0) {  // not already accepted by k_greedy
                        p = pp;
                        L.start(R.packed + R.pack_off[pp.cand], R.len_gf[pp.cand],
                                R.packed + R.pack_off[pp.rep], R.len_gf[pp.rep],
                                R.cut_base[pp.cand]);
                        busy = true;
                    }
                }
            }
            if (base + __popc(need) >= np) more = false;
            need = __ballot_sync(kFull, !busy);
        }
        if (!__any_sync(kFull, busy)) break;
        // one block of 32 text bases; an idle lane runs it with no bases
        uint32_t tw0 = 0, tw1 = 0;
        if (busy) {
            if (L.x0 < L.T) tw0 = __ldg(L.pt + (L.x0 >> 4));
            if (L.x0 + 16 < L.T) tw1 = __ldg(L.pt + (L.x0 >> 4) + 1);
        }
#pragma unroll 1
        for (int j0 = 0; j0 < 32; j0 += G) L.template steps<G>(j0 < 16 ? tw0 : tw1, j0);
        if (busy) {
            done++;
            const int d = L.finish_block();
            if (d >= 0) {
                cells += (unsigned long long)L.T * (unsigned long long)L.q;
                if (d) {
                    acc++;
                    on_accept<BATCH>(st, A, p, pass);
                }
                busy = false;
                L.T = 0;
            }
        }
    }
    acc = (unsigned)warp_sum_i((int)acc);
    if (!BATCH && lane == 0 && acc) atomicAdd(&st->cnt_accepted, (unsigned long long)acc);
    if (cells) atomicAdd(&st->cells, cells);
    // cells: 32 bases x the window's W words x 32 bits per block
    if (done) atomicAdd(&st->cells_done, (unsigned long long)done * (32ull * 32 * W));
}

// Banded alignment (lcs_bandg.cuh) of the pairs of group class cls: one pair
// per group of G lanes (window of 4G words); a group whose pair is decided
// takes the next one from the class queue at the next block of 32 text bases.
template <int G, bool BATCH>
__global__ void __launch_bounds__(kAlignThreads) k_bandg(DevReads R, RoundState* st, AlignArgs A,
                                                         int cls) {
    if (st->done) return;
    if (BATCH && (st->pair_overflow || st->n_tent == 0)) return;
    const int np = min(st->n_pairs[cls], A.seg_cap);
    if (np <= 0) return;
    const int pass = BATCH ? st->pass : 0;
    const int lane = threadIdx.x & 31;
    const bool leader = (lane & (G - 1)) == 0;
    const unsigned lt_mask = (1u << lane) - 1u;
    const Pair* list = A.pairs + (size_t)cls * A.seg_cap;
    int* work = A.work + cls;
    __shared__ uint4 btab[kAlignThreads / 32][4 * 32];  // match masks, per warp
    __shared__ unsigned s_done[kAlignThreads / 32];  // blocks of 32 bases run by busy groups
    if (lane == 0) s_done[threadIdx.x >> 5] = 0;
    BandGroup<G> L;
    L.init_lane(lane, btab[threadIdx.x >> 5]);
    L.clear();
    Pair p{-1, -1};
    bool busy = false, more = true;
    unsigned long long cells = 0;
    unsigned acc = 0;
    while (true) {
        // idle groups take the next pairs (one atomic per warp, by the leaders)
        unsigned need = __ballot_sync(kFull, leader && !busy);
        while (need && more) {
            int base = 0;
            if (lane == 0) base = atomicAdd(work, __popc(need));
            base = __shfl_sync(kFull, base, 0);
            const int mine = base + __popc(need & lt_mask);  // meaningful in idle leaders
            const int i = __shfl_sync(kFull, mine, 0, G);
            if (!busy && i < np) {
                const Pair pp = list[i];
                if (pp.rep >= 0) {  // not already accepted by k_greedy
                    p = pp;
                    L.start(R.packed + R.pack_off[pp.cand], R.len_gf[pp.cand],
                            R.packed + R.pack_off[pp.rep], R.len_gf[pp.rep], R.cut_base[pp.cand]);
                    busy = true;
                }
            }
            if (base + __popc(need) >= np) more = false;
            need = __ballot_sync(kFull, leader && !busy);
        }
        if (!__any_sync(kFull, busy)) break;
        uint32_t tw0 = 0, tw1 = 0;
        if (busy) {
            if (L.x0 < L.T) tw0 = __ldg(L.pt + (L.x0 >> 4));
            if (L.x0 + 16 < L.T) tw1 = __ldg(L.pt + (L.x0 >> 4) + 1);
        }
        // a block inside every busy group's text takes the table path
        if (__all_sync(kFull, !busy || L.x0 + 32 <= L.T)) L.block_full(tw0, tw1);
        else L.block(tw0, tw1);
        const int d = L.finish_block(busy);
        {
            const unsigned ran = __ballot_sync(kFull, busy && leader);
            if (lane == 0) s_done[threadIdx.x >> 5] += __popc(ran);
        }
        if (busy && d >= 0) {
            if (leader) {
                cells += (unsigned long long)L.T * (unsigned long long)L.q;
                if (d) {
                    acc++;
                    on_accept<BATCH>(st, A, p, pass);
                }
            }
            busy = false;
            L.clear();
        }
    }
    acc = (unsigned)warp_sum_i((int)acc);
    if (!BATCH && lane == 0 && acc) atomicAdd(&st->cnt_accepted, (unsigned long long)acc);
    if (cells) atomicAdd(&st->cells, cells);
    // cells: 32 bases x the window's 4G words x 32 bits per block
    if (lane == 0 && s_done[threadIdx.x >> 5])
        atomicAdd(&st->cells_done,
                  (unsigned long long)s_done[threadIdx.x >> 5] * (32ull * 32 * 4 * G));
}

// Pairs whose pattern has more rows than one group of 8 warps x 32 lanes x 8
// words holds (class kLongClass): one block per pair runs the pattern in
// chunks of 65,536 rows (lcs_sys_pair's chunk mode), the carry sequence
// between chunks in the block's pair of global buffers; the decision is the
// zero count summed over the chunks against the cutoff (no early exit).
constexpr int kChunkRows = 32 * kMaxPatternWords;

template <bool BATCH>
__global__ void __launch_bounds__(kAlignThreads, 1) k_align_long(DevReads R, RoundState* st,
                                                                 AlignArgs A, uint32_t* carry,
                                                                 int carry_words) {
    __shared__ SysGroup S;
    __shared__ int s_idx;
    extern __shared__ __align__(16) uint32_t peq_all[];  // sys_peq_words(8) per warp
    if (st->done) return;
    if (BATCH && (st->pair_overflow || st->n_tent == 0)) return;
    const int np = min(st->n_pairs[kLongClass], A.seg_cap);
    if (np <= 0 || !carry) return;
    const int pass = BATCH ? st->pass : 0;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t* buf0 = carry + (size_t)blockIdx.x * 2 * carry_words;
    uint32_t* buf1 = buf0 + carry_words;
    unsigned long long acc = 0, cells = 0, done = 0;
    while (true) {
        if (threadIdx.x == 0) s_idx = atomicAdd(A.work + kLongClass, 1);
        __syncthreads();
        const int i = s_idx;
        __syncthreads();
        if (i >= np) break;
        const Pair p = A.pairs[(size_t)kLongClass * A.seg_cap + i];
        if (p.rep < 0) continue;  // already accepted by k_greedy
        const int T = R.len_gf[p.rep], q = R.len_gf[p.cand], c = R.cut_base[p.cand];
        int ok = trivial_decision(T, q, c);
        if (ok < 0) {
            const uint32_t* pq = R.packed + R.pack_off[p.cand];
            const uint32_t* pt = R.packed + R.pack_off[p.rep];
            const int nch = (q + kChunkRows - 1) / kChunkRows;
            int ztot = 0;
            bool err = false;
            for (int k = 0; k < nch && !err; k++) {
                if (threadIdx.x == 0) {
                    for (int b = 0; b < 8; b++) {
                        S.ready[b] = 0;
                        S.consumed[b] = 0;
                    }
                    S.stop = 0;
                    S.result = 0;
                    S.error = 0;
                }
                __syncthreads();
                const int qk = min(kChunkRows, q - k * kChunkRows);
                const int B = (((qk + 31) >> 5) + 32 * 8 - 1) / (32 * 8);
                const uint32_t* cin = k > 0 ? ((k & 1) ? buf0 : buf1) : nullptr;
                uint32_t* cout = k + 1 < nch ? ((k & 1) ? buf1 : buf0) : nullptr;
                if (warp < B)
                    done += (unsigned long long)lcs_sys_pair<8>(
                                S, peq_all + warp * sys_peq_words(8),
                                pq + (size_t)k * (kChunkRows / 16), qk, pt, T, c, B, warp, lane,
                                &st->error, true, cin, cout) *
                            (32ull * 32 * 32 * 8);
                __syncthreads();
                err = *(volatile int*)&S.error != 0;
                ztot += *(volatile int*)&S.result;
                __syncthreads();
            }
            ok = err ? 0 : (ztot >= c ? 1 : 0);
        }
        if (threadIdx.x == 0) {
            cells += (unsigned long long)T * (unsigned long long)q;
            if (ok) {
                acc++;
                on_accept<BATCH>(st, A, p, pass);
            }
        }
    }
    if (threadIdx.x == 0) {
        if (!BATCH && acc) atomicAdd(&st->cnt_accepted, acc);
        if (cells) atomicAdd(&st->cells, cells);
    }
    if (lane == 0 && done) atomicAdd(&st->cells_done, done);
}

__global__ void k_compact(RoundState* st, const int32_t* __restrict__ remain_in,
                          int32_t* __restrict__ remain_out, const int32_t* __restrict__ cluster) {
    if (st->done) return;
    const int n = st->n_remain;
    const int lane = threadIdx.x & 31;
    int local_min = 0x7fffffff;
    const int stride = gridDim.x * blockDim.x;
    for (int base = blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < n; base += stride) {
        const int idx = base + lane;
        int j = -1;
        bool keep = false;
        if (idx < n) {
            j = remain_in[idx];
            keep = cluster[j] == -1;
        }
        const unsigned m = __ballot_sync(kFull, keep);
        if (!m) continue;
        int pos = 0;
        if (lane == 0) pos = atomicAdd(&st->n_next, __popc(m));
        pos = __shfl_sync(kFull, pos, 0);
        if (keep) {
            remain_out[pos + __popc(m & ((1u << lane) - 1u))] = j;
            local_min = min(local_min, j);
        }
    }
    local_min = __reduce_min_sync(kFull, local_min);
    if (lane == 0 && local_min != 0x7fffffff) atomicMin(&st->next_min, local_min);
}

__device__ void reset_align_counters(RoundState* st, int* align_work) {
    st->n_pig = 0;
    for (int c = 0; c < kAlignClasses; c++) {
        st->n_pairs[c] = 0;
        align_work[c] = 0;
    }
    align_work[kSingleWorkSlot] = 0;  // k_align_single's shared queue
}

__global__ void k_advance(RoundState* st, int32_t* cluster, int* align_work) {
    if (st->done) return;
    st->rounds += 1;
    st->passes += 1;
    if (st->error || st->pair_overflow) {
        st->done = 1;
        return;
    }
    const int n = st->n_next;
    if (n == 0) {
        st->done = 1;
        return;
    }
    // a run stopped after pass_limit rounds (timing runs, checkpoints) leaves
    // the next representative unclustered, so that cluster[] alone is the
    // loop's state: a resumed run takes it as the smallest unclustered read
    if (st->pass_limit > 0 && st->passes >= st->pass_limit) {
        st->done = 1;
        return;
    }
    const int rep = st->next_min;
    cluster[rep] = rep;
    st->rep = rep;
    st->n_remain = n;
    st->n_next = 0;
    st->next_min = 0x7fffffff;
    reset_align_counters(st, align_work);
}

// ---------------------------------------------------------------- batched form

// Next R unclustered indices at or after the cursor, in increasing order.
__global__ void __launch_bounds__(1024) k_bselect(RoundState* st, const int32_t* __restrict__ cluster,
                                                  int n, int32_t* tent, uint32_t* tidx,
                                                  uint32_t* tt, uint32_t* ttrow, uint32_t* survive,
                                                  int* align_work) {
    __shared__ int warp_cnt[32];
    __shared__ int s_nt;
    if (st->done) return;
    const int Rq = st->R;
    const int pass = st->pass;
    int pos = st->cursor;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_nt = 0;
    __syncthreads();
    while (pos < n) {
        const int nt = s_nt;
        if (nt >= Rq) break;
        const int idx = pos + threadIdx.x;
        const bool un = idx < n && cluster[idx] == -1;
        const unsigned m = __ballot_sync(kFull, un);
        if (lane == 0) warp_cnt[warp] = __popc(m);
        __syncthreads();
        int before = 0, total = 0;
        for (int w = 0; w < 32; w++) {
            const int c = warp_cnt[w];
            if (w < warp) before += c;
            total += c;
        }
        const int rank = nt + before + __popc(m & ((1u << lane) - 1u));
        if (un && rank < Rq) {
            tent[rank] = idx;
            tidx[idx] = ((uint32_t)pass << 12) | (uint32_t)rank;
        }
        __syncthreads();
        if (threadIdx.x == 0) s_nt = min(Rq, nt + total);
        pos += blockDim.x;
        __syncthreads();
    }
    const int nt = s_nt;
    for (int i = threadIdx.x; i < nt * kTTWords; i += blockDim.x) tt[i] = 0u;
    if (threadIdx.x < kTTWords) {
        ttrow[threadIdx.x] = 0u;
        survive[threadIdx.x] = 0u;
    }
    if (threadIdx.x == 0) {
        st->n_tent = nt;
        st->n_acc = 0;
        st->n_amb = 0;
        st->acc_overflow = 0;
        st->pair_overflow = 0;
        st->survivors = 0;
        st->absorbed = 0;
        reset_align_counters(st, align_work);
        if (nt == 0) st->done = 1;
    }
}

// Per-tentative tables, transposed (k_bfilter_tab): for each k-mer the counts
// of a group's RG tentatives lie side by side (RG u16 = RG/8 16-byte words),
// so one candidate entry (k-mer, count c) costs RG/8 vector loads and, per
// pair of tentatives, one paired 16-bit min against (c, c) and one paired
// 16-bit add into the lane's sums.  A sum is at most the candidate's k-mer
// count (< 65536), so the halves never carry into each other, and a warp-wide
// 32-bit reduction adds both halves at once.
template <int K>
struct TabGroup {
    static constexpr int RG = K <= 5 ? 32 : K == 6 ? 16 : 4;
    static constexpr int NB = 1 << (2 * K);
    // u16 per k-mer row: the group's RG counts, padded by 16 bytes where a
    // row is read with 16-byte loads.  A warp reads random rows; with a
    // 32-byte (64-byte) stride the first 16 bytes of a row fall in only 4 (2)
    // of the 8 16-byte bank groups of a 128-byte line, with 48 (80) bytes in
    // all 8, which cuts the bank conflicts of a quarter-warp's loads.
    static constexpr int ROW = RG >= 8 ? RG + 8 : RG;
    static constexpr int smem = NB * ROW * 2;  // 80 KB (k 5), 192 KB (k 6), 128 KB (k 7)
};
constexpr int kTabThreads = 1024;

template <int K>
__global__ void __launch_bounds__(kTabThreads, 1) k_bfilter_tab(DevReads R, RoundState* st,
                                                                const int32_t* __restrict__ remain,
                                                                const int32_t* __restrict__ tent,
                                                                Pair* pairs, int seg_cap) {
    constexpr int RG = TabGroup<K>::RG;
    constexpr int ROW = TabGroup<K>::ROW;
    constexpr int W = RG / 2;  // packed sums per lane
    constexpr int WARPS = kTabThreads / 32;
    extern __shared__ __align__(16) uint16_t tab[];  // [NB][ROW], RG counts used per row
    __shared__ int4 tcomp[RG];
    __shared__ int ttent[RG];
    // a pass with a single tentative is k_filter's (launched before this one)
    if (st->done || st->n_tent <= 1) return;
    const int nt = st->n_tent;
    const int n = st->n_remain;
    const int ngroups = (nt + RG - 1) / RG;
    const int parts = max(1, (int)gridDim.x / ngroups);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned n_pf = 0, n_wf = 0, n_al = 0;
    unsigned long long bytes = 0;
    int cur_group = -1;
    for (int item = blockIdx.x; item < ngroups * parts; item += gridDim.x) {
        const int g = item % ngroups, part = item / ngroups;
        const int t0 = g * RG;
        const int ng = min(RG, nt - t0);
        if (g != cur_group) {
            __syncthreads();
            if (threadIdx.x < RG) {
                const int i = t0 + threadIdx.x;
                ttent[threadIdx.x] = threadIdx.x < ng ? tent[i] : 0x7fffffff;
                tcomp[threadIdx.x] = threadIdx.x < ng ? R.comp[tent[i]] : make_int4(0, 0, 0, 0);
            }
            uint4* t4 = reinterpret_cast<uint4*>(tab);
            for (int i = threadIdx.x; i < TabGroup<K>::smem / 16; i += kTabThreads)
                t4[i] = make_uint4(0u, 0u, 0u, 0u);
            __syncthreads();
            // kernel_makeTable (func.cu:712-723) for each tentative: order > 0 only
            for (int t = warp; t < ng; t += WARPS) {
                const int rep = ttent[t];
                const uint32_t* e = R.kmer + R.kmer_off[rep];
                const int ne = R.n_kmer[rep];
                for (int i = lane; i < ne; i += 32) {
                    const uint32_t v = __ldg(e + i);
                    const uint32_t c = v & 0xffffu;
                    if (c) tab[(v >> 16) * ROW + t] = (uint16_t)c;
                }
            }
            __syncthreads();
            cur_group = g;
        }
        const int per = (n + parts - 1) / parts;
        const int lo = part * per, hi = min(n, lo + per);
        for (int idx = lo + warp; idx < hi; idx += WARPS) {
            const int q = remain[idx];
            if (g == 0) bytes += cand_bytes(R, q, false);  // once per launch
            // lane t < RG: order and composition bound of tentative t
            bool ok = false;
            if (lane < ng) {
                ok = ttent[lane] < q &&
                     prefilter_pass(tcomp[lane], R.comp[q], R.cut_base[q] - R.strict);
                n_pf += ttent[lane] < q;
            }
            const unsigned mask = __ballot_sync(kFull, ok);
            if (!mask) continue;
            n_wf += ok;
            uint32_t acc[W];
#pragma unroll
            for (int w = 0; w < W; w++) acc[w] = 0u;
            const int ne4 = (R.n_kmer[q] + 3) >> 2;
            const uint4* e4 = reinterpret_cast<const uint4*>(R.kmer + R.kmer_off[q]);
            for (int i = lane; i < ne4; i += 32) {
                const uint4 v = __ldcs(e4 + i);
                const uint32_t ev[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const uint32_t c = ev[e] & 0xffffu;
                    const uint32_t cc = c | (c << 16);
                    const uint32_t* row = reinterpret_cast<const uint32_t*>(tab + (ev[e] >> 16) * ROW);
                    if constexpr (RG >= 8) {
#pragma unroll
                        for (int w = 0; w < W; w += 4) {
                            const uint4 m = *reinterpret_cast<const uint4*>(row + w);
                            acc[w] = __vadd2(acc[w], __vminu2(m.x, cc));
                            acc[w + 1] = __vadd2(acc[w + 1], __vminu2(m.y, cc));
                            acc[w + 2] = __vadd2(acc[w + 2], __vminu2(m.z, cc));
                            acc[w + 3] = __vadd2(acc[w + 3], __vminu2(m.w, cc));
                        }
                    } else {
                        const uint2 m = *reinterpret_cast<const uint2*>(row);
                        acc[0] = __vadd2(acc[0], __vminu2(m.x, cc));
                        acc[1] = __vadd2(acc[1], __vminu2(m.y, cc));
                    }
                }
            }
            const int cw = R.cut_word[q];
            uint32_t mine = 0;
#pragma unroll
            for (int w = 0; w < W; w++) {
                const uint32_t s = __reduce_add_sync(kFull, acc[w]);
                if ((lane >> 1) == w) mine = s;
            }
            const int sum = (int)((lane & 1) ? (mine >> 16) : (mine & 0xffffu));
            const bool pass = ok && !(sum < cw);
            if (pass) push_pair(st, pairs, seg_cap, R, ttent[lane], q, kBandMaxW);
            n_al += pass;
        }
    }
    n_pf = (unsigned)warp_sum_i((int)n_pf);
    n_wf = (unsigned)warp_sum_i((int)n_wf);
    n_al = (unsigned)warp_sum_i((int)n_al);
    if (lane == 0) {
        if (n_pf) atomicAdd(&st->cnt_prefilter, (unsigned long long)n_pf);
        if (n_wf) atomicAdd(&st->cnt_word, (unsigned long long)n_wf);
        if (n_al) atomicAdd(&st->cnt_aligned, (unsigned long long)n_al);
        if (bytes) atomicAdd(&st->filter_bytes, bytes);
    }
}

// Drop mode, batched (clusteringDrop, func.cu:1068-1097): only the lossless
// composition bound (kernel_preFilter, func.cu:738-754) runs before the
// alignment.  A CTA stages 32 tentatives; one warp per candidate, lane t
// tests tentative t.
__global__ void __launch_bounds__(kFilterThreads) k_bprefilter(DevReads R, RoundState* st,
                                                               const int32_t* __restrict__ remain,
                                                               const int32_t* __restrict__ tent,
                                                               Pair* pairs, int seg_cap) {
    constexpr int RG = 32;
    __shared__ int4 tcomp[RG];
    __shared__ int ttent[RG];
    if (st->done || st->n_tent == 0) return;
    const int nt = st->n_tent;
    const int n = st->n_remain;
    const int ngroups = (nt + RG - 1) / RG;
    const int parts = max(1, (int)gridDim.x / ngroups);
    const int lane = threadIdx.x & 31;
    unsigned n_pf = 0, n_al = 0;
    unsigned long long bytes = 0;
    int cur_group = -1;
    for (int item = blockIdx.x; item < ngroups * parts; item += gridDim.x) {
        const int g = item % ngroups, part = item / ngroups;
        const int t0 = g * RG;
        const int ng = min(RG, nt - t0);
        if (g != cur_group) {
            __syncthreads();
            if (threadIdx.x < RG) {
                const int i = t0 + threadIdx.x;
                ttent[threadIdx.x] = threadIdx.x < ng ? tent[i] : 0x7fffffff;
                tcomp[threadIdx.x] = threadIdx.x < ng ? R.comp[tent[i]] : make_int4(0, 0, 0, 0);
            }
            __syncthreads();
            cur_group = g;
        }
        // this item's slice of the candidate list, one warp per candidate
        const int per = (n + parts - 1) / parts;
        const int lo = part * per, hi = min(n, lo + per);
        for (int idx = lo + (threadIdx.x >> 5); idx < hi; idx += kFilterThreads / 32) {
            const int q = remain[idx];
            if (g == 0) bytes += cand_bytes(R, q, true);  // once per launch
            bool ok = false;
            if (lane < ng) {
                ok = ttent[lane] < q &&
                     prefilter_pass(tcomp[lane], R.comp[q], R.cut_base[q] - R.strict);
                n_pf += ttent[lane] < q;
            }
            if (ok) push_pair(st, pairs, seg_cap, R, ttent[lane], q, kBandMaxW);
            n_al += ok;
        }
    }
    n_pf = (unsigned)warp_sum_i((int)n_pf);
    n_al = (unsigned)warp_sum_i((int)n_al);
    if (lane == 0) {
        if (n_pf) atomicAdd(&st->cnt_prefilter, (unsigned long long)n_pf);
        if (n_al) atomicAdd(&st->cnt_aligned, (unsigned long long)n_al);
        if (bytes) atomicAdd(&st->filter_bytes, bytes);
    }
}

// ---- word filter by two-level k-mer count bitmaps (k <= kMaxBitsK) --------
//
// Per read two 4^k-bit bitmaps: level 1 holds the k-mers with a stored count
// of at least one, level 2 those with at least two; E3 is the excess above
// two, sum over k-mers of max(count - 2, 0).  The word sum of kernel_filter
// (func.cu:803-826) is S = sum over k-mers of min(c_t, c_q), and since
// min(c_t, c_q) = [both >= 1] + [both >= 2] + max(min(c_t, c_q) - 2, 0),
//     lo = D1 + D2 <= S <= lo + min(E3_t, E3_q),
// with D1, D2 the popcounts of the two levels' intersections.  k_bfilter_bits
// forms lo with 2 x 4^k / 32 AND + POPC per pair (lane = tentative, no table
// lookups, no bank conflicts) and decides every pair outside the gap; the few
// pairs inside it go to k_bexact_t, which forms S itself.  The second level
// keeps the gap small where one level leaves it wide (reads holding a large
// share of the k-mer space, whose counts are mostly 1 or 2).

// Carry-save adder: a + b + c = s + 2 * carry, bit by bit (two LOP3s).
__device__ __forceinline__ void csa(uint32_t& s, uint32_t& carry, uint32_t a, uint32_t b,
                                    uint32_t c) {
    s = a ^ b ^ c;
    carry = (a & b) | (c & (a ^ b));
}

// The summed population count of eight words with four POPCs (the POPC pipe
// bounds the bitmap filter): a tree of carry-save adders (Harley and Seal)
// reduces them to words of weight 1, 1, 2 and 4 first.
__device__ __forceinline__ int popc8(uint32_t w0, uint32_t w1, uint32_t w2, uint32_t w3,
                                     uint32_t w4, uint32_t w5, uint32_t w6, uint32_t w7) {
    uint32_t s1, c1, s2, c2, s3, c3, t2, f4;
    csa(s1, c1, w0, w1, w2);
    csa(s2, c2, w3, w4, w5);
    csa(s3, c3, s1, s2, w6);
    csa(t2, f4, c1, c2, c3);
    return __popc(s3) + __popc(w7) + 2 * __popc(t2) + 4 * __popc(f4);
}

// Shared memory of k_bfilter_bits: the group's two bitmap levels as
// [level][quad][tentative] (lane t reads consecutive 16 bytes: conflict-free),
// each warp's candidate bitmaps, and the group's tentatives, compositions and
// excesses.  k <= 6: 128 tentatives per CTA of 32 warps (163 KB); k = 7, whose
// bitmaps are four times larger: 32 tentatives per CTA of 16 warps (193 KB).
template <int K>
struct BitsSmem {
    static constexpr int NQ = (1 << (2 * K)) / 128;  // 16-byte words of one bitmap
    static constexpr int RG = K <= 6 ? 128 : 32;     // tentatives staged per CTA
    static constexpr int THREADS = K <= 6 ? 1024 : 512;
    static constexpr int WARPS = THREADS / 32;
    static constexpr size_t tb_quads = 2 * (size_t)NQ * RG;
    static constexpr size_t cb_quads = (size_t)WARPS * 2 * NQ;
    static constexpr size_t bytes = 16 * (tb_quads + cb_quads) + RG * (16 + 4 + 4);
};

template <int K>
__global__ void __launch_bounds__(BitsSmem<K>::THREADS, 1) k_bfilter_bits(DevReads R, RoundState* st,
                                                                  const int32_t* __restrict__ remain,
                                                                  const int32_t* __restrict__ tent,
                                                                  Pair* pairs, int seg_cap, Pair* amb,
                                                                  int amb_cap) {
    using L = BitsSmem<K>;
    constexpr int NQ = L::NQ;
    constexpr int RG = L::RG;
    constexpr int WARPS = L::WARPS;
    extern __shared__ __align__(16) uint4 bsm[];
    uint4* tb = bsm;                                  // tb[(level * NQ + w) * RG + t]
    uint4* cball = bsm + L::tb_quads;                 // cb[(warp * 2 + level) * NQ + w]
    int4* tcomp = reinterpret_cast<int4*>(cball + L::cb_quads);
    int* ttent = reinterpret_cast<int*>(tcomp + RG);
    int* textra = ttent + RG;
    if (st->done) return;
    const int nt = st->n_tent;
    if (nt <= 1) return;  // a single tentative's pass runs k_filter instead
    const int n = st->n_remain;
    const int ngroups = (nt + RG - 1) / RG;
    const int parts = max(1, (int)gridDim.x / ngroups);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint4* cb = cball + warp * 2 * NQ;
    const uint4* kb1 = reinterpret_cast<const uint4*>(R.kbits);
    const uint4* kb2 = reinterpret_cast<const uint4*>(R.kbits2);
    unsigned n_pf = 0, n_wf = 0, n_al = 0;
    unsigned long long bytes = 0;
    int cur_group = -1;
    for (int item = blockIdx.x; item < ngroups * parts; item += gridDim.x) {
        const int g = item % ngroups, part = item / ngroups;
        const int t0 = g * RG;
        const int ng = min(RG, nt - t0);
        if (g != cur_group) {
            __syncthreads();
            if (threadIdx.x < RG) {
                const bool in = (int)threadIdx.x < ng;
                const int rep = in ? tent[t0 + threadIdx.x] : 0;
                ttent[threadIdx.x] = in ? rep : 0x7fffffff;
                tcomp[threadIdx.x] = in ? R.comp[rep] : make_int4(0, 0, 0, 0);
                textra[threadIdx.x] = in ? R.kextra3[rep] : 0;
            }
            for (int i = threadIdx.x; i < 2 * NQ * RG; i += L::THREADS) {
                const int t = i % RG, lw = i / RG, lv = lw / NQ, w = lw % NQ;
                uint4 v = make_uint4(0u, 0u, 0u, 0u);
                if (t < ng) v = __ldg((lv ? kb2 : kb1) + (size_t)tent[t0 + t] * NQ + w);
                tb[i] = v;
            }
            __syncthreads();
            cur_group = g;
        }
        const int per = (n + parts - 1) / parts;
        const int lo = part * per, hi = min(n, lo + per);
        for (int idx = lo + warp; idx < hi; idx += WARPS) {
            const int q = remain[idx];
            if (g == 0) bytes += kCandFixedBytes + 2ull * 16 * NQ;  // once per launch
            const int4 cq = R.comp[q];
            const int cbq = R.cut_base[q] - R.strict;  // the prefilter's cutoff
            unsigned ok_bits[RG / 32];
            bool any = false;
#pragma unroll
            for (int h = 0; h < RG / 32; h++) {
                const int t = 32 * h + lane;
                const bool before = t < ng && ttent[t] < q;
                n_pf += before;
                // kernel_preFilter (func.cu:738-754) first
                const bool ok = before && prefilter_pass(tcomp[t], cq, cbq);
                ok_bits[h] = __ballot_sync(kFull, ok);
                any |= ok_bits[h] != 0;
            }
            if (!any) continue;
            for (int i = lane; i < 2 * NQ; i += 32)
                cb[i] = __ldcs((i < NQ ? kb1 : kb2) + (size_t)q * NQ + (i % NQ));
            __syncwarp();
            const int cw = R.cut_word[q];
            const int exq = R.kextra3[q];
            // word by word: the candidate's two quads load once and serve every
            // chunk of 32 tentatives with a pair left (fewer shared loads: the
            // kernel is bound by their issue queue and the POPC pipe)
            int dsum[RG / 32];
#pragma unroll
            for (int h = 0; h < RG / 32; h++) dsum[h] = 0;
#pragma unroll 1
            for (int w = 0; w < NQ; w++) {
                const uint4 a1 = cb[w], a2 = cb[NQ + w];
#pragma unroll
                for (int h = 0; h < RG / 32; h++) {
                    if (!ok_bits[h]) continue;
                    const int t = 32 * h + lane;
                    const uint4 b1 = tb[w * RG + t], b2 = tb[(NQ + w) * RG + t];
                    dsum[h] += popc8(a1.x & b1.x, a1.y & b1.y, a1.z & b1.z, a1.w & b1.w,
                                     a2.x & b2.x, a2.y & b2.y, a2.z & b2.z, a2.w & b2.w);
                }
            }
#pragma unroll
            for (int h = 0; h < RG / 32; h++) {
                if (!ok_bits[h]) continue;
                const int t = 32 * h + lane;
                const int d = dsum[h];
                if ((ok_bits[h] >> lane) & 1u) {
                    n_wf++;
                    if (d >= cw) {
                        push_pair(st, pairs, seg_cap, R, ttent[t], q, kBandMaxW);
                        n_al++;
                    } else if (d + min(textra[t], exq) >= cw) {
                        const int slot = atomicAdd(&st->n_amb, 1);
                        if (slot < amb_cap) amb[slot] = Pair{ttent[t], q};
                        else st->pair_overflow = 1;
                    }
                }
            }
            __syncwarp();
        }
    }
    n_pf = (unsigned)warp_sum_i((int)n_pf);
    n_wf = (unsigned)warp_sum_i((int)n_wf);
    n_al = (unsigned)warp_sum_i((int)n_al);
    if (lane == 0) {
        if (n_pf) atomicAdd(&st->cnt_prefilter, (unsigned long long)n_pf);
        if (n_wf) atomicAdd(&st->cnt_word, (unsigned long long)n_wf);
        if (n_al) atomicAdd(&st->cnt_aligned, (unsigned long long)n_al);
        if (bytes) atomicAdd(&st->filter_bytes, bytes);
    }
}

// The open pairs grouped by tentative.  In the early passes of long-read
// jobs most pairs are open (477k of 668k in the seventh pass of the 200k-read
// workload, ~4,600 per tentative); one table per pair would be zeroed and
// refilled ~4,600 times per tentative.  A counting sort of the queue by tentative index
// (k_amb_count, k_amb_scan, k_amb_place) lets k_bexact_t build each
// tentative's table once per CTA for a run of its pairs.  The order of the
// pairs inside a tentative's run does not matter: each decision is a pure
// function of its pair.
//
// amb_idx holds four arrays of kMaxBatch + 1: per tentative the pair count
// (kept zero between passes), the run offsets, the placement cursors and the
// work items (runs of up to kExactChunk pairs), as exclusive prefix sums.
constexpr int kExactChunk = 64;
constexpr int kAmbThreads = 256;

__device__ __forceinline__ int amb_n(const RoundState* st, int amb_cap) {
    return min(st->n_amb, amb_cap);
}

// Per-CTA histogram of the open pairs' tentatives, added into the global one.
__global__ void __launch_bounds__(kAmbThreads) k_amb_count(RoundState* st, const Pair* __restrict__ amb,
                                                          int amb_cap, const uint32_t* __restrict__ tidx,
                                                          int* amb_idx) {
    __shared__ int h[kMaxBatch];
    if (st->done || st->n_tent == 0) return;
    const int na = amb_n(st, amb_cap);
    if (na <= 0) return;
    const int nt = st->n_tent;
    for (int t = threadIdx.x; t < nt; t += blockDim.x) h[t] = 0;
    __syncthreads();
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < na; k += gridDim.x * blockDim.x)
        atomicAdd(&h[tidx[amb[k].rep] & 0xfff], 1);
    __syncthreads();
    for (int t = threadIdx.x; t < nt; t += blockDim.x)
        if (h[t]) atomicAdd(&amb_idx[t], h[t]);
}

// One CTA of 1,024 threads: run offsets, cursors and work items; the counts
// go back to zero for the next pass.
__global__ void __launch_bounds__(1024) k_amb_scan(RoundState* st, int amb_cap, int* amb_idx) {
    __shared__ int ws[2][32];
    if (st->done || st->n_tent == 0) return;
    if (amb_n(st, amb_cap) <= 0) return;
    const int nt = st->n_tent;
    int* cnt = amb_idx;
    int* off = amb_idx + (kMaxBatch + 1);
    int* cur = amb_idx + 2 * (kMaxBatch + 1);
    int* items = amb_idx + 3 * (kMaxBatch + 1);
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int c = t < nt ? cnt[t] : 0;
    const int ch = (c + kExactChunk - 1) / kExactChunk;
    int ic = c, ich = ch;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int a = __shfl_up_sync(kFull, ic, d), b = __shfl_up_sync(kFull, ich, d);
        if (lane >= d) ic += a, ich += b;
    }
    if (lane == 31) ws[0][warp] = ic, ws[1][warp] = ich;
    __syncthreads();
    int bc = 0, bch = 0;
    for (int w = 0; w < warp; w++) bc += ws[0][w], bch += ws[1][w];
    const int ec = bc + ic - c, ech = bch + ich - ch;
    if (t < nt) {
        off[t] = ec;
        cur[t] = ec;
        items[t] = ech;
        cnt[t] = 0;
    }
    if (t == nt - 1) {
        off[nt] = ec + c;
        items[nt] = ech + ch;
    }
}

// Each CTA places a contiguous range of the queue: a shared histogram, one
// global reservation per (CTA, tentative), then the pairs.
__global__ void __launch_bounds__(kAmbThreads) k_amb_place(RoundState* st, const Pair* __restrict__ amb,
                                                          int amb_cap, const uint32_t* __restrict__ tidx,
                                                          int* amb_idx, Pair* amb2) {
    __shared__ int h[kMaxBatch];
    if (st->done || st->n_tent == 0) return;
    const int na = amb_n(st, amb_cap);
    if (na <= 0) return;
    const int nt = st->n_tent;
    int* cur = amb_idx + 2 * (kMaxBatch + 1);
    const int per = (na + gridDim.x - 1) / gridDim.x;
    const int lo = blockIdx.x * per, hi = min(na, lo + per);
    if (lo >= hi) return;
    for (int t = threadIdx.x; t < nt; t += blockDim.x) h[t] = 0;
    __syncthreads();
    for (int k = lo + threadIdx.x; k < hi; k += blockDim.x) atomicAdd(&h[tidx[amb[k].rep] & 0xfff], 1);
    __syncthreads();
    for (int t = threadIdx.x; t < nt; t += blockDim.x)
        if (h[t]) h[t] = atomicAdd(&cur[t], h[t]);
    __syncthreads();
    for (int k = lo + threadIdx.x; k < hi; k += blockDim.x) {
        const Pair p = amb[k];
        amb2[atomicAdd(&h[tidx[p.rep] & 0xfff], 1)] = p;
    }
}

// The word sum S of the open pairs, run by run: a CTA takes a contiguous range
// of work items, builds the tentative's count table in shared memory when the
// tentative changes, and each warp streams one candidate's (k-mer, count)
// entries against it (kernel_filter, func.cu:803-826).
template <int K>
__global__ void __launch_bounds__(kAmbThreads) k_bexact_t(DevReads R, RoundState* st,
                                                        const Pair* __restrict__ amb2,
                                                        const int* __restrict__ amb_idx,
                                                        int amb_cap,
                                                        const int32_t* __restrict__ tent,
                                                        Pair* pairs, int seg_cap) {
    constexpr int NB = 1 << (2 * K);
    extern __shared__ __align__(16) uint16_t xtab[];  // NB counts
    __shared__ int s_items[kMaxBatch + 1];
    if (st->done || st->n_tent == 0) return;
    if (amb_n(st, amb_cap) <= 0) return;
    const int nt = st->n_tent;
    const int* off = amb_idx + (kMaxBatch + 1);
    const int* items = amb_idx + 3 * (kMaxBatch + 1);
    for (int i = threadIdx.x; i <= nt; i += blockDim.x) s_items[i] = items[i];
    __syncthreads();
    const int total = s_items[nt];
    const int per = (total + gridDim.x - 1) / gridDim.x;
    const int i0 = blockIdx.x * per, i1 = min(total, i0 + per);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
    unsigned n_al = 0;
    int cur_t = -1;
    for (int item = i0; item < i1; item++) {
        // the tentative of this item: the last t with s_items[t] <= item
        int lo = 0, hi = nt;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (s_items[mid] <= item) lo = mid;
            else hi = mid;
        }
        const int t = lo;
        if (t != cur_t) {
            __syncthreads();
            uint4* t4 = reinterpret_cast<uint4*>(xtab);
            for (int i = threadIdx.x; i < NB / 8; i += blockDim.x) t4[i] = make_uint4(0u, 0u, 0u, 0u);
            __syncthreads();
            const int rep = tent[t];
            const uint32_t* et = R.kmer + R.kmer_off[rep];
            const int ne = R.n_kmer[rep];
            for (int i = threadIdx.x; i < ne; i += blockDim.x) {
                const uint32_t v = __ldg(et + i);
                const uint32_t c = v & 0xffffu;
                if (c) xtab[v >> 16] = (uint16_t)c;  // kernel_makeTable: only order > 0
            }
            __syncthreads();
            cur_t = t;
        }
        const int k0 = off[t] + (item - s_items[t]) * kExactChunk;
        const int k1 = min(off[t + 1], k0 + kExactChunk);
        for (int k = k0 + warp; k < k1; k += warps) {
            const Pair p = amb2[k];
            const uint32_t* eq = R.kmer + R.kmer_off[p.cand];
            const int nq = R.n_kmer[p.cand];
            int sum = 0;
            for (int i = lane; i < nq; i += 32) {
                const uint32_t v = __ldg(eq + i);
                sum += min((uint32_t)xtab[v >> 16], v & 0xffffu);
            }
            sum = warp_sum_i(sum);
            if (!(sum < R.cut_word[p.cand])) {
                if (lane == 0) push_pair(st, pairs, seg_cap, R, p.rep, p.cand, kBandMaxW);
                n_al++;
            }
        }
    }
    if (lane == 0 && n_al) atomicAdd(&st->cnt_aligned, (unsigned long long)n_al);
}

// ---- word filter by inverted index (sparse k-mer spaces) -------------------
//
// With short reads and k = 7 a tentative holds ~1% of the 4^k k-mers, so the
// table form spends almost every lookup on a zero.  Instead, each pass lists,
// per k-mer, the tentatives that hold it (k_bindex), and every candidate walks
// the lists of its own k-mers once, adding min(count in tentative, count in
// candidate) into one 16-bit counter per tentative (k_bfilter_idx).  The sums
// are the same integers kernel_filter forms (func.cu:803-826); only the order
// of the additions differs.

constexpr int kIndexThreads = 1024;

// One CTA: histogram of the tentatives' k-mers, exclusive scan into idx_off,
// scatter of (tentative << 16 | count) into idx_post.  The order inside one
// k-mer's list is arbitrary; the filter's sums do not depend on it.  With
// off16/post16 (capacity below 65536) it also writes the 16-bit copy that
// k_bfilter_idx keeps in shared memory: (tentative << 6 | min(count, 63)).
template <int K>
__global__ void __launch_bounds__(kIndexThreads, 1) k_bindex(DevReads R, RoundState* st,
                                                          const int32_t* __restrict__ tent,
                                                          uint32_t* idx_off, uint32_t* idx_post,
                                                          uint16_t* off16, uint16_t* post16,
                                                          long long idx_cap) {
    constexpr int NB = 1 << (2 * K);
    constexpr int PER = NB >= kIndexThreads ? NB / kIndexThreads : 1;
    extern __shared__ uint32_t cnt[];  // NB counters, then the scatter cursors
    __shared__ uint32_t wsum[32];
    if (st->done || st->n_tent == 0) return;
    const int nt = st->n_tent;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < NB; i += kIndexThreads) cnt[i] = 0u;
    __syncthreads();
    for (int t = warp; t < nt; t += kIndexThreads / 32) {
        const int rep = tent[t];
        const uint32_t* e = R.kmer + R.kmer_off[rep];
        const int ne = R.n_kmer[rep];
        for (int i = lane; i < ne; i += 32) {
            const uint32_t v = __ldg(e + i);
            if (v & 0xffffu) atomicAdd(&cnt[v >> 16], 1u);
        }
    }
    __syncthreads();
    // exclusive scan: thread i owns counters [i*PER, i*PER + PER)
    const int base = threadIdx.x * PER;
    uint32_t run = 0;
#pragma unroll
    for (int j = 0; j < PER; j++) run += base + j < NB ? cnt[base + j] : 0u;
    uint32_t incl = run;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t o = __shfl_up_sync(kFull, incl, d);
        if (lane >= d) incl += o;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    uint32_t before = 0, total = 0;
    for (int w = 0; w < kIndexThreads / 32; w++) {
        const uint32_t s = wsum[w];
        if (w < warp) before += s;
        total += s;
    }
    uint32_t pos = before + incl - run;
#pragma unroll
    for (int j = 0; j < PER; j++) {
        if (base + j < NB) {
            const uint32_t c = cnt[base + j];
            idx_off[base + j] = pos;
            if (off16) off16[base + j] = (uint16_t)pos;
            cnt[base + j] = pos;  // becomes the scatter cursor
            pos += c;
        }
    }
    if (threadIdx.x == 0) {
        idx_off[NB] = total;
        if (off16) off16[NB] = (uint16_t)total;
    }
    if ((long long)total > idx_cap) {
        // cannot happen for length-sorted reads (the capacity holds the R_max
        // longest k-mer lists); stop the job instead of writing past the end
        if (threadIdx.x == 0) {
            st->error = 3;
            st->done = 1;
        }
        return;
    }
    __syncthreads();
    for (int t = warp; t < nt; t += kIndexThreads / 32) {
        const int rep = tent[t];
        const uint32_t* e = R.kmer + R.kmer_off[rep];
        const int ne = R.n_kmer[rep];
        for (int i = lane; i < ne; i += 32) {
            const uint32_t v = __ldg(e + i);
            const uint32_t c = v & 0xffffu;
            if (c) {
                const uint32_t at = atomicAdd(&cnt[v >> 16], 1u);
                idx_post[at] = ((uint32_t)t << 16) | c;
                if (post16) post16[at] = (uint16_t)(((uint32_t)t << 6) | min(c, 63u));
            }
        }
    }
}

// Shared memory of k_bfilter_idx, in 32-bit words, every region on a 16-byte
// boundary.  SMEM form: the whole index as 16-bit entries (offsets, and
// postings (tentative << 6 | min(count, 63)), 63 meaning "read the exact count
// from the 32-bit list"); otherwise the 32-bit offsets only.  Then the
// tentatives, and per warp the 16-bit sums (two per word).
constexpr int kIdxGroups = 8;  // groups of 32 k-mer entries held in registers at a time
struct IndexSmem {
    int off_words, post_words, tent_words, acc_words;
    __host__ __device__ IndexSmem(int k, int r_max, long long cap, bool smem_index) {
        const int nb1 = (1 << (2 * k)) + 1;
        off_words = smem_index ? ((nb1 + 7) & ~7) / 2 : (nb1 + 3) & ~3;
        post_words = smem_index ? (int)(((cap + 7) & ~7LL) / 2) : 0;
        tent_words = (r_max + 3) & ~3;
        acc_words = ((r_max + 1) / 2 + 3) & ~3;
    }
    __host__ __device__ int warp_words() const { return acc_words; }
    __host__ __device__ int bytes(int warps) const {
        return 4 * (off_words + post_words + tent_words + warps * warp_words());
    }
};

template <int K, bool SMEM>
__global__ void __launch_bounds__(1024, 1) k_bfilter_idx(
    DevReads R, RoundState* st, const int32_t* __restrict__ remain,
    const int32_t* __restrict__ tent, const uint32_t* __restrict__ idx_off,
    const uint32_t* __restrict__ idx_post, const uint16_t* __restrict__ off16,
    const uint16_t* __restrict__ post16, int r_max, long long cap, Pair* pairs, int seg_cap) {
    constexpr int NB = 1 << (2 * K);
    extern __shared__ __align__(16) uint32_t sm[];
    if (st->done || st->n_tent == 0) return;
    const IndexSmem L(K, r_max, cap, SMEM);
    const int warps = blockDim.x >> 5;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint16_t* s_off16 = reinterpret_cast<uint16_t*>(sm);
    uint32_t* s_off32 = sm;
    uint16_t* s_post16 = reinterpret_cast<uint16_t*>(sm + L.off_words);
    int32_t* s_tent = reinterpret_cast<int32_t*>(sm + L.off_words + L.post_words);
    uint32_t* const acc = sm + L.off_words + L.post_words + L.tent_words + warp * L.warp_words();
    const int nt = st->n_tent;
    const int n = st->n_remain;
    if (SMEM) {
        const int total = (int)idx_off[NB];
        const uint4* g = reinterpret_cast<const uint4*>(post16);
        uint4* d = reinterpret_cast<uint4*>(s_post16);
        for (int i = threadIdx.x; i < (total + 7) >> 3; i += blockDim.x) d[i] = __ldg(g + i);
        const uint4* go = reinterpret_cast<const uint4*>(off16);
        uint4* dof = reinterpret_cast<uint4*>(s_off16);
        for (int i = threadIdx.x; i < (NB + 1 + 7) >> 3; i += blockDim.x) dof[i] = __ldg(go + i);
    } else {
        for (int i = threadIdx.x; i < NB + 1; i += blockDim.x) s_off32[i] = __ldg(idx_off + i);
    }
    for (int i = threadIdx.x; i < nt; i += blockDim.x) s_tent[i] = tent[i];
    for (int i = lane; i < L.acc_words; i += 32) acc[i] = 0u;
    __syncthreads();
    unsigned long long n_pf = 0, bytes = 0;
    unsigned n_wf = 0, n_al = 0;
    const int nwarps = gridDim.x * warps;
    // software pipeline over the warp's candidates: the next candidate's read
    // index and k-mer list position load while this one is summed
    int idx = blockIdx.x * warps + warp;
    int q_nx = idx < n ? remain[idx] : 0;
    const uint32_t* e_nx = R.kmer + (idx < n ? R.kmer_off[q_nx] : 0);
    int ne_nx = idx < n ? R.n_kmer[q_nx] : 0;
    for (; idx < n; idx += nwarps) {
        const int q = q_nx;
        const uint32_t* const e = e_nx;
        const int ne = ne_nx;
        if (idx + nwarps < n) q_nx = remain[idx + nwarps];
        // tentatives before q: the first ntq of the ascending list (all of
        // them for every candidate past the last tentative)
        int lo = 0, hi = nt;
        if (s_tent[nt - 1] < q) lo = nt;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (s_tent[mid] < q) lo = mid + 1;
            else hi = mid;
        }
        const int ntq = lo;
        n_pf += ntq;
        bytes += kCandFixedBytes + 4ull * (unsigned)ne;
        // sum over q's k-mers of min(count in q, count in tentative), per
        // tentative.  The warp takes 32 k-mers at a time, one per lane, and
        // lays their tentative lists end to end (a prefix sum of the list
        // lengths); then every lane takes one position of that concatenation
        // per step and finds the k-mer it belongs to by binary search over the
        // lanes' start positions, so no lane idles while another list is long.
        // Up to kIdxGroups groups of 32 entries load at once.
        for (int c0 = 0; c0 < (ntq > 0 ? ne : 0); c0 += 32 * kIdxGroups) {
            uint32_t vg[kIdxGroups];
#pragma unroll
            for (int g = 0; g < kIdxGroups; g++) {
                const int i = c0 + 32 * g + lane;
                vg[g] = i < ne ? __ldcs(e + i) : 0u;
            }
            if (c0 == 0 && idx + nwarps < n) {
                // the next candidate's list position (its index arrived by now)
                e_nx = R.kmer + R.kmer_off[q_nx];
                ne_nx = R.n_kmer[q_nx];
            }
#pragma unroll
            for (int g = 0; g < kIdxGroups; g++) {
                if (c0 + 32 * g >= ne) break;
                const uint32_t v = vg[g];
                const uint32_t km = v >> 16;
                const uint32_t c = v & 0xffffu;
                const uint32_t s0 = SMEM ? s_off16[km] : s_off32[km];
                const uint32_t sz = c ? (SMEM ? s_off16[km + 1] : s_off32[km + 1]) - s0 : 0u;
                uint32_t incl = sz;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const uint32_t o = __shfl_up_sync(kFull, incl, d);
                    if (lane >= d) incl += o;
                }
                const uint32_t excl = incl - sz;
                const uint32_t total = __shfl_sync(kFull, incl, 31);
                const uint32_t jbase = s0 - excl;  // posting index = jbase + position
                for (uint32_t base = 0; base < total; base += 32) {
                    const uint32_t p = base + lane;
                    // the last lane whose list starts at or before p owns p
                    int o = 0;
#pragma unroll
                    for (int step = 16; step >= 1; step >>= 1) {
                        const uint32_t x = __shfl_sync(kFull, excl, o + step);
                        if (x <= p) o += step;
                    }
                    const uint32_t j = __shfl_sync(kFull, jbase, o) + p;
                    const uint32_t co = __shfl_sync(kFull, c, o);
                    if (p < total) {
                        uint32_t t, ct;
                        if (SMEM) {
                            const uint32_t pp = s_post16[j];
                            t = pp >> 6;
                            ct = pp & 63u;
                            if (ct == 63u) ct = __ldg(idx_post + j) & 0xffffu;
                        } else {
                            const uint32_t pp = __ldg(idx_post + j);
                            t = pp >> 16;
                            ct = pp & 0xffffu;
                        }
                        // 16-bit halves cannot carry: a sum is at most the
                        // candidate's k-mer count, below 65536
                        if (t < (uint32_t)ntq)
                            atomicAdd(&acc[t >> 1], min(ct, co) << ((t & 1u) << 4));
                    }
                }
            }
        }
        if (!(ntq > 0 && ne > 0) && idx + nwarps < n) {
            e_nx = R.kmer + R.kmer_off[q_nx];
            ne_nx = R.n_kmer[q_nx];
        }
        if (ntq == 0) continue;
        __syncwarp();
        // the tentatives whose sum reaches the cutoff pass the word filter;
        // the composition bound (kernel_preFilter, func.cu:738-754) decides
        // the rest.  The sums are cleared on the way.
        const int cw = R.cut_word[q];
        uint4* a4 = reinterpret_cast<uint4*>(acc);
        const int w4 = (ntq + 7) >> 3;
        for (int i = lane; i < w4; i += 32) {
            const uint4 a = a4[i];
            a4[i] = make_uint4(0u, 0u, 0u, 0u);
            const uint32_t w[4] = {a.x, a.y, a.z, a.w};
#pragma unroll
            for (int h = 0; h < 8; h++) {
                const int t = 8 * i + h;
                const int s = (int)((w[h >> 1] >> ((h & 1) << 4)) & 0xffffu);
                if (t < ntq && !(s < cw)) {
                    n_wf++;
                    const int rep = s_tent[t];
                    if (prefilter_pass(R.comp[rep], R.comp[q], R.cut_base[q] - R.strict)) {
                        push_pair(st, pairs, seg_cap, R, rep, q, kBandMaxW);
                        n_al++;
                    }
                }
            }
        }
        __syncwarp();
    }
    // n_pf and bytes are the same in every lane; n_wf and n_al are per lane
    n_wf = (unsigned)warp_sum_i((int)n_wf);
    n_al = (unsigned)warp_sum_i((int)n_al);
    if (lane == 0) {
        if (n_pf) atomicAdd(&st->cnt_prefilter, n_pf);
        if (n_wf) atomicAdd(&st->cnt_word, (unsigned long long)n_wf);
        if (n_al) atomicAdd(&st->cnt_aligned, (unsigned long long)n_al);
        if (bytes) atomicAdd(&st->filter_bytes, bytes);
    }
}

// ---- word filter by tentative masks (short reads, sparse k-mer spaces) ----
//
// Per pass, for every k-mer m a row of R_max bits, bit t set iff tentative t
// holds m with a non-zero count (k_bmask; 2 MB for k = 7 and R_max 1024, held
// in L2).  A group of lanes per candidate (eight lanes of 16 bytes hold a row
// of 1,024 tentatives; four candidates per warp) copies the rows of the
// candidate's k-mers into shared memory and counts per tentative the rows
// that have its bit:
//     D1 = sum over k-mers of [c_t >= 1][c_q >= 1],
// in bit-sliced counters (plane b holds bit b of 32 tentatives' counts) that
// carry-save adders fill.  Since min(c_t, c_q) = [both >= 1] + (min - 1),
//     D1 <= S <= D1 + min(E_t, E_q),   E = sum over k-mers of (count - 1),
// so D1 >= cutoff passes a pair and D1 + min(E_t, E_q) < cutoff rejects it;
// the pairs between go to k_bexact_t, which forms S itself.  Per pair the
// kernel reads one bit per candidate k-mer and spends about three logic
// instructions per 32 pairs and k-mer, where the index form takes a warp
// step per posting of every shared k-mer.  A count never exceeds the
// candidate's k-mer entries: eight planes hold it where every read has at
// most kMaskEntries8 entries, ten up to kMaskMaxEntries (the form's limit).

constexpr int kMaskThreads = 256;

// One warp per tentative: sets the tentative's bit in the rows of its k-mers
// (the rows were zeroed before) and writes its excess E_t.
__global__ void __launch_bounds__(256) k_bmask(DevReads R, RoundState* st,
                                               const int32_t* __restrict__ tent, uint32_t* tmask,
                                               int32_t* tex, int rwq) {
    if (st->done || st->n_tent == 0) return;
    const int nt = st->n_tent;
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const size_t row_words = 4 * (size_t)rwq;
    for (int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < nt; t += nw) {
        const int rep = tent[t];
        const uint32_t* e = R.kmer + R.kmer_off[rep];
        const int ne = R.n_kmer[rep];
        const uint32_t bit = 1u << (t & 31);
        int ex = 0;
        for (int i = lane; i < ne; i += 32) {
            const uint32_t v = __ldg(e + i);
            const uint32_t c = v & 0xffffu;
            if (c) {
                atomicOr(tmask + (v >> 16) * row_words + (t >> 5), bit);
                ex += (int)c - 1;
            }
        }
        ex = warp_sum_i(ex);
        if (lane == 0) tex[t] = ex;
    }
}

// p += w0 + .. + w7, bit-sliced (NP planes, counts below 2^NP), in two parts:
// a Harley-Seal tree of carry-save adders into the planes of weight 1, 2 and
// 4 that returns the carry of weight 8, and bs_carry, which adds a carry
// into the planes from `from` up.  Two trees' carries meet in one more adder
// first (bs_pair8), so the ripple runs once per 16 words.
template <int NP>
__device__ __forceinline__ uint32_t bs_tree8(uint32_t (&p)[NP], uint32_t w0, uint32_t w1,
                                             uint32_t w2, uint32_t w3, uint32_t w4, uint32_t w5,
                                             uint32_t w6, uint32_t w7) {
    uint32_t t1, t2, t3, t4, f1, f2, e8;
    csa(p[0], t1, p[0], w0, w1);
    csa(p[0], t2, p[0], w2, w3);
    csa(p[1], f1, p[1], t1, t2);
    csa(p[0], t3, p[0], w4, w5);
    csa(p[0], t4, p[0], w6, w7);
    csa(p[1], f2, p[1], t3, t4);
    csa(p[2], e8, p[2], f1, f2);
    return e8;
}
template <int NP>
__device__ __forceinline__ void bs_carry(uint32_t (&p)[NP], int from, uint32_t c) {
#pragma unroll
    for (int b = 0; b < NP; b++) {
        if (b < from) continue;
        const uint32_t t = p[b] & c;
        p[b] ^= c;
        c = t;
    }
}
// Two weight-8 carries: one adder into plane 3, its weight-16 carry rippled.
template <int NP>
__device__ __forceinline__ void bs_pair8(uint32_t (&p)[NP], uint32_t a8, uint32_t b8) {
    uint32_t c16;
    csa(p[3], c16, p[3], a8, b8);
    bs_carry<NP>(p, 4, c16);
}

// Bits of the counts >= v.
template <int NP>
__device__ __forceinline__ uint32_t bs_ge(const uint32_t (&p)[NP], int v) {
    if (v <= 0) return 0xffffffffu;
    if (v > (1 << NP) - 1) return 0u;
    uint32_t gt = 0, eq = 0xffffffffu;
#pragma unroll
    for (int b = NP - 1; b >= 0; b--) {
        const uint32_t vb = ((v >> b) & 1) ? 0xffffffffu : 0u;
        gt |= eq & p[b] & ~vb;
        eq &= ~(p[b] ^ vb);
    }
    return gt | eq;
}

template <int NP>
__device__ __forceinline__ int bs_get(const uint32_t (&p)[NP], int bit) {
    int v = 0;
#pragma unroll
    for (int b = 0; b < NP; b++) v |= (int)((p[b] >> bit) & 1u) << b;
    return v;
}

struct MaskCounts {
    unsigned long long n_pf = 0, bytes = 0;
    unsigned n_wf = 0, n_al = 0;
};

// Rows stream through shared memory with cp.async, kMaskStages steps deep:
// each lane copies its own 16-byte words and reads back only those, so no
// warp barrier is needed (the kernel is bound by L2 latency, and the copies
// in flight hold no registers).
constexpr int kMaskStages = 3;
constexpr int kMaskStepBytes = 8 * 32 * 16;  // one step: 8 words of 16 bytes per lane

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, bool fill) {
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(gmem),
                 "r"(fill ? 16 : 0));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

// Rows of 16-byte words: lane (g, x) of a warp, g = lane / LPR, x = lane %
// LPR, works for candidate g of the warp's 32 / LPR consecutive candidates
// (consecutive in the remain list, so of similar length) and holds the counts
// of word x of the rows (tentatives 128 x .. 128 x + 127).  Each step a group
// copies the rows of 8 of its candidate's k-mers; a step's entries load two
// issues before its copies, and the copies kMaskStages - 1 steps before their
// counts.
template <int LPR, int NP>
__device__ __forceinline__ void mask_candidates(const DevReads& R, RoundState* st,
                                                const int32_t* __restrict__ remain,
                                                const int32_t* s_tent, uint4* stage, int nt,
                                                int n, const uint4* __restrict__ tm4, int rwq,
                                                const int32_t* __restrict__ tex, Pair* pairs,
                                                int seg_cap, Pair* amb, int amb_cap,
                                                MaskCounts& mc) {
    constexpr int G = 32 / LPR;   // candidates per warp
    constexpr int EPL = 8 / LPR;  // entries a lane loads per step
    const int lane = threadIdx.x & 31;
    const int g = lane / LPR, x = lane % LPR;
    const bool xin = x < ((nt + 127) >> 7);
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int stride = nwarps * G;
    // software pipeline over the warp's candidate sets: the read index of the
    // set after next and the list position of the next load while this set
    // is counted
    auto read_at = [&](int i) { return i < n ? remain[i] : -1; };
    int q1 = read_at(wid * G + g);
    int q2 = read_at(wid * G + stride + g);
    int64_t off1 = q1 >= 0 ? R.kmer_off[q1] : 0;
    int nk1 = q1 >= 0 ? R.n_kmer[q1] : 0;
    for (int base = wid * G; base < n; base += stride) {
        const int q = q1;
        const int64_t off = off1;
        const int nk = nk1;
        q1 = q2;
        q2 = read_at(base + 2 * stride + g);
        // tentatives before q: the first ntq of the ascending list
        int ntq = 0;
        if (q >= 0) {
            int lo = 0, hi = nt;
            if (s_tent[nt - 1] < q) lo = nt;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (s_tent[mid] < q) lo = mid + 1;
                else hi = mid;
            }
            ntq = lo;
        }
        const int ne = ntq > 0 ? nk : 0;
        const uint32_t* e = R.kmer + (ntq > 0 ? off : 0);
        if (x == 0) {
            mc.n_pf += ntq;
            if (ntq > 0) mc.bytes += kCandFixedBytes + 4ull * (unsigned)ne;
        }
        const int nsteps = __reduce_max_sync(kFull, (ne + 7) >> 3);
        if (nsteps == 0) {
            off1 = q1 >= 0 ? R.kmer_off[q1] : 0;
            nk1 = q1 >= 0 ? R.n_kmer[q1] : 0;
            continue;
        }
        // entries [8 j + EPL x, + EPL) of the candidate (the lists are padded
        // to 16 bytes, with slack after the last: whole vectors load).  They
        // stream from HBM, so they load two issues ahead of their copies.
        auto load_raw = [&](int j, uint32_t (&en)[EPL]) {
            const int i0 = 8 * j + EPL * x;
#pragma unroll
            for (int k = 0; k < EPL; k++) en[k] = 0u;
            if (i0 < ne) {
                if constexpr (EPL == 1) {
                    en[0] = __ldcs(e + i0);
                } else if constexpr (EPL == 2) {
                    const uint2 v = __ldcs(reinterpret_cast<const uint2*>(e + i0));
                    en[0] = v.x, en[1] = v.y;
                } else {
#pragma unroll
                    for (int k = 0; k < EPL; k += 4) {
                        const uint4 v = __ldcs(reinterpret_cast<const uint4*>(e + i0 + k));
                        en[k] = v.x, en[k + 1] = v.y, en[k + 2] = v.z, en[k + 3] = v.w;
                    }
                }
            }
        };
        int ex = 0;
        // stage buffers in turn: copies of step j go to `wr`, counts of step
        // s read `rd`
        uint4* const st0 = stage + lane;
        constexpr int SB = kMaskStepBytes / 16;
        int wr = 0, rd = 0;
        // step j: slot u of stage wr gets word x of the row of entry 8 j + u
        // (a row index of -1: no row, count 0 or past the list)
        auto issue = [&](int j, const uint32_t (&en)[EPL]) {
            int rb[EPL];
#pragma unroll
            for (int k = 0; k < EPL; k++) {
                const int c = 8 * j + EPL * x + k < ne ? (int)(en[k] & 0xffffu) : 0;
                ex += c > 0 ? c - 1 : 0;
                rb[k] = c > 0 ? (int)(en[k] >> 16) * rwq : -1;
            }
            uint4* dst = st0 + wr * SB;
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int r = EPL == 8 ? rb[u % EPL]
                                       : __shfl_sync(kFull, rb[u % EPL], g * LPR + u / EPL);
                const bool ok = xin && r >= 0;
                cp_async16(dst + 32 * u, tm4 + (ok ? r + x : 0), ok);
            }
            wr = wr == kMaskStages - 1 ? 0 : wr + 1;
        };
        uint32_t P[4][NP];
#pragma unroll
        for (int w = 0; w < 4; w++)
#pragma unroll
            for (int b = 0; b < NP; b++) P[w][b] = 0u;
        uint32_t c8[4] = {0u, 0u, 0u, 0u};  // weight-8 carries of an odd step
        uint32_t en0[EPL], en1[EPL];        // entries of the next two steps to issue
        load_raw(0, en0);
        load_raw(1, en1);
        int nexti = 0;  // next step to issue
        auto issue_next = [&]() {
            issue(nexti, en0);
#pragma unroll
            for (int k = 0; k < EPL; k++) en0[k] = en1[k];
            load_raw(nexti + 2, en1);
            nexti++;
        };
#pragma unroll
        for (int j = 0; j < kMaskStages - 1; j++) {
            if (j < nsteps) issue_next();
            cp_async_commit();
        }
        off1 = q1 >= 0 ? R.kmer_off[q1] : 0;
        nk1 = q1 >= 0 ? R.n_kmer[q1] : 0;
        for (int s = 0; s < nsteps; s++) {
            if (s + kMaskStages - 1 < nsteps) issue_next();
            cp_async_commit();
            cp_async_wait<kMaskStages - 1>();  // this lane's copies of step s
            const uint4* src = st0 + rd * SB;
            rd = rd == kMaskStages - 1 ? 0 : rd + 1;
            uint4 w[8];
#pragma unroll
            for (int u = 0; u < 8; u++) w[u] = src[32 * u];
            const uint32_t e0 = bs_tree8<NP>(P[0], w[0].x, w[1].x, w[2].x, w[3].x, w[4].x, w[5].x, w[6].x, w[7].x);
            const uint32_t e1 = bs_tree8<NP>(P[1], w[0].y, w[1].y, w[2].y, w[3].y, w[4].y, w[5].y, w[6].y, w[7].y);
            const uint32_t e2 = bs_tree8<NP>(P[2], w[0].z, w[1].z, w[2].z, w[3].z, w[4].z, w[5].z, w[6].z, w[7].z);
            const uint32_t e3 = bs_tree8<NP>(P[3], w[0].w, w[1].w, w[2].w, w[3].w, w[4].w, w[5].w, w[6].w, w[7].w);
            if (s & 1) {
                bs_pair8<NP>(P[0], c8[0], e0);
                bs_pair8<NP>(P[1], c8[1], e1);
                bs_pair8<NP>(P[2], c8[2], e2);
                bs_pair8<NP>(P[3], c8[3], e3);
            } else {
                c8[0] = e0, c8[1] = e1, c8[2] = e2, c8[3] = e3;
            }
        }
        if (nsteps & 1) {
#pragma unroll
            for (int w = 0; w < 4; w++) bs_carry<NP>(P[w], 3, c8[w]);
        }
        // E_q over the group's lanes
#pragma unroll
        for (int off = 1; off < LPR; off <<= 1) ex += __shfl_xor_sync(kFull, ex, off);
        if (ntq == 0 || !xin) continue;
        const int cw = R.cut_word[q];
        // counts >= v need a bit at or above plane floor(log2 v): most words
        // have none and skip the comparisons
        const int vlo = cw - ex;
        const int lb = vlo > 0 ? 31 - __clz(vlo) : 0;
        int4 cq = make_int4(0, 0, 0, 0);
        int cbq = 0;
        bool have_cq = false;
#pragma unroll
        for (int w = 0; w < 4; w++) {
            const int t0 = 32 * (4 * x + w);
            if (t0 >= ntq) break;
            const uint32_t valid = ntq - t0 >= 32 ? 0xffffffffu : (1u << (ntq - t0)) - 1u;
            uint32_t hiw = 0u;
#pragma unroll
            for (int b = 0; b < NP; b++)
                if (b >= lb) hiw |= P[w][b];
            if (vlo > (1 << NP) - 1 || !((vlo <= 0 ? 0xffffffffu : hiw) & valid)) continue;
            uint32_t pass = bs_ge<NP>(P[w], cw) & valid;
            uint32_t open = bs_ge<NP>(P[w], vlo) & valid & ~pass;
            if (!(pass | open)) continue;
            if (!have_cq) {
                cq = R.comp[q];
                cbq = R.cut_base[q] - R.strict;
                have_cq = true;
            }
            while (pass) {
                const int t = t0 + __ffs(pass) - 1;
                pass &= pass - 1;
                mc.n_wf++;
                const int rep = s_tent[t];
                // the composition bound (kernel_preFilter, func.cu:738-754)
                if (prefilter_pass(R.comp[rep], cq, cbq)) {
                    push_pair(st, pairs, seg_cap, R, rep, q, kBandMaxW);
                    mc.n_al++;
                }
            }
            while (open) {
                const int b = __ffs(open) - 1;
                open &= open - 1;
                const int t = t0 + b;
                if (bs_get<NP>(P[w], b) + min(tex[t], ex) < cw) continue;
                mc.n_wf++;
                const int rep = s_tent[t];
                if (prefilter_pass(R.comp[rep], cq, cbq)) {
                    const int slot = atomicAdd(&st->n_amb, 1);
                    if (slot < amb_cap) amb[slot] = Pair{rep, q};
                    else st->pair_overflow = 1;
                }
            }
        }
    }
    cp_async_wait<0>();
}

constexpr int kMaskSmem = (kMaskThreads / 32) * kMaskStages * kMaskStepBytes;

template <int NP>
__global__ void __launch_bounds__(kMaskThreads, 2) k_bfilter_mask(
    DevReads R, RoundState* st, const int32_t* __restrict__ remain,
    const int32_t* __restrict__ tent, const uint4* __restrict__ tm4, int rwq,
    const int32_t* __restrict__ tex, Pair* pairs, int seg_cap, Pair* amb, int amb_cap) {
    __shared__ int32_t s_tent[kMaxBatch];
    extern __shared__ __align__(16) uint4 mstage[];
    if (st->done || st->n_tent == 0) return;
    const int nt = st->n_tent;
    const int n = st->n_remain;
    for (int i = threadIdx.x; i < nt; i += blockDim.x) s_tent[i] = tent[i];
    __syncthreads();
    uint4* stage = mstage + (threadIdx.x >> 5) * kMaskStages * (kMaskStepBytes / 16);
    MaskCounts mc;
    const int quads = (nt + 127) >> 7;  // 16-byte words of the pass's rows
    if (quads > 4)
        mask_candidates<8, NP>(R, st, remain, s_tent, stage, nt, n, tm4, rwq, tex, pairs, seg_cap,
                           amb, amb_cap, mc);
    else if (quads > 2)
        mask_candidates<4, NP>(R, st, remain, s_tent, stage, nt, n, tm4, rwq, tex, pairs, seg_cap,
                           amb, amb_cap, mc);
    else if (quads > 1)
        mask_candidates<2, NP>(R, st, remain, s_tent, stage, nt, n, tm4, rwq, tex, pairs, seg_cap,
                           amb, amb_cap, mc);
    else
        mask_candidates<1, NP>(R, st, remain, s_tent, stage, nt, n, tm4, rwq, tex, pairs, seg_cap,
                           amb, amb_cap, mc);
    const unsigned n_wf = (unsigned)warp_sum_i((int)mc.n_wf);
    const unsigned n_al = (unsigned)warp_sum_i((int)mc.n_al);
    mc.n_pf = warp_sum_ull(mc.n_pf);
    mc.bytes = warp_sum_ull(mc.bytes);
    if ((threadIdx.x & 31) == 0) {
        if (mc.n_pf) atomicAdd(&st->cnt_prefilter, mc.n_pf);
        if (n_wf) atomicAdd(&st->cnt_word, (unsigned long long)n_wf);
        if (n_al) atomicAdd(&st->cnt_aligned, (unsigned long long)n_al);
        if (mc.bytes) atomicAdd(&st->filter_bytes, mc.bytes);
    }
}

// Survival of the tentatives in greedy order (one warp): a tentative survives
// iff no surviving earlier tentative accepted it.  Only rows with a bit can
// claim anything, so only those are visited, in increasing order.
__global__ void k_bsurvive(RoundState* st, const int32_t* __restrict__ tent,
                           const uint32_t* __restrict__ tt, const uint32_t* __restrict__ ttrow,
                           uint32_t* survive, int32_t* cluster) {
    if (st->done || st->n_tent == 0) return;
    if (st->pair_overflow || st->acc_overflow) return;
    const int nt = st->n_tent;
    const int lane = threadIdx.x;
    uint32_t claimed = 0;  // bits [32*lane, 32*lane+32) of the claimed set
    const uint32_t rows = ttrow[lane];
    for (int w = 0; w < kTTWords; w++) {
        uint32_t rw = __shfl_sync(kFull, rows, w);
        while (rw) {
            // the next eight rows with bits: their words are loaded together
            // (they do not depend on the claims), then applied in order
            constexpr int P = 8;
            int hs[P];
            uint32_t v[P];
#pragma unroll
            for (int j = 0; j < P; j++) {
                hs[j] = rw ? w * 32 + __ffs(rw) - 1 : -1;
                rw &= rw - 1u;
            }
#pragma unroll
            for (int j = 0; j < P; j++) v[j] = hs[j] >= 0 ? tt[hs[j] * kTTWords + lane] : 0u;
#pragma unroll
            for (int j = 0; j < P; j++) {
                if (hs[j] < 0) break;  // warp-uniform
                const uint32_t cw = __shfl_sync(kFull, claimed, hs[j] >> 5);
                if (!((cw >> (hs[j] & 31)) & 1u)) claimed |= v[j];
            }
        }
    }
    uint32_t valid;
    const int lo = lane * 32;
    valid = nt >= lo + 32 ? 0xffffffffu : (nt > lo ? ((1u << (nt - lo)) - 1u) : 0u);
    const uint32_t surv = ~claimed & valid;
    survive[lane] = surv;
    uint32_t s = surv;
    while (s) {
        const int i = lo + __ffs(s) - 1;
        s &= s - 1;
        cluster[tent[i]] = tent[i];
    }
    const int count = warp_sum_i(__popc(surv));
    if (lane == 0) {
        st->survivors = count;
        st->rounds += count;
    }
}

__global__ void k_bclaim(RoundState* st, const Pair* __restrict__ acc,
                         const uint32_t* __restrict__ tidx, const uint32_t* __restrict__ survive,
                         uint32_t* best) {
    if (st->done || st->n_tent == 0 || st->pair_overflow || st->acc_overflow) return;
    const int na = st->n_acc;
    const uint32_t pass = (uint32_t)st->pass;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < na; k += gridDim.x * blockDim.x) {
        const Pair p = acc[k];
        const int i = tidx[p.rep] & 0xfff;
        if ((survive[i >> 5] >> (i & 31)) & 1u) atomicMax(&best[p.cand], (pass << 12) | (4095u - i));
    }
}

__global__ void k_bapply(RoundState* st, const Pair* __restrict__ acc,
                         const uint32_t* __restrict__ tidx, const uint32_t* __restrict__ best,
                         int32_t* cluster) {
    if (st->done || st->n_tent == 0 || st->pair_overflow || st->acc_overflow) return;
    const int na = st->n_acc;
    const uint32_t pass = (uint32_t)st->pass;
    unsigned applied = 0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < na; k += gridDim.x * blockDim.x) {
        const Pair p = acc[k];
        const int i = tidx[p.rep] & 0xfff;
        if (best[p.cand] == ((pass << 12) | (4095u - i))) {
            cluster[p.cand] = p.rep;
            applied++;
        }
    }
    applied = __reduce_add_sync(kFull, applied);
    if ((threadIdx.x & 31) == 0 && applied) {
        atomicAdd(&st->absorbed, (int)applied);
        atomicAdd(&st->cnt_accepted, (unsigned long long)applied);
    }
}

__global__ void k_badvance(RoundState* st, const int32_t* __restrict__ tent, int* align_work,
                           int seg_cap, int acc_cap, int amb_cap, int drop) {
    if (st->done) return;
    st->passes += 1;
    st->pass += 1;
    if (st->error) {
        st->done = 1;
        return;
    }
    if (st->pair_overflow || st->acc_overflow) {
        // queues too small for this many tentatives: the pass changed nothing
        // (the compaction copied the remain list unchanged); redo it with fewer
        if (st->R == 1) {
            st->error = 2;
            st->done = 1;
            return;
        }
        st->R = max(1, st->R / 8);
        st->n_next = 0;
        return;
    }
    const int nt = st->n_tent;
    if (nt > 0) st->cursor = tent[nt - 1] + 1;
    const int surv = max(1, st->survivors);
    // a pass that queued fewer pairs than the device keeps in flight ran on
    // the latency of its longest pairs: grow R faster
    int queued = 0, fullest = 0;
    for (int c = 0; c < kAlignClasses; c++) {
        queued += st->n_pairs[c];
        fullest = max(fullest, st->n_pairs[c]);
    }
    if (st->absorbed > kAbsorbHigh * surv) {
        st->R = max(1, st->R / 2);
    } else {
        // (drop mode has no filter pass to share between tentatives: R grows
        // only while the passes are too small to fill the device, since every
        // tentative that an earlier one absorbs wastes its alignments)
        long long r = (long long)st->R * (queued < kFewPairs ? 8 : (drop ? 1 : 2));
        // queue use grows with the tentatives: keep the fullest alignment
        // queue and the accept list under 3/4 of their capacity (an overflow
        // costs a redone pass; without the cap, drop mode, where every
        // candidate pairs with every tentative, alternates between overflow
        // and a small R)
        if (nt > 0 && fullest > 0) r = min(r, (long long)nt * (3ll * seg_cap / 4) / fullest);
        if (nt > 0 && st->n_acc > 0) r = min(r, (long long)nt * (3ll * acc_cap / 4) / st->n_acc);
        // and the bitmap filter's queue of open pairs
        if (nt > 0 && amb_cap > 0 && st->n_amb > 0)
            r = min(r, (long long)nt * (3ll * amb_cap / 4) / st->n_amb);
        st->R = (int)max(1ll, min((long long)st->R_max, r));
    }
    const int n = st->n_next;
    st->n_next = 0;
    st->next_min = 0x7fffffff;
    if (n == 0) {
        st->done = 1;
        return;
    }
    st->n_remain = n;
    if (st->pass_limit > 0 && st->passes >= st->pass_limit) st->done = 1;  // timing runs
}

__global__ void k_init(RoundState* st, int32_t* cluster, int32_t* remain, uint32_t* tidx,
                       uint32_t* best, int n, int batched, int r_max, int pass_limit,
                       int* align_work) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        if (batched) {
            cluster[i] = -1;
            remain[i] = i;
            tidx[i] = 0xffffffffu;
            best[i] = 0u;
        } else {
            cluster[i] = i == 0 ? 0 : -1;
            if (i > 0) remain[i - 1] = i;
        }
    }
    if (i == 0) {
        RoundState s = {};
        s.rep = 0;
        s.n_remain = batched ? n : n - 1;
        s.next_min = 0x7fffffff;
        s.done = n <= 0 ? 1 : 0;
        s.pass = 1;
        s.R = 1;
        s.R_max = r_max;
        s.pass_limit = pass_limit;
        *st = s;
        for (int c = 0; c <= kSingleWorkSlot; c++) align_work[c] = 0;
    }
}

// Resume from a checkpoint: cluster[] (already on the device) is the state of
// an unfinished clustering -- every read either unclustered (-1) or joined to
// a representative taken earlier -- which is all the state the reference's
// loop carries between rounds (cluster[] and the next representative, the
// smallest unclustered read; cuda-version/func.cu:1001-1066).  Three steps:
// a fresh round state, the remain list of the unclustered reads (any order:
// every consumer of the list is order-independent) with their smallest index,
// then the next representative (plain) or the tentative cursor (batched).
__global__ void k_resume_state(RoundState* st, int r_max, int pass_limit, int* align_work) {
    RoundState s = {};
    s.rep = -1;
    s.next_min = 0x7fffffff;
    s.pass = 1;
    s.R = 1;
    s.R_max = r_max;
    s.pass_limit = pass_limit;
    *st = s;
    for (int c = 0; c <= kSingleWorkSlot; c++) align_work[c] = 0;
}

__global__ void k_resume_scan(RoundState* st, const int32_t* __restrict__ cluster,
                              int32_t* remain, uint32_t* tidx, uint32_t* best, int n,
                              int batched) {
    const int lane = threadIdx.x & 31;
    const int stride = gridDim.x * blockDim.x;
    for (int base = blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < n; base += stride) {
        const int i = base + lane;
        const bool un = i < n && cluster[i] == -1;
        if (batched && i < n) {
            tidx[i] = 0xffffffffu;
            best[i] = 0u;
        }
        const unsigned m = __ballot_sync(kFull, un);
        if (!m) continue;
        int pos = 0;
        if (lane == 0) {
            pos = atomicAdd(&st->n_remain, __popc(m));
            atomicMin(&st->next_min, base + __ffs(m) - 1);
        }
        pos = __shfl_sync(kFull, pos, 0);
        if (un) remain[pos + __popc(m & ((1u << lane) - 1u))] = i;
    }
}

__global__ void k_resume_start(RoundState* st, int32_t* cluster, int batched) {
    if (st->n_remain == 0) {
        st->done = 1;
        return;
    }
    const int first = st->next_min;
    st->next_min = 0x7fffffff;
    if (batched) {
        st->cursor = first;
    } else {
        // the next round's representative; it stays in the remain list, which
        // the plain filter skips, as after every compaction
        cluster[first] = first;
        st->rep = first;
    }
}

// ---------------------------------------------------------------- launchers

template <class KernelT>
int grid_for(KernelT kernel, int threads, int smem, int cap_per_sm) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
    if (per_sm < 1) per_sm = 1;
    if (per_sm > cap_per_sm) per_sm = cap_per_sm;
    return num_sms() * per_sm;
}

// The job's block shape: a grid of at most `blocks` CTAs per SM (0: the full
// grid, every CTA that fits).  The kernels loop over their work, so any grid
// size gives the same result.
int shaped(int grid, int blocks) {
    return blocks > 0 ? min(grid, num_sms() * blocks) : grid;
}

// tent: null for a plain round; the batched form's tentatives otherwise (the
// kernel then runs only in a pass with a single tentative).
template <int K, bool DROP>
void launch_filter_t(const DevReads& R, RoundBuffers& B, const int32_t* remain, cudaStream_t s,
                     const int32_t* tent = nullptr) {
    const int smem = DROP ? 0 : (1 << (2 * K)) * 2;
    static int grid = 0;
    if (!grid) {
        if (smem > 0)
            cudaFuncSetAttribute(k_filter<K, DROP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 smem);
        grid = grid_for(k_filter<K, DROP>, kFilterThreads, smem, 8);
    }
    k_filter<K, DROP><<<shaped(grid, R.filter_blocks), kFilterThreads, smem, s>>>(R, B.st, remain, B.pairs, B.seg_cap,
                                                         tent);
}

template <int K>
void launch_bfilter_tab_t(const DevReads& R, RoundBuffers& B, const int32_t* remain,
                          cudaStream_t s) {
    // passes with one tentative (the first passes of adaptive R) stream the
    // candidates once against one table: the plain kernel does that at HBM
    // speed, the grouped-table kernel skips them
    launch_filter_t<K, false>(R, B, remain, s, B.tent);
    constexpr int smem = TabGroup<K>::smem;
    static int grid = 0;
    if (!grid) {
        cudaFuncSetAttribute(k_bfilter_tab<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        grid = grid_for(k_bfilter_tab<K>, kTabThreads, smem, 2);
    }
    k_bfilter_tab<K><<<shaped(grid, R.filter_blocks), kTabThreads, smem, s>>>(R, B.st, remain, B.tent, B.pairs, B.seg_cap);
}

template <int K, bool DROP>
void launch_bfilter_t(const DevReads& R, RoundBuffers& B, const int32_t* remain, cudaStream_t s) {
    if constexpr (!DROP) {
        launch_bfilter_tab_t<K>(R, B, remain, s);
    } else {
        static int grid = 0;
        if (!grid) grid = grid_for(k_bprefilter, kFilterThreads, 0, 8);
        k_bprefilter<<<shaped(grid, R.filter_blocks), kFilterThreads, 0, s>>>(R, B.st, remain, B.tent, B.pairs, B.seg_cap);
    }
}

template <int K>
void launch_bfilter_idx_t(const DevReads& R, RoundBuffers& B, const int32_t* remain,
                          cudaStream_t s) {
    const bool in_smem = B.idx_post16 != nullptr;
    const int threads = in_smem ? 1024 : 256;
    const int ismem = (1 << (2 * K)) * 4;
    const int fsmem = IndexSmem(K, B.r_max, B.idx_cap, in_smem).bytes(threads / 32);
    static bool attr = false;
    if (!attr) {
        // the device's largest size, set once: jobs of one process may run
        // concurrently with different index sizes
        int dev = 0, optin = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaFuncSetAttribute(k_bindex<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, ismem);
        cudaFuncSetAttribute(k_bfilter_idx<K, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             optin);
        cudaFuncSetAttribute(k_bfilter_idx<K, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             optin);
        attr = true;
    }
    k_bindex<K><<<1, kIndexThreads, ismem, s>>>(R, B.st, B.tent, B.idx_off, B.idx_post,
                                                B.idx_off16, B.idx_post16, (long long)B.idx_cap);
    if (in_smem) {
        const int grid = grid_for(k_bfilter_idx<K, true>, threads, fsmem, 2);
        k_bfilter_idx<K, true><<<shaped(grid, R.filter_blocks), threads, fsmem, s>>>(
            R, B.st, remain, B.tent, B.idx_off, B.idx_post, B.idx_off16, B.idx_post16, B.r_max,
            (long long)B.idx_cap, B.pairs, B.seg_cap);
    } else {
        const int grid = grid_for(k_bfilter_idx<K, false>, threads, fsmem, 8);
        k_bfilter_idx<K, false><<<shaped(grid, R.filter_blocks), threads, fsmem, s>>>(
            R, B.st, remain, B.tent, B.idx_off, B.idx_post, nullptr, nullptr, B.r_max,
            (long long)B.idx_cap, B.pairs, B.seg_cap);
    }
}

// The exact sums of the open pairs: the queue sorted by tentative, then one
// table per run.
template <int K>
void launch_exact_t(const DevReads& R, RoundBuffers& B, cudaStream_t s) {
    constexpr int xsmem = (1 << (2 * K)) * 2;
    static int grid = 0;
    if (!grid) {
        cudaFuncSetAttribute(k_bexact_t<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, xsmem);
        grid = grid_for(k_bexact_t<K>, kAmbThreads, xsmem, 8);
    }
    const int ga = num_sms() * 2;
    k_amb_count<<<ga, kAmbThreads, 0, s>>>(B.st, B.amb, B.amb_cap, B.tidx, B.amb_idx);
    k_amb_scan<<<1, 1024, 0, s>>>(B.st, B.amb_cap, B.amb_idx);
    k_amb_place<<<ga, kAmbThreads, 0, s>>>(B.st, B.amb, B.amb_cap, B.tidx, B.amb_idx, B.amb2);
    k_bexact_t<K><<<shaped(grid, R.filter_blocks), kAmbThreads, xsmem, s>>>(
        R, B.st, B.amb2, B.amb_idx, B.amb_cap, B.tent, B.pairs, B.seg_cap);
}

template <int K>
void launch_bfilter_bits_t(const DevReads& R, RoundBuffers& B, const int32_t* remain,
                           cudaStream_t s) {
    // passes with one tentative (the first passes of adaptive R) go to the
    // plain kernel, which streams the candidates against one table
    launch_filter_t<K, false>(R, B, remain, s, B.tent);
    constexpr int bsmem = (int)BitsSmem<K>::bytes;
    constexpr int bthreads = BitsSmem<K>::THREADS;
    static int grid = 0;
    if (!grid) {
        cudaFuncSetAttribute(k_bfilter_bits<K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             bsmem);
        grid = grid_for(k_bfilter_bits<K>, bthreads, bsmem, 2);
    }
    k_bfilter_bits<K><<<shaped(grid, R.filter_blocks), bthreads, bsmem, s>>>(
        R, B.st, remain, B.tent, B.pairs, B.seg_cap, B.amb, B.amb_cap);
    launch_exact_t<K>(R, B, s);
}

template <int K>
void launch_bfilter_mask_t(const DevReads& R, RoundBuffers& B, const int32_t* remain,
                           cudaStream_t s) {
    static int grid8 = 0, grid10 = 0;
    if (!grid8) {
        cudaFuncSetAttribute(k_bfilter_mask<8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kMaskSmem);
        cudaFuncSetAttribute(k_bfilter_mask<10>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kMaskSmem);
        grid8 = grid_for(k_bfilter_mask<8>, kMaskThreads, kMaskSmem, 2);
        grid10 = grid_for(k_bfilter_mask<10>, kMaskThreads, kMaskSmem, 2);
    }
    cudaMemsetAsync(B.tmask, 0, sizeof(uint4) * ((size_t)1 << (2 * K)) * B.tmask_rwq, s);
    k_bmask<<<kMaxBatch / 8, 256, 0, s>>>(R, B.st, B.tent, reinterpret_cast<uint32_t*>(B.tmask),
                                          B.tmask_ex, B.tmask_rwq);
    // eight count planes where no read has more than 255 k-mer entries, else ten
    if (B.tmask_planes <= 8)
        k_bfilter_mask<8><<<shaped(grid8, R.filter_blocks), kMaskThreads, kMaskSmem, s>>>(
            R, B.st, remain, B.tent, B.tmask, B.tmask_rwq, B.tmask_ex, B.pairs, B.seg_cap, B.amb,
            B.amb_cap);
    else
        k_bfilter_mask<10><<<shaped(grid10, R.filter_blocks), kMaskThreads, kMaskSmem, s>>>(
            R, B.st, remain, B.tent, B.tmask, B.tmask_rwq, B.tmask_ex, B.pairs, B.seg_cap, B.amb,
            B.amb_cap);
    launch_exact_t<K>(R, B, s);
}

template <bool BATCH>
void launch_filter_any(const DevReads& R, RoundBuffers& B, const int32_t* remain, int drop,
                       cudaStream_t s) {
    if (!BATCH && !drop && R.k >= kWideK) {
        static int grid = 0;
        if (!grid) grid = grid_for(k_filter_g, kFilterThreads, 0, 8);
        k_gtab<<<64, 256, 0, s>>>(R, B.st, 0);
        k_filter_g<<<shaped(grid, R.filter_blocks), kFilterThreads, 0, s>>>(R, B.st, remain, B.pairs, B.seg_cap);
        k_gtab<<<64, 256, 0, s>>>(R, B.st, 1);
        return;
    }
    if (BATCH && !drop && B.tmask) {
        switch (R.k) {
            case 4: launch_bfilter_mask_t<4>(R, B, remain, s); break;
            case 5: launch_bfilter_mask_t<5>(R, B, remain, s); break;
            case 6: launch_bfilter_mask_t<6>(R, B, remain, s); break;
            default: launch_bfilter_mask_t<7>(R, B, remain, s); break;
        }
        return;
    }
    if (BATCH && !drop && B.amb) {
        switch (R.k) {
            case 4: launch_bfilter_bits_t<4>(R, B, remain, s); break;
            case 5: launch_bfilter_bits_t<5>(R, B, remain, s); break;
            case 6: launch_bfilter_bits_t<6>(R, B, remain, s); break;
            default: launch_bfilter_bits_t<7>(R, B, remain, s); break;
        }
        return;
    }
    if (BATCH && !drop && B.idx_off) {
        switch (R.k) {
            case 4: launch_bfilter_idx_t<4>(R, B, remain, s); break;
            case 5: launch_bfilter_idx_t<5>(R, B, remain, s); break;
            case 6: launch_bfilter_idx_t<6>(R, B, remain, s); break;
            default: launch_bfilter_idx_t<7>(R, B, remain, s); break;
        }
        return;
    }
    if (drop) {
        if (BATCH) launch_bfilter_t<4, true>(R, B, remain, s);
        else launch_filter_t<4, true>(R, B, remain, s);
        return;
    }
    switch (R.k) {
        case 4:
            BATCH ? launch_bfilter_t<4, false>(R, B, remain, s) : launch_filter_t<4, false>(R, B, remain, s);
            break;
        case 5:
            BATCH ? launch_bfilter_t<5, false>(R, B, remain, s) : launch_filter_t<5, false>(R, B, remain, s);
            break;
        case 6:
            BATCH ? launch_bfilter_t<6, false>(R, B, remain, s) : launch_filter_t<6, false>(R, B, remain, s);
            break;
        default:
            BATCH ? launch_bfilter_t<7, false>(R, B, remain, s) : launch_filter_t<7, false>(R, B, remain, s);
            break;
    }
}

AlignArgs align_args(RoundBuffers& B) {
    AlignArgs A;
    A.pairs = B.pairs;
    A.seg_cap = B.seg_cap;
    A.cluster = B.cluster;
    A.work = reinterpret_cast<int*>(B.st + 1);
    A.tidx = B.tidx;
    A.tt = B.tt;
    A.ttrow = B.ttrow;
    A.acc = B.acc;
    A.acc_cap = B.acc_cap;
    return A;
}

template <int G, int W, bool BATCH>
void launch_align_t(const DevReads& R, RoundBuffers& B, int cls, cudaStream_t s) {
    constexpr int smem = (kAlignThreads / 32) * sys_peq_words(W) * 4;
    static int grid = 0;
    if (!grid) {
        cudaFuncSetAttribute(k_align<G, W, BATCH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem);
        grid = grid_for(k_align<G, W, BATCH>, kAlignThreads, smem, 8);
    }
    k_align<G, W, BATCH><<<shaped(grid, R.align_blocks), kAlignThreads, smem, s>>>(R, B.st, align_args(B), cls);
}

template <int G, bool BATCH>
void launch_bandg_t(const DevReads& R, RoundBuffers& B, int cls, cudaStream_t s) {
    static int grid = 0;
    if (!grid) grid = grid_for(k_bandg<G, BATCH>, kAlignThreads, 0, 8);
    k_bandg<G, BATCH><<<shaped(grid, R.align_blocks), kAlignThreads, 0, s>>>(R, B.st, align_args(B), cls);
}

template <int W, bool BATCH>
void launch_band_t(const DevReads& R, RoundBuffers& B, int cls, cudaStream_t s) {
    static int grid = 0;
    if (!grid) grid = grid_for(k_band<W, BATCH>, kAlignThreads, 0, 8);
    k_band<W, BATCH><<<shaped(grid, R.align_blocks), kAlignThreads, 0, s>>>(R, B.st, align_args(B), cls);
}

template <bool BATCH>
void launch_align_long_t(const DevReads& R, RoundBuffers& B, cudaStream_t s) {
    constexpr int smem = (kAlignThreads / 32) * sys_peq_words(8) * 4;
    static bool set = false;
    if (!set) {
        cudaFuncSetAttribute(k_align_long<BATCH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem);
        set = true;
    }
    k_align_long<BATCH><<<num_sms(), kAlignThreads, smem, s>>>(R, B.st, align_args(B),
                                                               B.long_carry, B.long_words);
}

// Kernels launch_align_classes launches (after the greedy bound).
template <bool BATCH>
int align_launches(const RoundBuffers& B) {
    return kSysClasses - 1 - (BATCH ? 3 : 0) + (B.long_carry ? 1 : 0) +
           (BATCH || kPlainBandMaxW > 0 ? kBandClasses + kGroupClasses : 0);
}

template <bool BATCH>
void launch_align_classes(const DevReads& R, RoundBuffers& B, cudaStream_t s, bool greedy = true) {
    if (greedy) k_greedy<BATCH><<<num_sms() * 8, 256, 0, s>>>(R, B.st, align_args(B));
    if (BATCH || kPlainBandMaxW > 0) {
        launch_band_t<4, BATCH>(R, B, kSysClasses + 0, s);
        launch_band_t<8, BATCH>(R, B, kSysClasses + 1, s);
        launch_band_t<16, BATCH>(R, B, kSysClasses + 2, s);
        launch_band_t<32, BATCH>(R, B, kSysClasses + 3, s);
        constexpr int g0 = kSysClasses + kBandClasses;
        launch_bandg_t<32, BATCH>(R, B, g0 + 4, s);  // widest windows (longest work) first
        launch_bandg_t<16, BATCH>(R, B, g0 + 3, s);
        launch_bandg_t<8, BATCH>(R, B, g0 + 2, s);
        launch_bandg_t<4, BATCH>(R, B, g0 + 1, s);
        launch_bandg_t<2, BATCH>(R, B, g0 + 0, s);
    }
    if constexpr (!BATCH) {
        launch_align_t<1, 1, BATCH>(R, B, 0, s);
        launch_align_t<1, 2, BATCH>(R, B, 1, s);
    }
    if constexpr (BATCH) {
        constexpr int smem = (kAlignThreads / 32) * sys_peq_words(8) * 4;
        static int grid = 0;
        if (!grid) {
            cudaFuncSetAttribute(k_align_single, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 smem);
            grid = grid_for(k_align_single, kAlignThreads, smem, 8);
        }
        // the single-warp classes share one work counter
        k_align_single<<<shaped(grid, R.align_blocks), kAlignThreads, smem, s>>>(
            R, B.st, align_args(B), reinterpret_cast<int*>(B.st + 1) + kSingleWorkSlot);
        launch_align_t<2, 8, BATCH>(R, B, 4, s);
        launch_align_t<4, 8, BATCH>(R, B, 5, s);
        launch_align_t<8, 8, BATCH>(R, B, 6, s);
    } else {
        launch_align_t<2, 2, BATCH>(R, B, 2, s);
        launch_align_t<4, 2, BATCH>(R, B, 3, s);
        launch_align_t<8, 2, BATCH>(R, B, 4, s);
        launch_align_t<8, 4, BATCH>(R, B, 5, s);
        launch_align_t<8, 8, BATCH>(R, B, 6, s);
    }
    if (B.long_carry) launch_align_long_t<BATCH>(R, B, s);
}

}  // namespace

// Work counters of the alignment classes live right after the RoundState in
// the same allocation.
static int* align_work_of(RoundState* st) { return reinterpret_cast<int*>(st + 1); }

void init_rounds(const DevReads& R, RoundBuffers& B, int batched, int r_max, cudaStream_t s,
                 int pass_limit) {
    const int n = R.n;
    const int threads = 256;
    const int blocks = n > 0 ? (n + threads - 1) / threads : 1;
    k_init<<<blocks, threads, 0, s>>>(B.st, B.cluster, B.remain[0], B.tidx, B.best, n, batched,
                                      r_max, pass_limit, align_work_of(B.st));
    // the open pairs' per-tentative counts start at zero (k_amb_scan keeps them so)
    if (B.amb_idx) cudaMemsetAsync(B.amb_idx, 0, sizeof(int32_t) * (kMaxBatch + 1), s);
}

void resume_rounds(const DevReads& R, RoundBuffers& B, int batched, int r_max, cudaStream_t s,
                   int pass_limit) {
    const int n = R.n;
    k_resume_state<<<1, 1, 0, s>>>(B.st, r_max, pass_limit, align_work_of(B.st));
    const int want = (n + 255) / 256, cap = num_sms() * 8;
    const int blocks = n > 0 ? (want < cap ? want : cap) : 1;
    k_resume_scan<<<blocks, 256, 0, s>>>(B.st, B.cluster, B.remain[0], B.tidx, B.best, n,
                                         batched);
    k_resume_start<<<1, 1, 0, s>>>(B.st, B.cluster, batched);
    if (B.amb_idx) cudaMemsetAsync(B.amb_idx, 0, sizeof(int32_t) * (kMaxBatch + 1), s);
}

void launch_plain_round(const DevReads& R, RoundBuffers& B, int drop, int parity, cudaStream_t s,
                        long long* count, cudaEvent_t* ev4) {
    const int32_t* rin = B.remain[parity];
    int32_t* rout = B.remain[parity ^ 1];
    if (ev4) cudaEventRecordWithFlags(ev4[0], s, cudaEventRecordExternal);
    launch_filter_any<false>(R, B, rin, drop, s);
    if (R.pig_q && !drop) k_pigeon<false><<<num_sms() * 8, 256, 0, s>>>(R, B.st, B.pairs, B.seg_cap);
    if (ev4) cudaEventRecordWithFlags(ev4[1], s, cudaEventRecordExternal);
    launch_align_classes<false>(R, B, s);
    if (ev4) cudaEventRecordWithFlags(ev4[2], s, cudaEventRecordExternal);
    k_compact<<<num_sms() * 4, 256, 0, s>>>(B.st, rin, rout, B.cluster);
    k_advance<<<1, 1, 0, s>>>(B.st, B.cluster, align_work_of(B.st));
    if (ev4) cudaEventRecordWithFlags(ev4[3], s, cudaEventRecordExternal);
    if (count)
        *count += 4 + align_launches<false>(B) + (R.pig_q && !drop ? 1 : 0) +
                  (!drop && R.k >= kWideK ? 2 : 0);
}

void launch_align_stage(const DevReads& R, RoundBuffers& B, bool batched_mapping, bool greedy,
                        cudaStream_t s) {
    if (batched_mapping) launch_align_classes<true>(R, B, s, greedy);
    else launch_align_classes<false>(R, B, s, greedy);
}

int align_class_host(int words) {
    return words <= 32 ? 0 : words <= 64 ? 1 : words <= 128 ? 2 : words <= 256 ? 3
                         : words <= 512 ? 4 : words <= 1024 ? 5
                         : words <= kMaxPatternWords ? 6 : kLongClass;
}

void launch_batch_pass(const DevReads& R, RoundBuffers& B, int drop, int parity, cudaStream_t s,
                       long long* count, cudaEvent_t* ev4) {
    const int32_t* rin = B.remain[parity];
    int32_t* rout = B.remain[parity ^ 1];
    k_bselect<<<1, 1024, 0, s>>>(B.st, B.cluster, R.n, B.tent, B.tidx, B.tt, B.ttrow, B.survive,
                                 align_work_of(B.st));
    if (ev4) cudaEventRecordWithFlags(ev4[0], s, cudaEventRecordExternal);
    launch_filter_any<true>(R, B, rin, drop, s);
    if (R.pig_q && !drop) k_pigeon<true><<<num_sms() * 8, 256, 0, s>>>(R, B.st, B.pairs, B.seg_cap);
    if (ev4) cudaEventRecordWithFlags(ev4[1], s, cudaEventRecordExternal);
    launch_align_classes<true>(R, B, s);
    if (ev4) cudaEventRecordWithFlags(ev4[2], s, cudaEventRecordExternal);
    k_bsurvive<<<1, 32, 0, s>>>(B.st, B.tent, B.tt, B.ttrow, B.survive, B.cluster);
    const int g = num_sms() * 2;
    k_bclaim<<<g, 256, 0, s>>>(B.st, B.acc, B.tidx, B.survive, B.best);
    k_bapply<<<g, 256, 0, s>>>(B.st, B.acc, B.tidx, B.best, B.cluster);
    k_compact<<<num_sms() * 4, 256, 0, s>>>(B.st, rin, rout, B.cluster);
    k_badvance<<<1, 1, 0, s>>>(B.st, B.tent, align_work_of(B.st), B.seg_cap, B.acc_cap,
                               B.amb_cap, drop);
    if (ev4) cudaEventRecordWithFlags(ev4[3], s, cudaEventRecordExternal);
    if (count)
        *count += 8 + align_launches<true>(B) + (!drop ? 1 : 0) +
                  (R.pig_q && !drop ? 1 : 0) + (B.amb && !drop ? 4 : 0);
    // (a word-filter form launches two kernels, six with the open-pair
    // queue: the bitmap form k_filter, k_bfilter_bits, the mask form k_bmask,
    // k_bfilter_mask, then k_amb_count, k_amb_scan, k_amb_place, k_bexact_t)
}

// Whether a job's per-pass k-mer index (at most `cap` postings) is kept in
// shared memory by the index filter: 16-bit offsets need cap < 65536, and the
// layout for a 1024-thread CTA must fit the device's per-block maximum.
bool index_in_smem(int k, int r_max, int64_t cap, int smem_optin) {
    if (cap <= 0 || cap >= 65536) return false;
    return IndexSmem(k, r_max, cap, true).bytes(1024 / 32) <= smem_optin;
}

int set_spin_limit(int polls) {
    const int v = polls < 0 ? kSpinLimit : polls;
    return cudaMemcpyToSymbol(c_spin_limit, &v, sizeof(int)) == cudaSuccess ? 0 : -1;
}

}  // namespace gsdr
