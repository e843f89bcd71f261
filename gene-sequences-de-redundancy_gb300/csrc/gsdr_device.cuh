// gsdr_device.cuh -- device-side data layout and kernel entry points.
//
// Layout in HBM of one clustering job (n reads in length-sorted order):
//   raw bytes    the caller's sequence bytes, one H2D copy (or the FASTA
//                path's device copy of the file, read in place), read i at offset[i]
//   len, len_gf  raw length (with gaps) and gap-free length       i32[n]
//   pack_off     word offset of read i in `packed` (multiple of 4) i64[n+1]
//   packed       2-bit codes, 16 bases per u32, first base in bits 31:30
//                (the reference's kernel_compressData format)
//   comp         A/C/G/T counts of the gap-free read               int4[n]
//   cut_*        word / base / pigeon cutoffs                      i32[n]
//   kmer_off     entry offset of read i in `kmer` (multiple of 4)  i64[n+1]
//   n_kmer       distinct k-mers of read i                         i32[n]
//   kmer         (k-mer << 16) | multiplicity, u32 per distinct k-mer,
//                padded with zero entries to a multiple of 4 (one uint4 load)
//   cluster      -1 or the representative                          i32[n]
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gsdr {

constexpr int kMaxPatternWords = 2048;  // 8 warps x 32 lanes x 8 words: 65536 gap-free bases
constexpr int kSysClasses = 8;          // pattern length classes of the systolic alignment kernels
constexpr int kLongClass = kSysClasses - 1;  // patterns above kMaxPatternWords: in chunks
constexpr int64_t kMaxReadBases = 1ll << 24;  // longest read (raw bases) a job takes
constexpr int kBandClasses = 4;         // window classes (4, 8, 16, 32 words) of the banded kernel
constexpr int kGroupClasses = 5;        // group-banded classes: 2, 4, 8, 16, 32 lanes x 4 words
constexpr int kGroupMaxWords = 128;     // widest window of the group-banded kernel
constexpr int kAlignClasses = kSysClasses + kBandClasses + kGroupClasses;  // alignment queues
constexpr int kSingleWorkSlot = kAlignClasses;  // work counter of the merged single-warp systolic classes

// Group-banded class of a window of bw <= kGroupMaxWords words: the fewest
// lanes (2, 4, .. 32) whose 4 words each hold it.
__host__ __device__ __forceinline__ int group_class(int bw) {
    const int g = bw <= 8 ? 0 : bw <= 16 ? 1 : bw <= 32 ? 2 : bw <= 64 ? 3 : 4;
    return kSysClasses + kBandClasses + g;
}
constexpr int kMaxBatch = 1024;         // tentative representatives per batched pass
constexpr int kTTWords = kMaxBatch / 32;
constexpr int kMaxBitsK = 6;            // k-mer presence bitmaps for k <= 6 (4^k bits per read)
constexpr int kMaxBits2K = 7;           // the batched two-level bitmap filter: k <= 7
constexpr int kMaskMaxEntries = 1023;   // tentative-mask filter: reads of at most 1,023 k-mers
constexpr int kMaskEntries8 = 255;      // ... with eight count planes up to 255, else ten

struct Pair {
    int32_t rep;   // read index of the representative (or tentative)
    int32_t cand;  // read index of the candidate
};

struct DevReads {
    int32_t n;
    int32_t k;
    const uint8_t* bytes;
    const int64_t* off;
    const int32_t* len;
    int32_t* len_gf;
    const int64_t* pack_off;
    uint32_t* packed;
    int4* comp;
    int32_t* cut_word;
    int32_t* cut_base;
    int32_t* cut_pig;
    const int64_t* kmer_off;
    int32_t* n_kmer;
    uint32_t* kmer;
    // base bit-planes of the gap-free read: plane c (0..3) of read i starts
    // at bm[2*pack_off[i] + c*(pack_off[i+1]-pack_off[i])/2]; bit b of word w
    // is set iff base 32w+b equals c (bits past the read are zero)
    uint32_t* bm;
    // k <= kMaxBitsK: presence bitmap of the k-mers with a non-zero stored
    // multiplicity (4^k bits per read, read i at kbits[i * 4^k/32]) and the
    // multiplicity excess sum(count) - #distinct over those k-mers
    uint32_t* kbits;
    int32_t* kextra;
    // batched bitmap filter only (null otherwise): the second count level --
    // bitmap of the k-mers with a stored multiplicity of 2 or more (same
    // layout as kbits) and the excess above two, sum over k-mers of
    // max(count - 2, 0)
    uint32_t* kbits2;
    int32_t* kextra3;
    // pigeon filter (p 1; null otherwise), the reference's 4-mer position
    // index: pig[256 i + v] = inclusive prefix of read i's 4-mer bucket counts
    // (u16), pidx[off[i] + slot] = (u16) absolute position of a window's last
    // base in the reference's padded layout, positions descending within a
    // bucket; refoff16[i] = that layout's offset of read i (low 16 bits).
    uint16_t* pig;
    uint16_t* pidx;
    const uint16_t* refoff16;
    Pair* pig_q;        // pairs that passed the other filters, for the pigeon filter
    int32_t pig_cap;
    // word lengths above 7 (k-mer ids wider than 16 bits): kmer holds the
    // k-mer ids and kcnt their u16 counts (null for k <= 7); gtab is the
    // representative's 4^k-entry count table in global memory, as the
    // reference's (func.cu:712-736); khash is a per-CTA hash scratch for
    // counting each read's k-mers (khash_slots slots of {key, count})
    uint16_t* kcnt;
    uint16_t* gtab;
    uint32_t* khash;
    int32_t khash_slots;
    int32_t khash_ctas;  // CTAs of the hash count (each owns khash_slots slots)
    // largest serial work (text bases x window words) of a pair given to the
    // lane-per-pair banded kernel; longer pairs go to the systolic kernels
    int64_t band_serial;
    // block shape (gsdr_opts): resident CTAs per SM the alignment and the
    // word-filter kernels are launched with (0: as many as fit)
    int32_t align_blocks;
    int32_t filter_blocks;
    // widest window (words) given to the group-banded kernel (kGroupMaxWords;
    // 0: none, those pairs go to the systolic kernels)
    int32_t group_max_w;
    // semantics (gsdr_opts::variant): 1 = the SYCL program's.  brk (variant 1
    // with filters, null otherwise): bit g of read i (word pack_off[i] + g/32)
    // is set when a non-ACGT byte stands right before gap-free base g in the
    // raw read; a k-mer whose window holds such a break is not a k-mer there
    // (func.cpp:238-274 skips raw windows that hold a non-ACGT byte)
    uint32_t* brk;
    int32_t variant;
    // 1 with variant 1: cut_base holds the alignment's cutoff ceil(len * t)
    // + 1 (LCS > ceil(len * t), func.cpp:671) and the composition prefilter
    // compares with cut_base - strict (func.cpp:532-547)
    int32_t strict;
    float threshold;
};

// Per-job round state, in device memory; kernels read their work sizes here so
// that a whole sequence of rounds can be captured in one CUDA graph.
struct RoundState {
    int32_t rep;        // plain form: representative of the current round
    int32_t n_remain;   // entries in the current remain list
    int32_t n_next;     // entries written by the compaction
    int32_t next_min;   // smallest still-unclustered index seen by the compaction
    int32_t n_pairs[kAlignClasses];  // pairs queued per alignment class
    int32_t pair_overflow;
    int32_t done;
    int32_t error;
    // batched form
    int32_t pass;       // pass number (keys of tidx/best carry it), from 1
    int32_t R;          // tentatives requested for this pass
    int32_t R_max;
    int32_t cursor;     // first index not yet considered as a tentative
    int32_t n_tent;     // tentatives selected this pass
    int32_t n_acc;      // accepted pairs this pass
    int32_t acc_overflow;
    int32_t survivors;  // representatives confirmed this pass
    int32_t absorbed;   // reads absorbed this pass
    int32_t n_amb;      // pairs the bitmap or mask bound left to the exact word filter
    int32_t n_pig;      // pairs queued for the pigeon filter
    int32_t pass_limit; // > 0: stop after this many passes (timing runs; result unfinished)
    long long rounds;   // representatives taken so far
    long long passes;
    unsigned long long cnt_prefilter, cnt_word, cnt_aligned, cnt_accepted;
    unsigned long long cnt_pig_reject;  // pairs the pigeon filter removed
    unsigned long long cells;
    unsigned long long filter_bytes;
    // DP cells the alignment kernels stepped: per block of 32 text bases, the
    // 32-bit pattern (or band window) words a warp or lane held x 32 bits x 32
    // bases; early exits and bands make it smaller than `cells`
    unsigned long long cells_done;
};

// ---- prep.cu ----
// Parse + gap-free pack + composition + cutoffs, one warp per read.
void launch_pack(const DevReads& R, float t, int k, cudaStream_t s);
// Distinct k-mers with multiplicities for every read.
int launch_kmers(const DevReads& R, int k, cudaStream_t s);
// CTAs of the hash-based k-mer count (k >= 8): each owns R.khash_slots slots.
constexpr int kHashCtas = 128;
constexpr int kWideK = 8;  // word lengths from here on use the wide k-mer layout
// Default of DevReads::band_serial (GSDR_BAND_SERIAL overrides it).
constexpr long long kBandMaxSerial = 16384;
// Base bit-planes of every read (after launch_pack).
void launch_planes(const DevReads& R, cudaStream_t s);
// The pigeon filter's 4-mer position index of every read (p 1).
void launch_pigeon_index(const DevReads& R, cudaStream_t s);
int num_sms();

// ---- rounds.cu ----
struct RoundBuffers {
    RoundState* st;      // device
    int32_t* cluster;    // device, n
    int32_t* remain[2];  // device, n each
    Pair* pairs;         // device: kAlignClasses segments of seg_cap pairs
    // reads above kMaxPatternWords * 32 bases: per block of k_align_long two
    // buffers of long_words carry words (null when no read is that long)
    uint32_t* long_carry;
    int32_t long_words;
    int32_t seg_cap;
    // batched form
    int32_t* tent;       // kMaxBatch tentative read indices (ascending)
    uint32_t* tidx;      // n: (pass << 12) | tentative index, for reads that are tentatives
    uint32_t* best;      // n: (pass << 12) | (4095 - i) of the claiming tentative
    uint32_t* tt;        // kMaxBatch x kTTWords: tentative h accepted tentative i
    uint32_t* ttrow;     // kTTWords: rows of tt with any bit
    uint32_t* survive;   // kTTWords
    Pair* acc;           // accepted pairs of the pass
    int32_t acc_cap;
    // batched word filter by inverted index (sparse k-mer spaces; null = the
    // per-tentative table form): for k-mer m, idx_post[idx_off[m] ..
    // idx_off[m + 1]) holds (tentative << 16 | count) of every tentative with
    // a non-zero count of m.  Rebuilt every pass.
    uint32_t* idx_off;   // 4^k + 1
    uint32_t* idx_post;  // idx_cap
    uint16_t* idx_off16;   // 16-bit copies for the shared-memory form (null otherwise)
    uint16_t* idx_post16;
    int64_t idx_cap;
    int32_t r_max;       // largest R of the job (sizes the index filter's shared memory)
    // batched word filter by k-mer presence bitmaps or by tentative masks
    // (null = another form): pairs the bound D <= S <= D + min(excess)
    // cannot decide
    Pair* amb;           // amb_cap pairs
    int32_t amb_cap;
    Pair* amb2;          // the same pairs grouped by tentative (amb_cap)
    int32_t* amb_idx;    // 4 x (kMaxBatch + 1): per tentative counts (zero between
                         // passes), run offsets, cursors, work items
    // batched word filter by tentative masks (short reads, k <= 7; null =
    // another form): row m (tmask_rwq x 16 bytes) has bit t set iff tentative
    // t holds k-mer m; tmask_ex[t] = its excess, sum of (count - 1).  Zeroed
    // and rebuilt every pass.
    uint4* tmask;        // 4^k rows
    int32_t* tmask_ex;   // kMaxBatch
    int32_t tmask_rwq;   // 16-byte words per row: ceil(r_max / 128)
    int32_t tmask_planes;  // count planes: 8 (every read <= kMaskEntries8 entries) or 10
};
void init_rounds(const DevReads& R, RoundBuffers& B, int batched, int r_max, cudaStream_t s,
                 int pass_limit = 0);
// Polls each bounded wait of the alignment kernels makes on the current
// device before it gives up (polls < 0: the default, kSpinLimit); for tests
// that make a wait run out.  Returns 0 or -1 (CUDA error).
int set_spin_limit(int polls);
// Round state from a checkpoint instead of a fresh start: B.cluster already
// holds the unfinished clustering (-1 = unclustered); builds the remain list,
// the next representative (plain) or the tentative cursor (batched).
void resume_rounds(const DevReads& R, RoundBuffers& B, int batched, int r_max, cudaStream_t s,
                   int pass_limit = 0);
// One plain round (filter, align, compact, advance); `parity` picks which
// remain buffer is the input.  `count` accumulates kernel launches; `ev4`
// (optional) receives events around the filter and alignment stages.
void launch_plain_round(const DevReads& R, RoundBuffers& B, int drop, int parity,
                        cudaStream_t s, long long* count, cudaEvent_t* ev4);
// Only the alignment stage over the queued pairs (st->n_pairs), with the
// plain or the batched warp grouping, optionally after the greedy bound.
void launch_align_stage(const DevReads& R, RoundBuffers& B, bool batched_mapping, bool greedy,
                        cudaStream_t s);
int align_class_host(int words);
bool index_in_smem(int k, int r_max, int64_t cap, int smem_optin);
// One batched pass (select, filter, align, resolve, compact, advance).
void launch_batch_pass(const DevReads& R, RoundBuffers& B, int drop, int parity, cudaStream_t s,
                       long long* count, cudaEvent_t* ev4);

}  // namespace gsdr
