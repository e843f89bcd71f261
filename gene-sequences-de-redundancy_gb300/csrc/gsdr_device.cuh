// gsdr_device.cuh -- device-side data layout and kernel entry points.
//
// Layout in HBM of one clustering job (n reads in length-sorted order):
//   raw bytes    the caller's sequence bytes, one H2D copy, read i at offset[i]
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

constexpr int kMaxK = 8;             // k-mer length handled by the u32 entry format
constexpr int kMaxPatternWords = 1024;  // 32 lanes x 32 words: 32768 gap-free bases

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
    // pigeon filter (p 1)
    const int64_t* raw_off;  // the reference's padded byte offsets (copyData)
    uint16_t* pig;           // 256 inclusive prefix counts per read
    uint16_t* pig_idx;       // positions, at raw_off[i] + slot
};

// Per-job round state, in device memory; kernels read their work sizes here so
// that a whole sequence of rounds can be captured in one CUDA graph.
struct RoundState {
    int32_t rep;        // representative of the current round (plain form)
    int32_t n_remain;   // entries in the current remain list
    int32_t n_next;     // entries written by the compaction
    int32_t next_min;   // smallest still-unclustered index seen by the compaction
    int32_t n_pairs[2]; // pairs queued for alignment: short / long patterns
    int32_t pair_overflow;
    int32_t work_filter;
    int32_t done;
    int32_t error;
    int32_t batch_first;   // batched form: index of the first tentative in `tent`
    int32_t n_tent;        // batched form: tentatives this pass
    long long rounds;      // representatives taken so far
    long long passes;
    unsigned long long cnt_prefilter, cnt_word, cnt_aligned, cnt_accepted;
    unsigned long long cells;
    unsigned long long filter_bytes;
};

struct Pair {
    int32_t rep;
    int32_t cand;
};

// ---- prep.cu ----
// Parse + gap-free pack + composition + cutoffs, one warp per read.
void launch_pack(const DevReads& R, float t, int k, cudaStream_t s);
// Distinct k-mers with multiplicities for every read (k <= kMaxK).
int launch_kmers(const DevReads& R, int k, cudaStream_t s);
// Pigeon index (kernel_createPigeon1/2 semantics).
void launch_pigeon_index(const DevReads& R, cudaStream_t s);

// ---- rounds.cu ----
struct RoundBuffers {
    RoundState* st;      // device
    int32_t* cluster;    // device, n
    int32_t* remain[2];  // device, n each
    Pair* pairs;         // device
    int32_t pair_cap;
    int32_t* tent;       // batched form: tentative indices
    uint32_t* accept;    // batched form: accept bits per (tentative, candidate slot)
    int32_t batch;
};
void init_rounds(const DevReads& R, RoundBuffers& B, cudaStream_t s);
// Launches one plain round (filter, align, compact, advance); `parity` picks
// which remain buffer is the input.  `count` accumulates kernel launches.
void launch_plain_round(const DevReads& R, RoundBuffers& B, float t, int drop, int pigeon,
                        int parity, cudaStream_t s, long long* count, cudaEvent_t* ev4);
int filter_smem_bytes(int k, int drop);
int num_sms();

}  // namespace gsdr
