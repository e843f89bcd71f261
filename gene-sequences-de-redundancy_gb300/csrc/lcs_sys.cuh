// lcs_sys.cuh -- systolic bit-parallel LCS decision on a group of warps.
//
// Decides LCS(pattern, text) >= c, the test of the reference's kernel_align
// (cuda-version/func.cu:828-999, a full O(q*T) DP per thread), with Hyyro's
// recurrence over pattern bits:
//     U = V & M[x];  V' = (V + U) | (V & ~M[x]);   LCS = zeros of V.
// Pattern = candidate, text = representative.  Lane l of warp b holds the W
// pattern words (b*32 + l)*W .. +W-1.  The warp is a systolic array: at local
// step s lane l applies text base x = s - l, taking the carry of the addition
// from lane l-1's step s-1 (one shuffle per step), so a step is one short
// dependent chain instead of a warp-wide carry resolution.  Between warps the
// top lane's carry-out sequence (one bit per text base) is the next warp's
// lane-0 carry-in sequence, handed over in 32-bit words through a ring in
// shared memory.  Text bases come from a per-warp 64-entry ring (written twice
// so that a lane-skewed window is contiguous), one 32-bit word per base: the
// offset of the base's rows in a per-warp table of match masks in shared
// memory (peq_step reads the lane's column there), which keeps the integer
// pipe for the recurrence itself and costs a step no decoding of the base.
//
// Bases outside the text ("no base": pipeline fill before base 0, drain after
// base T-1) must leave V unchanged.  Their ring entry points at a fifth, all-
// zero row of the table: with M = 0, U = V & M = 0, and with a zero carry-in
// V + U + 0 = V and V' = V | (V & ~M) = V; the carry out is then zero too, so
// by induction every carry-in of such a step is zero.
//
// Decisions, taken every kSysCk blocks of 32 bases by the group's last warp
// from the zero counts every warp publishes:
//   accept  LCS(pattern, text[0..X]) >= c (never decreases with X);
//   reject  Z(q-R) + min(R, q) < c, R = bases after X, Z(i) = zeros below
//           pattern position i: any common subsequence has <= Z(i) matches
//           with text[0..X] and <= min(q-i, R) after, maximal at i = q-R.
// Every wait is bounded (c_spin_limit polls) and reports an error instead of
// hanging.
//
// Chunk mode (patterns above one group's 65,536 rows): the pattern is cut into
// chunks of rows run one after another over the whole text; the top lane's
// carry-out sequence of a chunk (one bit per text base, in 32-bit words) goes
// to a global buffer and is the next chunk's lane-0 carry-in sequence, as
// between the warps of a group.  The zeros of V then add up over the chunks,
// so a chunk takes no early decision and reports its zero count at the end of
// the text (S.result).
#pragma once
#include <stdint.h>

#include "lcs.cuh"

namespace gsdr {

constexpr int kSysRing = 4;     // carry words in flight between two warps
constexpr int kSysZRing = 16;   // checkpoints kept per warp
constexpr int kSysCk = 4;       // blocks of 32 bases between checkpoints
constexpr int kSpinLimit = 1 << 22;
// Polls a wait makes before it gives up: kSpinLimit unless a test lowered it
// (set_spin_limit, rounds.cu); with 0 every wait gives up at once.
static __constant__ int c_spin_limit = kSpinLimit;

// Shared state of a group of up to NW warps deciding one pair.
template <int NW>
struct SysGroupT {
    static constexpr int kWarps = NW;
    uint32_t carries[NW][kSysRing];
    int zc[NW][kSysZRing];    // zeros of the warp's words at a checkpoint
    int zp[NW][kSysZRing];    // zeros below q - R at that checkpoint
    int zf[NW];               // zeros at the end of the text
    int ready[NW];            // carry words published by warp b
    int consumed[NW];         // carry words of warp b read by warp b+1
    uint32_t ring[NW][128];   // text bases: their row offsets in the match-mask table
    int stop;
    int result;
    int idx;
    int error;
};
using SysGroup = SysGroupT<8>;

__device__ __forceinline__ int vload(const int* p) { return *(volatile const int*)p; }
__device__ __forceinline__ void vstore(int* p, int v) { *(volatile int*)p = v; }

__device__ __forceinline__ void group_bar(int id, int nthreads) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

__device__ __forceinline__ bool spin_until_ge(const int* p, int target, const int* stop) {
    for (int it = 0; it < c_spin_limit; it++) {
        if (vload(p) >= target) return true;
        if (vload(stop)) return true;
        if (it > 64) __nanosleep(20);
    }
    return false;
}

__device__ __forceinline__ uint32_t valid_bits(int q, int w) {
    const int rem = q - 32 * w;
    return rem >= 32 ? 0xffffffffu : (rem > 0 ? ((1u << rem) - 1u) : 0u);
}

template <int W>
__device__ __forceinline__ int zeros_below(const uint32_t (&V)[W], int w0, int lim) {
    int z = 0;
#pragma unroll
    for (int i = 0; i < W; i++) z += __popc(~V[i] & valid_bits(lim, w0 + i));
    return z;
}

// Ring entry of a text base: the word offset of its rows in the match-mask
// table (rows of 32 * W words per base code; row 4 is all zero, for "no base").
template <int W>
__device__ __forceinline__ uint32_t base_row(uint32_t code, bool valid) {
    return (valid ? (code & 3u) : 4u) * (32u * W);
}

template <class Group>
__device__ __forceinline__ void sys_fail(Group& S, int* err_flag, int lane) {
    if (lane == 0) {
        atomicExch(err_flag, 1);
        vstore(&S.error, 1);
        vstore(&S.stop, 1);
    }
}

// Eight steps of the systolic array from ring slot rb[0..7].
//   MULTI: lane 0 takes its carry-in from cin8 (the previous warp's carries,
//          bit j for step j) and lane 31 collects its carry-outs into out8;
//          otherwise lane 0's carry-in is zero.
//   SNAP:  lane l copies V into snapV after the step j == tj (per lane).
template <int W, bool MULTI, bool SNAP>
__device__ __forceinline__ void sys_steps8(const uint32_t* __restrict__ rb,
                                           const uint32_t* __restrict__ peq, uint32_t (&V)[W],
                                           uint32_t (&snapV)[W], uint32_t& from, uint32_t cin8,
                                           uint32_t& out8, uint32_t not_lane0, int tj, int jbase,
                                           int lane) {
#pragma unroll
    for (int j = 0; j < 8; j++) {
        uint32_t cin = from;
        if (MULTI) cin = not_lane0 ? from : ((cin8 >> j) & 1u);
        // lane 0 of a single warp has a zero carry-in: its carry enable is
        // not_lane0 = 0 (its `from` is its own carry-out, from the shuffle)
        peq_step<W>(V, peq + rb[j], cin, MULTI ? 0xffffffffu : not_lane0);
        if (MULTI) out8 |= cin << j;
        // lane 0 receives its own carry-out from the shuffle: a single warp
        // ignores it through the carry enable above, a group member through
        // the select of the previous warp's carry bits
        from = __shfl_up_sync(0xffffffffu, cin, 1);
        if (SNAP && jbase + j == tj) {
#pragma unroll
            for (int i = 0; i < W; i++) snapV[i] = V[i];
        }
    }
}

// One block of 32 steps (four unrolled groups of eight).
template <int W, bool MULTI, bool SNAP>
__device__ __forceinline__ void sys_block(const uint32_t* __restrict__ rb,
                                          const uint32_t* __restrict__ peq, uint32_t (&V)[W],
                                          uint32_t (&snapV)[W], uint32_t& from, uint32_t cin_word,
                                          uint32_t& cout_word, uint32_t not_lane0, int tj,
                                          int lane) {
    cout_word = 0;
#pragma unroll 1
    for (int g = 0; g < 4; g++) {
        uint32_t out8 = 0;
        sys_steps8<W, MULTI, SNAP>(rb + 8 * g, peq, V, snapV, from, cin_word >> (8 * g), out8,
                                   not_lane0, tj, 8 * g, lane);
        if (MULTI) cout_word |= out8 << (8 * g);
    }
}

// Shared memory of one warp's match-mask table (sys_peq_words(W) words): rows
// for the four base codes and the all-zero "no base" row.
__host__ __device__ constexpr int sys_peq_words(int W) { return 5 * W * 32; }

// The decision of one pair on B warps of a group (gw = this warp's index).
// The result lands in S.result (1 accept, 0 reject) once the group meets at
// its barrier; S.error is set if a wait gave up.  Returns the blocks of 32
// steps this warp ran (its computed cells: blocks x 32 x 32 lanes x W x 32).  peq: this warp's
// sys_peq_words(W) words of shared memory for the pattern's match masks.
// Chunk mode (chunk true): gcin (or null for the first chunk) holds the
// carry-in words of warp 0's lane 0, gcout (or null for the last chunk)
// receives the carry-out words of the last warp's lane 31 (a full chunk), and
// S.result is the chunk's zero count at the end of the text.
template <int W, class Group>
__device__ int lcs_sys_pair(Group& S, uint32_t* peq, const uint32_t* __restrict__ pq, int q,
                             const uint32_t* __restrict__ pt, int T, int c, int B, int gw,
                             int lane, int* err_flag, bool chunk = false,
                             const uint32_t* __restrict__ gcin = nullptr,
                             uint32_t* __restrict__ gcout = nullptr) {
    const int w0 = (gw * 32 + lane) * W;
    uint32_t V[W], snapV[W];
    peq += lane;
    peq_fill<W>(peq, pq, q, w0);
#pragma unroll
    for (int i = 0; i < W; i++) {
        V[i] = 0xffffffffu;
        snapV[i] = 0xffffffffu;
    }
    uint32_t* ring = S.ring[gw];
#pragma unroll
    for (int r = 0; r < 4; r++) ring[lane + 32 * r] = base_row<W>(0, false);
    __syncwarp();
    const int M = (T + 31 + 31) >> 5;  // blocks of 32 steps: steps 0 .. T+30
    const bool multi = B > 1 || gcin != nullptr || gcout != nullptr;
    const bool to_global = gcout != nullptr && gw == B - 1;
    const bool producer = gw < B - 1 || to_global;
    const uint32_t not_lane0 = lane == 0 ? 0u : 0xffffffffu;
    uint32_t from = 0;   // carry from lane l-1 at the previous step
    uint32_t wprev = 0;  // top lane: carry bits of the word being completed
    bool decided = false;
    int blocks = 0;
    for (int m = 0; m < M; m++) {
        if (vload(&S.stop)) return blocks;
        uint32_t cin_word = 0;
        if (gw == 0 && gcin) cin_word = __ldcg(gcin + m);
        if (gw > 0) {
            if (!spin_until_ge(&S.ready[gw - 1], m + 1, &S.stop)) {
                sys_fail(S, err_flag, lane);
                return blocks;
            }
            if (vload(&S.stop)) return blocks;
            __threadfence_block();
            cin_word = *(volatile uint32_t*)&S.carries[gw - 1][m % kSysRing];
            __syncwarp();
            if (lane == 0) vstore(&S.consumed[gw - 1], m + 1);
        }
        // this block's text bases 32m .. 32m+31 into the ring (twice)
        {
            const int x = 32 * m + lane;
            uint32_t code = 0;
            if (x < T) code = (__ldg(pt + (x >> 4)) >> (30 - 2 * (x & 15))) & 3u;
            const uint32_t bw = base_row<W>(code, x < T);
            ring[x & 63] = bw;
            ring[(x & 63) + 64] = bw;
        }
        __syncwarp();
        const uint32_t* rb = ring + ((32 * m - lane) & 63);
        // Zero-count snapshots for the checkpoint at base 32m'-1 (m' = next
        // phase-0 block): lane 0 reaches it at step 31 of the phase kSysCk-1
        // block, lane l >= 1 at step l-1 of the phase-0 block.
        const int phase = m % kSysCk;
        uint32_t cout_word = 0;
        if (phase == kSysCk - 1 || (phase == 0 && m > 0)) {
            const int tj = phase == 0 ? (lane == 0 ? -1 : lane - 1) : (lane == 0 ? 31 : -1);
            if (multi)
                sys_block<W, true, true>(rb, peq, V, snapV, from, cin_word, cout_word, not_lane0,
                                         tj, lane);
            else
                sys_block<W, false, true>(rb, peq, V, snapV, from, cin_word, cout_word,
                                          not_lane0, tj, lane);
        } else {
            if (multi)
                sys_block<W, true, false>(rb, peq, V, snapV, from, cin_word, cout_word,
                                          not_lane0, -1, lane);
            else
                sys_block<W, false, false>(rb, peq, V, snapV, from, cin_word, cout_word,
                                           not_lane0, -1, lane);
        }
        __syncwarp();
        blocks++;
        const bool last_block = m == M - 1;
        // end of text: final zero counts, published before the last carry word
        if (last_block) {
            const int zf = warp_sum_i(zeros_below<W>(V, w0, q));
            if (lane == 0) S.zf[gw] = zf;
        }
        // top lane's carry-outs this block: bits for bases 32m-31 .. 32m
        // (step j carries base 32m+j-31): bits 1..31 finish word m-1, bit 31 of
        // the block is bit 0 of word m.
        if (producer) {
            const uint32_t cw = __shfl_sync(0xffffffffu, cout_word, 31);
            const uint32_t wdone = wprev | (cw << 1);
            const uint32_t wlast = cw >> 31;
            const int nw = last_block ? 2 : 1;  // words m-1 (and m at the end)
            for (int k2 = 0; k2 < nw; k2++) {
                const int widx = m - 1 + k2;
                if (widx < 0) continue;
                if (to_global) {  // chunk mode: the next chunk reads it after this one
                    if (lane == 0) __stcg(gcout + widx, k2 == 0 ? wdone : wlast);
                    continue;
                }
                if (!spin_until_ge(&S.consumed[gw], widx + 1 - kSysRing, &S.stop)) {
                    sys_fail(S, err_flag, lane);
                    return blocks;
                }
                if (lane == 0) S.carries[gw][widx % kSysRing] = k2 == 0 ? wdone : wlast;
                __threadfence_block();
                __syncwarp();
                if (lane == 0) vstore(&S.ready[gw], widx + 1);
            }
            wprev = wlast;
        }
        // checkpoint for base 32m-1, decided by the last warp
        const int Xck = 32 * m - 1;
        if (!chunk && phase == 0 && m > 0 && Xck < T - 1) {
            const int Rck = T - 1 - Xck;
            const int lim = q - Rck;
            const int zf_ck = warp_sum_i(zeros_below<W>(snapV, w0, q));
            const int zp_ck = lim > 0 ? warp_sum_i(zeros_below<W>(snapV, w0, lim)) : 0;
            const int slot = (m / kSysCk) % kSysZRing;
            if (lane == 0) {
                S.zc[gw][slot] = zf_ck;
                S.zp[gw][slot] = zp_ck;
            }
            __threadfence_block();
            __syncwarp();
            if (gw == B - 1) {
                int zt = 0, zpt = 0;
                for (int b2 = 0; b2 < B; b2++) {
                    zt += *(volatile int*)&S.zc[b2][slot];
                    zpt += *(volatile int*)&S.zp[b2][slot];
                }
                const int ub = (lim > 0 ? zpt : 0) + min(Rck, q);
                int d = -1;
                if (zt >= c) d = 1;
                else if (ub < c) d = 0;
                if (d >= 0) {
                    if (lane == 0) {
                        vstore(&S.result, d);
                        __threadfence_block();
                        vstore(&S.stop, 1);
                    }
                    decided = true;
                }
            }
        }
        if (decided) return blocks;
    }
    if (gw == B - 1) {
        int zt = 0;
        for (int b2 = 0; b2 < B; b2++) zt += *(volatile int*)&S.zf[b2];
        if (lane == 0) {
            vstore(&S.result, chunk ? zt : (zt >= c ? 1 : 0));
            __threadfence_block();
            vstore(&S.stop, 1);
        }
    }
    return blocks;
}

}  // namespace gsdr
