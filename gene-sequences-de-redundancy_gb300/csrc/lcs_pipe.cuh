// lcs_pipe.cuh -- bit-parallel LCS decision spread over a group of warps.
//
// The decision of the reference's kernel_align (cuda-version/func.cu:828-999):
// LCS(pattern, text) >= c over gap-free bases, here pattern = candidate and
// text = representative.  Hyyro's recurrence over the pattern bits,
//     U = V & M[ch];  V' = (V + U) | (V & ~M[ch]);   LCS = zeros of V,
// is one long addition per text base.  The pattern words are split into
// consecutive blocks, one per warp; lane l of warp b holds words
// b*32*W + l*W .. +W-1.  Inside a warp the carry crosses lanes by a
// carry-lookahead on two ballots (carry into lane l = bit l of
// (G + (G|P) + cin) ^ G ^ (G|P)).  Between warps the carry-out sequence of
// block b (one bit per text base) is the carry-in sequence of block b+1, so
// the warps run as a pipeline over the text: warp b hands block b+1 a 32-bit
// word of carries every 32 bases through shared memory.  The last warp is the
// slowest; at the end of every 32-base chunk it adds up the zero counts every
// warp published for that chunk and decides:
//   accept  as soon as LCS(pattern, text[0..x]) >= c (the LCS of a text prefix
//           never decreases);
//   reject  as soon as Z(q-R) + min(R, q) < c, where R = text bases left and
//           Z(i) = LCS(pattern[0..i), text[0..x]); every common subsequence
//           splits at some pattern position i into <= Z(i) matches before and
//           <= min(q-i, R) after, and that bound is largest at i = q-R.
// Every wait is bounded: after kSpinLimit polls the group records an error in
// the round state and gives up on the pair.
#pragma once
#include <stdint.h>

#include "lcs.cuh"

namespace gsdr {

constexpr int kPipeRing = 4;      // carry words in flight between two warps
constexpr int kPipeZRing = 32;    // checkpoints kept per warp (>= 7*kPipeRing + 1)
constexpr int kSpinLimit = 1 << 22;

struct PipeGroup {
    uint32_t carries[8][kPipeRing];
    int zc[8][kPipeZRing];   // zero count of the warp's words after the chunk
    int zp[8][kPipeZRing];   // zeros at positions < q - R
    int ready[8];            // chunks published by warp b
    int consumed[8];         // chunks of warp b read by warp b+1
    int stop;
    int result;
    int idx;
    int error;
};

__device__ __forceinline__ int vload(const int* p) { return *(volatile const int*)p; }
__device__ __forceinline__ void vstore(int* p, int v) { *(volatile int*)p = v; }

__device__ __forceinline__ void group_bar(int id, int nthreads) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// Waits until *p >= target; false if the poll limit ran out.
__device__ __forceinline__ bool spin_until_ge(const int* p, int target, const int* stop) {
    for (int it = 0; it < kSpinLimit; it++) {
        if (vload(p) >= target) return true;
        if (vload(stop)) return true;
        __nanosleep(32);
    }
    return false;
}

__device__ __forceinline__ uint32_t valid_bits(int q, int w) {
    const int rem = q - 32 * w;
    return rem >= 32 ? 0xffffffffu : (rem > 0 ? ((1u << rem) - 1u) : 0u);
}

// Zero bits of the lane's words at pattern positions < lim.
template <int W>
__device__ __forceinline__ int zeros_below(const uint32_t (&V)[W], int w0, int lim) {
    int z = 0;
#pragma unroll
    for (int i = 0; i < W; i++) z += __popc(~V[i] & valid_bits(lim, w0 + i));
    return z;
}

// One pair on `B` warps of a group (gw = this warp's index in the group).
// The decision lands in S.result (1 accept, 0 reject) once the group meets
// at its barrier; S.error is set if a wait gave up.
template <int W>
__device__ void lcs_pipe_pair(PipeGroup& S, const uint32_t* __restrict__ pq, int q,
                             const uint32_t* __restrict__ pt, int T, int c, int B, int gw,
                             int lane, int* err_flag) {
    const int w0 = (gw * 32 + lane) * W;  // first pattern word of this lane
    uint32_t H[W], Lo[W], V[W];
#pragma unroll
    for (int i = 0; i < W; i++) {
        const int w = w0 + i;
        uint32_t hi = 0, lo = 0;
        if (w * 32 < q) planes32(__ldg(pq + 2 * w), __ldg(pq + 2 * w + 1), hi, lo);
        H[i] = hi;
        Lo[i] = lo;
        V[i] = 0xffffffffu;
    }
    const unsigned lane_bit = 1u << lane;
    const int nchunks = (T + 31) >> 5;
    for (int m = 0; m < nchunks; m++) {
        if (vload(&S.stop)) break;
        uint32_t cin_word = 0;
        if (gw > 0) {
            if (!spin_until_ge(&S.ready[gw - 1], m + 1, &S.stop)) {
                if (lane == 0) {
                    atomicExch(err_flag, 1);
                    vstore(&S.error, 1);
                    vstore(&S.stop, 1);
                }
                break;
            }
            if (vload(&S.stop)) break;
            __threadfence_block();
            cin_word = *(volatile uint32_t*)&S.carries[gw - 1][m % kPipeRing];
            __syncwarp();
            if (lane == 0) vstore(&S.consumed[gw - 1], m + 1);
        }
        if (gw < B - 1) {
            if (!spin_until_ge(&S.consumed[gw], m + 1 - kPipeRing, &S.stop)) {
                if (lane == 0) {
                    atomicExch(err_flag, 1);
                    vstore(&S.error, 1);
                    vstore(&S.stop, 1);
                }
                break;
            }
        }
        // 32 text bases: words 2m and 2m+1 of the text
        const int x0 = m << 5;
        const uint32_t t0 = __ldg(pt + 2 * m);
        const uint32_t t1 = (x0 + 16 < T) ? __ldg(pt + 2 * m + 1) : 0u;
        const int nb = min(32, T - x0);
        uint32_t cout_word = 0;
        for (int b = 0; b < nb; b++) {
            const uint32_t tw = b < 16 ? t0 : t1;
            const uint32_t cc = (tw >> (30 - 2 * (b & 15))) & 3u;
            const uint32_t ch = 0u - (cc >> 1), cl = 0u - (cc & 1u);
            uint32_t carry = 0, ones = 0xffffffffu;
#pragma unroll
            for (int i = 0; i < W; i++) {
                const uint32_t mk = ~((H[i] ^ ch) | (Lo[i] ^ cl));
                const uint64_t t = (uint64_t)V[i] + (V[i] & mk) + carry;
                carry = (uint32_t)(t >> 32);
                ones &= (uint32_t)t;
            }
            const uint32_t G = __ballot_sync(0xffffffffu, carry != 0);
            const uint32_t P = __ballot_sync(0xffffffffu, ones == 0xffffffffu);
            const uint32_t Y = G | P;
            const uint64_t sum = (uint64_t)G + Y + ((cin_word >> b) & 1u);
            const uint32_t cins = (uint32_t)sum ^ G ^ Y;
            cout_word |= (uint32_t)(sum >> 32) << b;
            uint32_t cin = (cins & lane_bit) ? 1u : 0u;
#pragma unroll
            for (int i = 0; i < W; i++) {
                const uint32_t mk = ~((H[i] ^ ch) | (Lo[i] ^ cl));
                const uint64_t t = (uint64_t)V[i] + (V[i] & mk) + cin;
                cin = (uint32_t)(t >> 32);
                V[i] = (uint32_t)t | (V[i] & ~mk);
            }
        }
        // publish this chunk: carries for the next warp and zero counts
        const int x_last = x0 + nb - 1;
        const int R = T - 1 - x_last;  // text bases still to come
        const int lim = q - R;
        const int z_full = warp_sum_i(zeros_below<W>(V, w0, q));
        const int z_pre = lim > 0 ? warp_sum_i(zeros_below<W>(V, w0, lim)) : 0;
        if (lane == 0) {
            if (gw < B - 1) S.carries[gw][m % kPipeRing] = cout_word;
            S.zc[gw][m % kPipeZRing] = z_full;
            S.zp[gw][m % kPipeZRing] = z_pre;
        }
        __threadfence_block();
        __syncwarp();
        if (lane == 0) vstore(&S.ready[gw], m + 1);
        if (gw == B - 1) {
            int zt = 0, zpt = 0;
            for (int b2 = 0; b2 < B; b2++) {
                zt += *(volatile int*)&S.zc[b2][m % kPipeZRing];
                zpt += *(volatile int*)&S.zp[b2][m % kPipeZRing];
            }
            const int ub = (lim > 0 ? zpt : 0) + min(R, q);
            int decided = -1;
            if (zt >= c) decided = 1;
            else if (ub < c || m == nchunks - 1) decided = 0;
            if (decided >= 0) {
                if (lane == 0) {
                    vstore(&S.result, decided);
                    __threadfence_block();
                    vstore(&S.stop, 1);
                }
                break;
            }
        }
    }
    __syncwarp();
}

}  // namespace gsdr
