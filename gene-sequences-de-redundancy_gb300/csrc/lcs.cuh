// lcs.cuh -- warp-cooperative bit-parallel LCS decision.
//
// Decides LCS(pattern, text) >= c over gap-free 2-bit packed sequences, the
// test of the reference's kernel_align (cuda-version/func.cu:828-999, a full
// O(q*T) DP per thread).  Here one warp evaluates one pair with Hyyro's
// bit-vector recurrence over the pattern positions:
//     U = V & M[c];  V' = (V + U) | (V & ~M[c]);   LCS = zeros of V
// Lane l holds pattern words l*W .. l*W+W-1 (bit b of word w <-> position 32w+b),
// so one text character advances 32*W*32 DP cells per warp step.  The carry of
// the multi-word addition crosses lanes with a carry-lookahead on two ballots:
// with G = lanes that generate a carry and P = lanes that propagate one, the
// carry into lane l is bit l of ((G + (G|P)) ^ P).
//
// Match masks are built per step from two bit planes of the pattern (high and
// low bit of each base): M[c] = ~((H ^ ch) | (L ^ cl)), ch/cl = the text
// base's bits broadcast to all 32 positions.  Bits above the pattern length
// never influence lower bits (carries only move up), so padding needs no mask
// except when counting zeros.
//
// Early exits are exact: the LCS of the pattern with a text prefix never
// decreases, so the pair is accepted as soon as it reaches c, and rejected as
// soon as even matching every remaining text base could not reach c.
#pragma once
#include <stdint.h>

namespace gsdr {

__device__ __forceinline__ uint32_t even_bits(uint32_t x) {
    x &= 0x55555555u;
    x = (x | (x >> 1)) & 0x33333333u;
    x = (x | (x >> 2)) & 0x0f0f0f0fu;
    x = (x | (x >> 4)) & 0x00ff00ffu;
    x = (x | (x >> 8)) & 0x0000ffffu;
    return x;
}

// High / low bit planes of 32 bases held in two packed words (first base in
// bits 31:30 of u0): bit b of the result belongs to base b.
__device__ __forceinline__ void planes32(uint32_t u0, uint32_t u1, uint32_t& hi, uint32_t& lo) {
    const uint32_t b0 = __brev(u0), b1 = __brev(u1);
    hi = even_bits(b0) | (even_bits(b1) << 16);
    lo = even_bits(b0 >> 1) | (even_bits(b1 >> 1) << 16);
}

// s[i] = v[i] + u[i] (+ carry) over 1, 2 or 4 words as one add-with-carry
// chain; cy is the carry in and out (0 or 1).
__device__ __forceinline__ void add1_carry(uint32_t& s0, uint32_t v0, uint32_t u0, uint32_t& cy) {
    asm("{\n\t"
        ".reg .u32 t;\n\t"
        "add.cc.u32 t, %1, 0xffffffff;\n\t"
        "addc.cc.u32 %0, %2, %3;\n\t"
        "addc.u32 %1, 0, 0;\n\t"
        "}"
        : "=r"(s0), "+r"(cy)
        : "r"(v0), "r"(u0));
}

__device__ __forceinline__ void add2_carry(uint32_t& s0, uint32_t& s1, uint32_t v0, uint32_t v1,
                                           uint32_t u0, uint32_t u1, uint32_t& cy) {
    asm("{\n\t"
        ".reg .u32 t;\n\t"
        "add.cc.u32 t, %2, 0xffffffff;\n\t"
        "addc.cc.u32 %0, %3, %5;\n\t"
        "addc.cc.u32 %1, %4, %6;\n\t"
        "addc.u32 %2, 0, 0;\n\t"
        "}"
        : "=r"(s0), "=r"(s1), "+r"(cy)
        : "r"(v0), "r"(v1), "r"(u0), "r"(u1));
}

__device__ __forceinline__ void add4_carry(uint32_t& s0, uint32_t& s1, uint32_t& s2, uint32_t& s3,
                                           uint32_t v0, uint32_t v1, uint32_t v2, uint32_t v3,
                                           uint32_t u0, uint32_t u1, uint32_t u2, uint32_t u3,
                                           uint32_t& cy) {
    asm("{\n\t"
        ".reg .u32 t;\n\t"
        "add.cc.u32 t, %4, 0xffffffff;\n\t"
        "addc.cc.u32 %0, %5, %9;\n\t"
        "addc.cc.u32 %1, %6, %10;\n\t"
        "addc.cc.u32 %2, %7, %11;\n\t"
        "addc.cc.u32 %3, %8, %12;\n\t"
        "addc.u32 %4, 0, 0;\n\t"
        "}"
        : "=r"(s0), "=r"(s1), "=r"(s2), "=r"(s3), "+r"(cy)
        : "r"(v0), "r"(v1), "r"(v2), "r"(v3), "r"(u0), "r"(u1), "r"(u2), "r"(u3));
}

// The same chains with an enable of the carry in: the chain starts from
// cy + en, which carries out iff cy = 1 and en = ~0, so en = 0 ignores cy (a
// lane whose carry-in must be zero passes 0 instead of clearing cy first).
__device__ __forceinline__ void add1_carry_en(uint32_t& s0, uint32_t v0, uint32_t u0, uint32_t& cy,
                                           uint32_t en) {
    asm("{\n\t"
        ".reg .u32 t;\n\t"
        "add.cc.u32 t, %1, %4;\n\t"
        "addc.cc.u32 %0, %2, %3;\n\t"
        "addc.u32 %1, 0, 0;\n\t"
        "}"
        : "=r"(s0), "+r"(cy)
        : "r"(v0), "r"(u0), "r"(en));
}

__device__ __forceinline__ void add2_carry_en(uint32_t& s0, uint32_t& s1, uint32_t v0, uint32_t v1,
                                           uint32_t u0, uint32_t u1, uint32_t& cy,
                                           uint32_t en) {
    asm("{\n\t"
        ".reg .u32 t;\n\t"
        "add.cc.u32 t, %2, %7;\n\t"
        "addc.cc.u32 %0, %3, %5;\n\t"
        "addc.cc.u32 %1, %4, %6;\n\t"
        "addc.u32 %2, 0, 0;\n\t"
        "}"
        : "=r"(s0), "=r"(s1), "+r"(cy)
        : "r"(v0), "r"(v1), "r"(u0), "r"(u1), "r"(en));
}

__device__ __forceinline__ void add3_carry_en(uint32_t& s0, uint32_t& s1, uint32_t& s2,
                                              uint32_t v0, uint32_t v1, uint32_t v2, uint32_t u0,
                                              uint32_t u1, uint32_t u2, uint32_t& cy, uint32_t en) {
    asm("{\n\t"
        ".reg .u32 t;\n\t"
        "add.cc.u32 t, %3, %10;\n\t"
        "addc.cc.u32 %0, %4, %7;\n\t"
        "addc.cc.u32 %1, %5, %8;\n\t"
        "addc.cc.u32 %2, %6, %9;\n\t"
        "addc.u32 %3, 0, 0;\n\t"
        "}"
        : "=r"(s0), "=r"(s1), "=r"(s2), "+r"(cy)
        : "r"(v0), "r"(v1), "r"(v2), "r"(u0), "r"(u1), "r"(u2), "r"(en));
}

__device__ __forceinline__ void add4_carry_en(uint32_t& s0, uint32_t& s1, uint32_t& s2, uint32_t& s3,
                                           uint32_t v0, uint32_t v1, uint32_t v2, uint32_t v3,
                                           uint32_t u0, uint32_t u1, uint32_t u2, uint32_t u3,
                                           uint32_t& cy, uint32_t en) {
    asm("{\n\t"
        ".reg .u32 t;\n\t"
        "add.cc.u32 t, %4, %13;\n\t"
        "addc.cc.u32 %0, %5, %9;\n\t"
        "addc.cc.u32 %1, %6, %10;\n\t"
        "addc.cc.u32 %2, %7, %11;\n\t"
        "addc.cc.u32 %3, %8, %12;\n\t"
        "addc.u32 %4, 0, 0;\n\t"
        "}"
        : "=r"(s0), "=r"(s1), "=r"(s2), "=r"(s3), "+r"(cy)
        : "r"(v0), "r"(v1), "r"(v2), "r"(v3), "r"(u0), "r"(u1), "r"(u2), "r"(u3), "r"(en));
}

// One text base applied to W pattern words (Hyyro's LCS recurrence):
//   M = match mask of the base (from the pattern's high / low bit planes H, Lo
//   and the base's bits as full masks ch, cl), U = V & M & keep,
//   V' = (V + U + cy) | (V & ~M), cy = carry out of the top word.
// keep = 0 makes the step a no-op for a zero carry-in (U = 0, V' = V).
template <int W>
__device__ __forceinline__ void hyyro_step(uint32_t (&V)[W], const uint32_t (&H)[W],
                                           const uint32_t (&Lo)[W], uint32_t ch, uint32_t cl,
                                           uint32_t keep, uint32_t& cy) {
    constexpr int C = W >= 4 ? 4 : W;
#pragma unroll
    for (int i = 0; i < W; i += C) {
        uint32_t m[C], u[C], s[C];
#pragma unroll
        for (int j = 0; j < C; j++) {
            m[j] = ~((H[i + j] ^ ch) | (Lo[i + j] ^ cl));
            u[j] = V[i + j] & m[j] & keep;
        }
        if constexpr (C == 4)
            add4_carry(s[0], s[1], s[2], s[3], V[i], V[i + 1], V[i + 2], V[i + 3], u[0], u[1],
                       u[2], u[3], cy);
        else if constexpr (C == 2)
            add2_carry(s[0], s[1], V[i], V[i + 1], u[0], u[1], cy);
        else
            add1_carry(s[0], V[i], u[0], cy);
#pragma unroll
        for (int j = 0; j < C; j++) V[i + j] = s[j] | (V[i + j] & ~m[j]);
    }
}

// The same step with the match masks read from a table in shared memory
// instead of formed from the bit planes (that moves two logic operations per
// word off the integer pipe, which bounds these kernels): pm[32 * i] is the
// match mask of word i for this step's base (one lane's row of the table;
// the all-zero row for "no base" gives U = 0).  en = 0 ignores the carry in
// (add*_carry).
template <int W>
__device__ __forceinline__ void peq_step(uint32_t (&V)[W], const uint32_t* __restrict__ pm,
                                         uint32_t& cy, uint32_t en = 0xffffffffu) {
    // the lane's words in add-with-carry chains of four, then one of W % 4;
    // the carry between chains is always taken
    constexpr int NFULL = W / 4, TAIL = W % 4;
#pragma unroll
    for (int k = 0; k < NFULL; k++) {
        const int i = 4 * k;
        uint32_t m[4], s[4];
#pragma unroll
        for (int j = 0; j < 4; j++) m[j] = pm[32 * (i + j)];
        add4_carry_en(s[0], s[1], s[2], s[3], V[i], V[i + 1], V[i + 2], V[i + 3], V[i] & m[0],
                      V[i + 1] & m[1], V[i + 2] & m[2], V[i + 3] & m[3], cy,
                      k == 0 ? en : 0xffffffffu);
#pragma unroll
        for (int j = 0; j < 4; j++) V[i + j] = s[j] | (V[i + j] & ~m[j]);
    }
    if constexpr (TAIL > 0) {
        constexpr int i = 4 * NFULL;
        const uint32_t e = NFULL == 0 ? en : 0xffffffffu;
        uint32_t m[TAIL], s[TAIL];
#pragma unroll
        for (int j = 0; j < TAIL; j++) m[j] = pm[32 * (i + j)];
        if constexpr (TAIL == 3)
            add3_carry_en(s[0], s[1], s[2], V[i], V[i + 1], V[i + 2], V[i] & m[0],
                          V[i + 1] & m[1], V[i + 2] & m[2], cy, e);
        else if constexpr (TAIL == 2)
            add2_carry_en(s[0], s[1], V[i], V[i + 1], V[i] & m[0], V[i + 1] & m[1], cy, e);
        else
            add1_carry_en(s[0], V[i], V[i] & m[0], cy, e);
#pragma unroll
        for (int j = 0; j < TAIL; j++) V[i + j] = s[j] | (V[i + j] & ~m[j]);
    }
}

// Match-mask table of one lane's W pattern words: peq[(b * W + i) * 32] =
// positions of word i holding base b (b = 0..3; lane-interleaved, so a warp's
// lanes read consecutive words), and row b = 4 all zero (a step that must
// leave V unchanged).  Positions past the pattern match base 0, as the zero
// bit planes do in hyyro_step; their carries only move upward and their bits
// are never counted.
template <int W>
__device__ __forceinline__ void peq_fill(uint32_t* peq, const uint32_t* __restrict__ pq, int q,
                                         int w0) {
#pragma unroll
    for (int i = 0; i < W; i++) {
        const int w = w0 + i;
        uint32_t h = 0, l = 0;
        if (w * 32 < q) planes32(__ldg(pq + 2 * w), __ldg(pq + 2 * w + 1), h, l);
        peq[(0 * W + i) * 32] = ~h & ~l;
        peq[(1 * W + i) * 32] = ~h & l;
        peq[(2 * W + i) * 32] = h & ~l;
        peq[(3 * W + i) * 32] = h & l;
        peq[(4 * W + i) * 32] = 0u;
    }
}

__device__ __forceinline__ int warp_sum_i(int v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
    return v;
}

__device__ __forceinline__ unsigned long long warp_sum_ull(unsigned long long v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
    return v;
}

// Returns true iff LCS(pattern, text) >= c.  pq: pattern packed words
// (q bases); pt: text packed words (T bases).  Requires 1 <= c, q <= 1024*W.
// STORE = keep the step's masks and sums in registers (small W) or recompute
// them in a second pass (large W, fewer live registers).
template <int W, bool STORE>
__device__ bool lcs_reaches_warp(const uint32_t* __restrict__ pq, int q,
                                 const uint32_t* __restrict__ pt, int T, int c, int lane) {
    uint32_t H[W], Lo[W], V[W];
#pragma unroll
    for (int i = 0; i < W; i++) {
        const int w = lane * W + i;
        uint32_t hi = 0, lo = 0;
        if (w * 32 < q) planes32(__ldg(pq + 2 * w), __ldg(pq + 2 * w + 1), hi, lo);
        H[i] = hi;
        Lo[i] = lo;
        V[i] = 0xffffffffu;
    }
    const unsigned lane_bit = 1u << lane;
    const int tw_count = (T + 15) >> 4;
    int x = 0;
    int zeros = 0;
    while (x < T) {
        // 32 text words (512 bases) per refill, one per lane.
        const int wbase = x >> 4;
        const uint32_t tw_lane = (wbase + lane < tw_count) ? __ldg(pt + wbase + lane) : 0u;
        const int xend = min(T, x + 512);
        while (x < xend) {
            const uint32_t tw = __shfl_sync(0xffffffffu, tw_lane, (x >> 4) & 31);
            const int bend = min(16, xend - x);
            for (int b = 0; b < bend; b++, x++) {
                const uint32_t cc = (tw >> (30 - 2 * b)) & 3u;
                const uint32_t ch = 0u - (cc >> 1), cl = 0u - (cc & 1u);
                if (STORE) {
                    uint32_t m[W], s[W];
                    uint32_t carry = 0, ones = 0xffffffffu;
#pragma unroll
                    for (int i = 0; i < W; i++) {
                        m[i] = ~((H[i] ^ ch) | (Lo[i] ^ cl));
                        const uint64_t t = (uint64_t)V[i] + (V[i] & m[i]) + carry;
                        s[i] = (uint32_t)t;
                        carry = (uint32_t)(t >> 32);
                        ones &= s[i];
                    }
                    const unsigned G = __ballot_sync(0xffffffffu, carry != 0);
                    const unsigned P = __ballot_sync(0xffffffffu, ones == 0xffffffffu);
                    uint32_t cin = (((G + (G | P)) ^ P) & lane_bit) ? 1u : 0u;
#pragma unroll
                    for (int i = 0; i < W; i++) {
                        const uint64_t t = (uint64_t)s[i] + cin;
                        cin = (uint32_t)(t >> 32);
                        V[i] = (uint32_t)t | (V[i] & ~m[i]);
                    }
                } else {
                    uint32_t carry = 0, ones = 0xffffffffu;
#pragma unroll
                    for (int i = 0; i < W; i++) {
                        const uint32_t m = ~((H[i] ^ ch) | (Lo[i] ^ cl));
                        const uint64_t t = (uint64_t)V[i] + (V[i] & m) + carry;
                        carry = (uint32_t)(t >> 32);
                        ones &= (uint32_t)t;
                    }
                    const unsigned G = __ballot_sync(0xffffffffu, carry != 0);
                    const unsigned P = __ballot_sync(0xffffffffu, ones == 0xffffffffu);
                    uint32_t cin = (((G + (G | P)) ^ P) & lane_bit) ? 1u : 0u;
#pragma unroll
                    for (int i = 0; i < W; i++) {
                        const uint32_t m = ~((H[i] ^ ch) | (Lo[i] ^ cl));
                        const uint64_t t = (uint64_t)V[i] + (V[i] & m) + cin;
                        cin = (uint32_t)(t >> 32);
                        V[i] = (uint32_t)t | (V[i] & ~m);
                    }
                }
                if ((x & 31) == 31) {
                    int z = 0;
#pragma unroll
                    for (int i = 0; i < W; i++) {
                        const int w = lane * W + i;
                        const int rem = q - 32 * w;
                        const uint32_t valid =
                            rem >= 32 ? 0xffffffffu : (rem > 0 ? ((1u << rem) - 1u) : 0u);
                        z += __popc(~V[i] & valid);
                    }
                    zeros = warp_sum_i(z);
                    if (zeros >= c) return true;
                    if (zeros + (T - 1 - x) < c) return false;
                }
            }
        }
    }
    int z = 0;
#pragma unroll
    for (int i = 0; i < W; i++) {
        const int w = lane * W + i;
        const int rem = q - 32 * w;
        const uint32_t valid = rem >= 32 ? 0xffffffffu : (rem > 0 ? ((1u << rem) - 1u) : 0u);
        z += __popc(~V[i] & valid);
    }
    zeros = warp_sum_i(z);
    return zeros >= c;
}

}  // namespace gsdr
