// lcs_band.cuh -- banded bit-parallel LCS decision, one pair per lane.
//
// Decides LCS(pattern, text) >= c (the test of the reference's kernel_align,
// cuda-version/func.cu:828-999) with the same recurrence over pattern bits as
// lcs_sys.cuh (Hyyro: U = V & M[x]; V' = (V + U) | (V & ~M[x]); LCS = zeros
// of V), but only on the diagonal band that a long enough common subsequence
// can use.
//
// A common subsequence of length >= c leaves at most q - c pattern bases and
// T - c text bases unmatched, so its path through the DP grid never strays
// more than T - c diagonals to one side and q - c to the other: at text base x
// it is on pattern rows x - (T - c) .. x + (q - c).  The lane keeps W pattern
// words (32W rows) covering those rows for a whole block of 32 text bases and
// slides the window down one word when the band leaves its first word.  Rows
// above the window are frozen (their zeros are counted once, in Zf); rows
// below keep their initial state until they enter.  Every cell of the
// resulting grid holds either the recurrence's value over its neighbours, or
// the true DP value of an earlier text base, or the value of the row above it,
// so the computed L' satisfies  banded-LCS <= L' <= LCS, and since every path
// with >= c matches lies in the band, L' >= c exactly when LCS >= c.  The
// accept test (L' of a text prefix >= c) and the reject bound (zeros below
// row q - R plus min(R, q) < c, R = text bases left) hold for L' as they do
// for the full DP.
#pragma once
#include <stdint.h>

#include "lcs.cuh"

namespace gsdr {

// Words a lane's window needs for a pair: 32W must exceed the band's height
// plus one block of 32 bases of slide plus word alignment.
__host__ __device__ __forceinline__ int band_words(int T, int q, int c) {
    return ((T - c) + (q - c) + 62) / 32 + 1;
}

// One text base on the window: ch / cl are the base's high / low bit as full
// masks, vm is all ones for a real base and zero past the end of the text
// (U = 0 and a zero carry leave V unchanged).
template <int W>
__device__ __forceinline__ void band_step(uint32_t (&V)[W], const uint32_t (&H)[W],
                                          const uint32_t (&Lo)[W], uint32_t ch, uint32_t cl,
                                          uint32_t vm) {
    uint32_t cy = 0;
    hyyro_step<W>(V, H, Lo, ch, cl, vm, cy);
}

// Rows of word w below row `lim` (bits of real pattern positions < lim).
__device__ __forceinline__ uint32_t rows_below(int lim, int w) {
    const int rem = lim - 32 * w;
    return rem >= 32 ? 0xffffffffu : (rem > 0 ? ((1u << rem) - 1u) : 0u);
}

// Zeros of the window's words below row `lim`.
template <int W>
__device__ __forceinline__ int band_zeros(const uint32_t (&V)[W], int wlo, int lim) {
    int z = 0;
#pragma unroll
    for (int i = 0; i < W; i++) z += __popc(~V[i] & rows_below(lim, wlo + i));
    return z;
}

// The state of one lane's pair.
template <int W>
struct BandLane {
    uint32_t V[W], H[W], Lo[W];
    const uint32_t* pq;  // pattern, packed
    const uint32_t* pt;  // text, packed
    int q, T, c;         // gap-free lengths and the cutoff
    int lo_off;          // T - c: rows x - lo_off and above have left the band
    int x0;              // first text base of the next block
    int wlo;             // pattern word in window slot 0
    int zf;              // zeros of the frozen words above the window

    __device__ __forceinline__ void load_word(int slot, int w) {
        uint32_t h = 0, l = 0;
        if (32 * w < q) planes32(__ldg(pq + 2 * w), __ldg(pq + 2 * w + 1), h, l);
        H[slot] = h;
        Lo[slot] = l;
    }

    __device__ __forceinline__ void start(const uint32_t* pat, int q_, const uint32_t* txt, int T_,
                                          int c_) {
        pq = pat;
        pt = txt;
        q = q_;
        T = T_;
        c = c_;
        lo_off = T_ - c_;
        x0 = 0;
        wlo = 0;
        zf = 0;
#pragma unroll
        for (int i = 0; i < W; i++) {
            V[i] = 0xffffffffu;
            load_word(i, i);
        }
    }

    // An idle lane: no text, so every step leaves the state unchanged.
    __device__ __forceinline__ void clear() {
#pragma unroll
        for (int i = 0; i < W; i++) V[i] = H[i] = Lo[i] = 0u;
        pq = pt = nullptr;
        q = T = c = lo_off = x0 = wlo = zf = 0;
    }

    // G text bases x0 + j0 .. x0 + j0 + G - 1 from the packed text word tw
    // holding bases x0 + 16 * (j0 / 16) .. + 15.
    template <int G>
    __device__ __forceinline__ void steps(uint32_t tw, int j0) {
#pragma unroll
        for (int j = 0; j < G; j++) {
            const int jj = j0 + j;
            const int sh = 2 * (jj & 15);
            const uint32_t ch = (uint32_t)((int32_t)(tw << sh) >> 31);
            const uint32_t cl = (uint32_t)((int32_t)(tw << (sh + 1)) >> 31);
            const uint32_t vm = x0 + jj < T ? 0xffffffffu : 0u;
            band_step<W>(V, H, Lo, ch, cl, vm);
        }
    }

    // After a block: -1 undecided, 1 accept, 0 reject; otherwise advances x0
    // and slides the window for the next block.
    __device__ __forceinline__ int finish_block() {
        x0 += 32;
        const int z = zf + band_zeros<W>(V, wlo, q);
        if (z >= c) return 1;
        if (x0 >= T) return 0;
        const int R = T - x0;  // text bases not yet applied
        const int lim = q - R;
        int zp = 0;
        if (lim > 0) zp = lim <= 32 * wlo ? zf : zf + band_zeros<W>(V, wlo, lim);
        if (zp + min(R, q) < c) return 0;
        // the next block needs rows from x0 - lo_off on
        if (x0 - lo_off >= 32 * (wlo + 1)) {
            zf += __popc(~V[0] & rows_below(q, wlo));
#pragma unroll
            for (int i = 0; i + 1 < W; i++) {
                V[i] = V[i + 1];
                H[i] = H[i + 1];
                Lo[i] = Lo[i + 1];
            }
            V[W - 1] = 0xffffffffu;
            wlo++;
            load_word(W - 1, wlo + W - 1);
        }
        return -1;
    }
};

}  // namespace gsdr
