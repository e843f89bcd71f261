// lcs_bandg.cuh -- banded bit-parallel LCS decision, one pair per group of G
// lanes (G = 2 .. 32) of a warp.
//
// The same decision and the same band as lcs_band.cuh (LCS(pattern, text) >=
// c, the test of the reference's kernel_align, cuda-version/func.cu:828-999,
// on the diagonal band a common subsequence of length >= c can use), for
// pairs whose band is too tall or whose text is too long for one lane: the
// window of G x kGroupWords pattern words is spread over the group, lane j of
// the group holding window words 4j .. 4j+3.  All lanes of a group apply the
// same text base at the same time; the carry of the window-wide addition
// V + U crosses lanes by carry lookahead: each lane adds its own words with a
// zero carry in, two warp ballots give the lanes that generate a carry
// (carry out) and those that would pass one on (sum all ones), and the carry
// into lane j is bit j of (X + Y) ^ X ^ Y with X = generate and Y = generate
// | propagate (the carries of that one 32-bit addition are the lookahead
// chain g_j | (p_j & c_j)).  The window slides down one word (a shuffle
// between neighbouring lanes) when the band leaves its first word, with the
// frozen / initial-state rules of lcs_band.cuh, so the decision is exact for
// the same reason: banded-LCS <= L' <= LCS and every path with >= c matches
// lies in the band.
//
// Match masks: each lane keeps its window words' masks for the four base
// codes in a per-warp table in shared memory (rebuilt from the bit planes
// when the window slides, at most once per 32 bases), so a step of a block
// that lies wholly inside every busy group's text reads one 16-byte entry
// instead of forming four masks from the planes (block_full); a warp with a
// group at the end of its text takes the plane path with the end mask.
#pragma once
#include <stdint.h>

#include "lcs.cuh"
#include "lcs_band.cuh"

namespace gsdr {

constexpr int kGroupWords = 4;  // pattern words per lane
constexpr unsigned kGroupFull = 0xffffffffu;

// s += cy over four words (cy 0 or 1; the carry out is dropped).
__device__ __forceinline__ void add4_inc(uint32_t& s0, uint32_t& s1, uint32_t& s2, uint32_t& s3,
                                         uint32_t cy) {
    asm("{\n\t"
        "add.cc.u32 %0, %0, %4;\n\t"
        "addc.cc.u32 %1, %1, 0;\n\t"
        "addc.cc.u32 %2, %2, 0;\n\t"
        "addc.u32 %3, %3, 0;\n\t"
        "}"
        : "+r"(s0), "+r"(s1), "+r"(s2), "+r"(s3)
        : "r"(cy));
}

template <int G>
__device__ __forceinline__ int group_sum(int v) {
#pragma unroll
    for (int d = G / 2; d > 0; d >>= 1) v += __shfl_xor_sync(kGroupFull, v, d);
    return v;
}

// The state of one group's pair, held by each lane of the group (the scalars
// are the same in every lane of the group).  Every member function is called
// by all 32 lanes of the warp together (they shuffle and vote).
template <int G>
struct BandGroup {
    static constexpr int W = kGroupWords;
    static_assert(W == 4, "refresh() and the 16-byte table entries hold four words");
    uint32_t V[W], H[W], Lo[W];
    const uint32_t* pq;  // pattern, packed
    const uint32_t* pt;  // text, packed
    int q, T, c;         // gap-free lengths and the cutoff
    int lo_off;          // T - c
    int x0;              // first text base of the next block
    int wlo;             // pattern word in window slot 0 (lane 0, word 0)
    int zf;              // zeros of the frozen words above the window
    int lane, j;         // lane in the warp, lane in the group
    uint32_t gmask;      // the group's lanes
    uint4* tab;          // this lane's masks: tab[32 * code] (the warp's table + lane)

    // wtab: the warp's 4 x 32 entries of shared memory (entry code * 32 + lane,
    // so a quarter-warp's loads hit eight different 16-byte bank groups)
    __device__ __forceinline__ void init_lane(int lane_, uint4* wtab) {
        lane = lane_;
        j = lane_ & (G - 1);
        gmask = G == 32 ? 0xffffffffu : ((1u << G) - 1u) << (lane_ & ~(G - 1));
        tab = wtab + lane_;
    }

    // The masks of the four base codes for the window words held now.
    __device__ __forceinline__ void refresh() {
#pragma unroll
        for (int code = 0; code < 4; code++) {
            const uint32_t ch = (code & 2) ? 0xffffffffu : 0u;
            const uint32_t cl = (code & 1) ? 0xffffffffu : 0u;
            uint32_t m[W];
#pragma unroll
            for (int i = 0; i < W; i++) m[i] = ~((H[i] ^ ch) | (Lo[i] ^ cl));
            tab[32 * code] = make_uint4(m[0], m[1], m[2], m[3]);
        }
    }

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
            load_word(i, W * j + i);
        }
        refresh();
    }

    // An idle group: no text, so every step leaves the state unchanged.
    __device__ __forceinline__ void clear() {
#pragma unroll
        for (int i = 0; i < W; i++) V[i] = H[i] = Lo[i] = 0u;
        pq = pt = nullptr;
        q = T = c = lo_off = x0 = wlo = zf = 0;
    }

    // One text base (ch / cl: its bits as full masks; vm all ones for a
    // real base, zero past the end of the text).
    __device__ __forceinline__ void step(uint32_t ch, uint32_t cl, uint32_t vm) {
        uint32_t m[W];
#pragma unroll
        for (int i = 0; i < W; i++) m[i] = ~((H[i] ^ ch) | (Lo[i] ^ cl));
        step_masks(m, vm);
    }

    // The rest of a step once the match masks m are known (vm: all ones for a
    // real base, zero past the end of the text).
    __device__ __forceinline__ void step_masks(const uint32_t (&m)[W], uint32_t vm) {
        uint32_t u[W], s[W];
#pragma unroll
        for (int i = 0; i < W; i++) u[i] = V[i] & m[i] & vm;
        uint32_t cy = 0;
        add4_carry(s[0], s[1], s[2], s[3], V[0], V[1], V[2], V[3], u[0], u[1], u[2], u[3], cy);
        const uint32_t all = s[0] & s[1] & s[2] & s[3];
        const uint32_t gen = __ballot_sync(kGroupFull, cy != 0u);
        const uint32_t pro = __ballot_sync(kGroupFull, all == 0xffffffffu);
        const uint32_t X = gen & gmask, Y = (gen | pro) & gmask;
        const uint32_t cin = (((X + Y) ^ X ^ Y) >> lane) & 1u;
        add4_inc(s[0], s[1], s[2], s[3], cin);
#pragma unroll
        for (int i = 0; i < W; i++) V[i] = s[i] | (V[i] & ~m[i]);
    }

    // 32 text bases that lie inside the text of every busy group of the warp
    // (an idle group has V = 0, which any step leaves at 0): the masks come
    // from the table, indexed by the base's code.
    __device__ __forceinline__ void block_full(uint32_t tw0, uint32_t tw1) {
#pragma unroll
        for (int jj = 0; jj < 32; jj++) {
            const uint32_t tw = jj < 16 ? tw0 : tw1;
            const uint32_t code = (tw >> (30 - 2 * (jj & 15))) & 3u;
            const uint4 mm = tab[32 * code];
            const uint32_t m[W] = {mm.x, mm.y, mm.z, mm.w};
            step_masks(m, 0xffffffffu);
        }
    }

    // The 32 text bases x0 .. x0 + 31 (packed words tw0: x0 .. x0 + 15,
    // tw1: x0 + 16 .. x0 + 31).
    __device__ __forceinline__ void block(uint32_t tw0, uint32_t tw1) {
#pragma unroll 4
        for (int jj = 0; jj < 32; jj++) {
            const uint32_t tw = jj < 16 ? tw0 : tw1;
            const int sh = 2 * (jj & 15);
            const uint32_t ch = (uint32_t)((int32_t)(tw << sh) >> 31);
            const uint32_t cl = (uint32_t)((int32_t)(tw << (sh + 1)) >> 31);
            const uint32_t vm = x0 + jj < T ? 0xffffffffu : 0u;
            step(ch, cl, vm);
        }
    }

    // After a block, for a busy group: -1 undecided, 1 accept, 0 reject;
    // otherwise advances x0 and slides the window for the next block.  An
    // idle group (busy false) only takes part in the shuffles.
    __device__ __forceinline__ int finish_block(bool busy) {
        const int nx = x0 + 32;
        const int R = T - nx;  // text bases not yet applied
        const int lim = q - R;
        int lz = 0, lzp = 0;
#pragma unroll
        for (int i = 0; i < W; i++) {
            const int w = wlo + W * j + i;
            lz += __popc(~V[i] & rows_below(q, w));
            lzp += __popc(~V[i] & rows_below(lim, w));
        }
        const int z = zf + group_sum<G>(lz);
        const int zb = group_sum<G>(lzp);
        // slide: rows from nx - lo_off on are needed by the next block
        const bool slide = busy && nx - lo_off >= 32 * (wlo + 1);
        const int top = __shfl_sync(kGroupFull, __popc(~V[0] & rows_below(q, wlo)), 0, G);
        uint32_t nv = __shfl_down_sync(kGroupFull, V[0], 1, G);
        uint32_t nh = __shfl_down_sync(kGroupFull, H[0], 1, G);
        uint32_t nl = __shfl_down_sync(kGroupFull, Lo[0], 1, G);
        if (!busy) return -1;
        x0 = nx;
        if (z >= c) return 1;
        if (nx >= T) return 0;
        const int zp = lim > 0 ? zf + zb : 0;
        if (zp + min(R, q) < c) return 0;
        if (slide) {
            zf += top;
#pragma unroll
            for (int i = 0; i + 1 < W; i++) {
                V[i] = V[i + 1];
                H[i] = H[i + 1];
                Lo[i] = Lo[i + 1];
            }
            wlo++;
            if (j == G - 1) {
                V[W - 1] = 0xffffffffu;
                load_word(W - 1, wlo + G * W - 1);
            } else {
                V[W - 1] = nv;
                H[W - 1] = nh;
                Lo[W - 1] = nl;
            }
            refresh();
        }
        return -1;
    }
};

}  // namespace gsdr
