// prep.cu -- one-time per-job preparation kernels.
//
// k_pack fuses the reference's kernel_baseToNumber, kernel_compressData,
// kernel_createPrefix and kernel_createCutoff (cuda-version/func.cu:139-186,
// 272-403, 312-349): one warp per read streams the raw bytes with aligned
// 16-byte loads, drops non-ACGT bytes, packs 16 bases per u32 (first base in
// the two most significant bits), counts the bases and computes the cutoffs
// with the reference's float/double types.
//
// k_kmers_hist replaces kernel_createWords*/sortWords/mergeWords
// (cuda-version/func.cu:405-653): instead of a per-thread Shell sort of every
// k-mer, a CTA counts the read's k-mers in a shared-memory histogram and
// emits one (k-mer, multiplicity) entry per distinct k-mer.  The word filter
// only needs that multiset, not an order.
#include <cuda_runtime.h>

#include "gsdr_device.cuh"

namespace gsdr {

namespace {

constexpr int kPackWarps = 8;

__device__ __forceinline__ int base_code(uint32_t b) {
    // A/a->0, C/c->1, G/g->2, T/t/U/u->3, anything else->4 (func.cu:139-179),
    // without branches: b | 0x20 is 'a' .. 'u' only for those letters' two
    // cases (and for the other letters), and a 64-bit table holds the 3-bit
    // codes of 'a' .. 'u' (21 entries: a 0, c 1, g 2, t 3, u 3, the rest 4)
    constexpr unsigned long long kCodes = 0x37249249248a4860ull;
    const uint32_t idx = (b | 0x20u) - 0x61u;
    return idx < 21u ? (int)((kCodes >> (3u * idx)) & 7u) : 4;
}

__device__ __forceinline__ int warp_sum(int v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
    return v;
}

// kernel_createCutoff (cuda-version/func.cu:312-337) with explicit rounding
// intrinsics so that no contraction can change a result.
__device__ void cutoffs(int length, float t, int k, int* word, int* base, int* pig) {
    int required = length - k + 1;
    double c1 = ceil(__dmul_rn((double)(float)length, __dsub_rn(1.0, (double)t)));
    int cutoff = (int)__dmul_rn(c1, (double)k);
    required -= cutoff;
    required = max(required, 1);
    float offset;
    if ((double)t >= 0.9) {
        offset = (float)__dsub_rn(1.1, __dmul_rn(fabs(__dsub_rn((double)t, 0.95)), 2.0));
    } else {
        offset = 1.0f;
    }
    *word = (int)ceilf(__fmul_rn((float)required, offset));
    *base = (int)ceilf(__fmul_rn((float)length, t));
    *pig = (int)__dmul_rn(c1, 4.0);
}

// createCutoff of the SYCL program (func.cpp:339-373): the same formulas in
// float, the offset forced to 1; its alignment accepts LCS > ceil(len * t)
// (func.cpp:671), stored here as the cutoff ceil(len * t) + 1 of an LCS >=
// test (the prefilter subtracts DevReads::strict again).
__device__ void cutoffs_sycl(int length, float t, int k, int* word, int* base) {
    int required = length - k + 1;
    const float slack = ceilf(__fmul_rn((float)length, __fsub_rn(1.0f, t)));
    const int cutoff = (int)__fmul_rn(slack, (float)k);
    required -= cutoff;
    required = max(required, 1);
    *word = required;
    *base = (int)ceilf(__fmul_rn((float)length, t)) + 1;
}

__global__ void __launch_bounds__(kPackWarps * 32) k_pack(DevReads R, float t, int k) {
    __shared__ uint32_t stage_all[kPackWarps][36];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    uint32_t* stage = stage_all[wib];
    const int nwarps = gridDim.x * kPackWarps;
    for (int r = blockIdx.x * kPackWarps + wib; r < R.n; r += nwarps) {
        const uint8_t* src = R.bytes + R.off[r];
        const int L = R.len[r];
        const uintptr_t start = (uintptr_t)src;
        const uintptr_t a0 = start & ~(uintptr_t)15;
        const int head = (int)(start - a0);
        const long long nchunks = ((long long)head + L + 15) >> 4;
        uint32_t* out = R.packed + R.pack_off[r];
        for (int w = lane; w < 36; w += 32) stage[w] = 0;
        __syncwarp();
        int gcount = 0;
        int cnt0 = 0, cnt1 = 0, cnt2 = 0, cnt3 = 0;
        uint32_t* brk = R.brk ? R.brk + R.pack_off[r] : nullptr;
        bool gap_before = false;  // the byte before this iteration's first chunk
        for (long long c0 = 0; c0 < nchunks; c0 += 32) {
            const long long c = c0 + lane;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (c < nchunks) v = __ldcs(reinterpret_cast<const uint4*>(a0) + c);
            const uint32_t words[4] = {v.x, v.y, v.z, v.w};
            int nb = 0;
            uint32_t acc = 0;
            uint32_t gaps = 0;   // bit jj: byte jj of the chunk is a non-ACGT byte of the read
            uint32_t marks = 0;  // bit b: the chunk's b-th base follows a non-ACGT byte
            uint32_t before = 0; // the byte before the chunk is one
            if (brk) {
                // the previous lane's last byte, or for lane 0 the last byte of
                // the previous iteration
                const long long p15 = 16 * c + 15 - head;
                const bool v15 = (c < nchunks) && p15 >= 0 && p15 < L;
                const uint32_t last_gap = v15 && base_code(words[3] >> 24) == 4 ? 1u : 0u;
                before = __shfl_up_sync(0xffffffffu, last_gap, 1);
                if (lane == 0) before = gap_before ? 1u : 0u;
                gap_before = __shfl_sync(0xffffffffu, last_gap, 31) != 0;
            }
            // the chunk holds read positions p0 .. p0 + 15; every step below is
            // a select, not a branch (lanes see different bases)
            const int p0 = (int)(16 * c - head);
            const bool in_range = c < nchunks;
#pragma unroll
            for (int jj = 0; jj < 16; jj++) {
                const int pos = p0 + jj;
                const bool valid = in_range && pos >= 0 && pos < L;
                const int code = valid ? base_code((words[jj >> 2] >> (8 * (jj & 3))) & 0xffu) : 4;
                gaps |= (valid && code == 4 ? 1u : 0u) << jj;
                const bool ok = code < 4;
                const uint32_t prev_gap = (jj == 0 ? before : (gaps >> (jj - 1))) & 1u;
                marks |= ok && prev_gap ? 1u << nb : 0u;
                acc = ok ? (acc << 2) | (uint32_t)code : acc;
                nb += ok ? 1 : 0;
                cnt0 += code == 0;
                cnt1 += code == 1;
                cnt2 += code == 2;
                cnt3 += code == 3;
            }

            acc = nb ? (acc << (2 * (16 - nb))) : 0u;
            int incl = nb;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                int x = __shfl_up_sync(0xffffffffu, incl, d);
                if (lane >= d) incl += x;
            }
            const int excl = incl - nb;
            const int total = __shfl_sync(0xffffffffu, incl, 31);
            const int gpos = gcount + excl;
            const int wrel = (gpos >> 4) - (gcount >> 4);
            const int sh = gpos & 15;
            if (nb) {
                atomicOr(&stage[wrel], acc >> (2 * sh));
                if (sh + nb > 16) atomicOr(&stage[wrel + 1], acc << (2 * (16 - sh)));
            }
            if (brk && marks) {  // bits gpos .. gpos + nb - 1 of the read's break map
                const int bs = gpos & 31;
                atomicOr(&brk[gpos >> 5], marks << bs);
                if (bs + nb > 32) atomicOr(&brk[(gpos >> 5) + 1], marks >> (32 - bs));
            }
            __syncwarp();
            const int nfull = ((gcount + total) >> 4) - (gcount >> 4);
            for (int w = lane; w < nfull; w += 32) out[(gcount >> 4) + w] = stage[w];
            const uint32_t carry = stage[nfull];
            __syncwarp();
            for (int w = lane; w < 36; w += 32) stage[w] = 0;
            __syncwarp();
            if (lane == 0) stage[0] = carry;
            __syncwarp();
            gcount += total;
        }
        // kernel_compressData always stores the trailing (possibly empty) word.
        if (lane == 0) out[gcount >> 4] = stage[0];
        cnt0 = warp_sum(cnt0);
        cnt1 = warp_sum(cnt1);
        cnt2 = warp_sum(cnt2);
        cnt3 = warp_sum(cnt3);
        if (lane == 0) {
            R.len_gf[r] = gcount;
            R.comp[r] = make_int4(cnt0, cnt1, cnt2, cnt3);
            int cw, cb, cp = 0;
            if (R.variant == 1) cutoffs_sycl(L, t, k, &cw, &cb);
            else cutoffs(L, t, k, &cw, &cb, &cp);
            R.cut_word[r] = cw;
            R.cut_base[r] = cb;
            R.cut_pig[r] = cp;
        }
        __syncwarp();
    }
}

// Variant 1: the window of k gap-free bases from p holds a break (bits p + 1
// .. p + k - 1 of the read's break map), so the SYCL program has no k-mer there.
__device__ __forceinline__ bool window_broken(const uint32_t* brk, int p, int k) {
    const int a = p + 1, nbits = k - 1;
    const int w = a >> 5, sh = a & 31;
    uint64_t v = __ldg(brk + w);
    if (sh + nbits > 32) v |= (uint64_t)__ldg(brk + w + 1) << 32;
    return ((v >> sh) & ((1ull << nbits) - 1ull)) != 0ull;
}

template <int K>
__global__ void __launch_bounds__(256) k_kmers_hist(DevReads R) {
    constexpr int NB = 1 << (2 * K);
    // presence bitmaps: k <= 6 always (the plain filter's bound), k = 7 only
    // for the batched two-level filter (kbits allocated)
    constexpr bool BITS_T = K <= kMaxBits2K;
    constexpr int NBW = BITS_T ? NB / 32 : 1;
    extern __shared__ __align__(16) uint32_t sm[];
    uint32_t* hist = sm;
    uint16_t* list = reinterpret_cast<uint16_t*>(sm + NB);
    __shared__ uint32_t bits[NBW], bits2[NBW];
    __shared__ int nlist, sumcnt, sum3;
    const bool BITS = BITS_T && R.kbits != nullptr;
    const bool level2 = BITS && R.kbits2 != nullptr;
    for (int i = threadIdx.x; i < NB; i += blockDim.x) hist[i] = 0;
    for (int i = threadIdx.x; i < NBW; i += blockDim.x) bits[i] = bits2[i] = 0;
    if (threadIdx.x == 0) {
        nlist = 0;
        sumcnt = 0;
        sum3 = 0;
    }
    __syncthreads();
    for (int r = blockIdx.x; r < R.n; r += gridDim.x) {
        const int gf = R.len_gf[r];
        const int nk = gf - K + 1;
        uint32_t* out = R.kmer + R.kmer_off[r];
        const uint32_t* pk = R.packed + R.pack_off[r];
        const uint32_t* bk = R.brk ? R.brk + R.pack_off[r] : nullptr;
        for (int p = threadIdx.x; p < nk; p += blockDim.x) {
            if (bk && window_broken(bk, p, K)) continue;
            const int w = p >> 4, o = p & 15;
            const uint64_t v = ((uint64_t)__ldg(pk + w) << 32) | __ldg(pk + w + 1);
            const uint32_t km = (uint32_t)(v >> (64 - 2 * o - 2 * K)) & (uint32_t)(NB - 1);
            const uint32_t old = atomicAdd(&hist[km], 1u);
            if (old == 0) list[atomicAdd(&nlist, 1)] = (uint16_t)km;
        }
        __syncthreads();
        const int nl = nlist;
        int my_sum = 0, my_sum3 = 0;
        for (int s = threadIdx.x; s < nl; s += blockDim.x) {
            const uint32_t km = list[s];
            const uint32_t c = hist[km] & 0xffffu;  // the reference's u16 multiplicity
            out[s] = (km << 16) | c;
            hist[km] = 0;
            if (BITS && c) {
                atomicOr(&bits[km >> 5], 1u << (km & 31));
                my_sum += (int)c - 1;
                if (level2 && c >= 2) {
                    atomicOr(&bits2[km >> 5], 1u << (km & 31));
                    my_sum3 += (int)c - 2;
                }
            }
        }
        const int padded = (nl + 3) & ~3;
        for (int s = nl + threadIdx.x; s < padded; s += blockDim.x) out[s] = 0u;
        if (BITS) {
            my_sum = warp_sum(my_sum);
            if ((threadIdx.x & 31) == 0 && my_sum) atomicAdd(&sumcnt, my_sum);
            if (level2) {
                my_sum3 = warp_sum(my_sum3);
                if ((threadIdx.x & 31) == 0 && my_sum3) atomicAdd(&sum3, my_sum3);
            }
        }
        __syncthreads();
        if (BITS) {
            uint32_t* ob = R.kbits + (size_t)r * NBW;
            for (int i = threadIdx.x; i < NBW; i += blockDim.x) {
                ob[i] = bits[i];
                bits[i] = 0;
            }
            if (level2) {
                uint32_t* ob2 = R.kbits2 + (size_t)r * NBW;
                for (int i = threadIdx.x; i < NBW; i += blockDim.x) {
                    ob2[i] = bits2[i];
                    bits2[i] = 0;
                }
            }
        }
        if (threadIdx.x == 0) {
            R.n_kmer[r] = nl;
            if (BITS) R.kextra[r] = sumcnt;
            if (level2) R.kextra3[r] = sum3;
            nlist = 0;
            sumcnt = 0;
            sum3 = 0;
        }
        __syncthreads();
    }
}

template <int K>
int kmers_hist_launch(const DevReads& R, cudaStream_t s) {
    constexpr int NB = 1 << (2 * K);
    const int smem = NB * 4 + NB * 2;
    if (smem > 0) {
        cudaError_t e = cudaFuncSetAttribute(k_kmers_hist<K>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return 1;
    }
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_kmers_hist<K>, 256, smem);
    if (per_sm < 1) per_sm = 1;
    int grid = num_sms() * per_sm;
    if (grid > R.n) grid = R.n > 0 ? R.n : 1;
    k_kmers_hist<K><<<grid, 256, smem, s>>>(R);
    return 0;
}

}  // namespace

int num_sms() {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    return sms;
}

// One thread per 32-base word of a read: the four one-hot bit-planes of the
// word, from its two packed words (first base in the high bits).
__global__ void k_planes(DevReads R) {
    const int lane = threadIdx.x & 31;
    const int nwarps = gridDim.x * (blockDim.x >> 5);
    for (int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < R.n; r += nwarps) {
        const int gf = R.len_gf[r];
        const int64_t po = R.pack_off[r];
        const int stride = (int)((R.pack_off[r + 1] - po) >> 1);
        const int nw = (gf + 31) >> 5;
        const uint32_t* pk = R.packed + po;
        uint32_t* out = R.bm + 2 * po;
        for (int w = lane; w < stride; w += 32) {
            uint32_t p0 = 0, p1 = 0, p2 = 0, p3 = 0;
            if (w < nw) {
                uint32_t hi, lo;
                // two packed words hold bases 32w .. 32w+31
                const uint32_t u0 = pk[2 * w], u1 = pk[2 * w + 1];
                const uint32_t b0 = __brev(u0), b1 = __brev(u1);
                auto ev = [](uint32_t x) {
                    x &= 0x55555555u;
                    x = (x | (x >> 1)) & 0x33333333u;
                    x = (x | (x >> 2)) & 0x0f0f0f0fu;
                    x = (x | (x >> 4)) & 0x00ff00ffu;
                    x = (x | (x >> 8)) & 0x0000ffffu;
                    return x;
                };
                hi = ev(b0) | (ev(b1) << 16);
                lo = ev(b0 >> 1) | (ev(b1 >> 1) << 16);
                const int rem = gf - 32 * w;
                const uint32_t valid = rem >= 32 ? 0xffffffffu : ((1u << rem) - 1u);
                p0 = ~hi & ~lo & valid;
                p1 = ~hi & lo & valid;
                p2 = hi & ~lo & valid;
                p3 = hi & lo & valid;
            }
            out[w] = p0;
            out[stride + w] = p1;
            out[2 * stride + w] = p2;
            out[3 * stride + w] = p3;
        }
    }
}

// kernel_createPigeon1 / kernel_createPigeon2 (cuda-version/func.cu:188-250)
// for every read, one warp per read.  Over the raw codes (before the gap-free
// packing), every position p >= 3 whose window p-3..p holds four A/C/G/T
// bases adds one to bucket v = its 4-mer (first base most significant); pig
// receives the inclusive prefix of the bucket counts (u16).  Within a bucket
// the reference fills slots from the top down as p ascends, so the r-th
// window (0-based, ascending p) of bucket v takes slot pig[v] - 1 - r; it
// stores the window's last position in the reference's padded layout,
// truncated to 16 bits.  Ranks within a 32-position chunk come from
// __match_any_sync, across chunks from running per-bucket counts.
constexpr int kPigWarps = 8;

__global__ void __launch_bounds__(kPigWarps * 32) k_pigeon_index(DevReads R) {
    __shared__ uint32_t cnt[kPigWarps][256];
    __shared__ uint32_t run[kPigWarps][256];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned lt = (1u << lane) - 1u;
    const int nwarps = gridDim.x * kPigWarps;
    uint32_t* c = cnt[warp];
    uint32_t* rn = run[warp];
    for (int r = blockIdx.x * kPigWarps + warp; r < R.n; r += nwarps) {
        const int L = R.len[r];
        const uint8_t* b = R.bytes + R.off[r];
        for (int i = lane; i < 256; i += 32) {
            c[i] = 0u;
            rn[i] = 0u;
        }
        __syncwarp();
        // bucket of the window ending at p, or -1
        auto window = [&](int p) -> int {
            if (p < 3 || p >= L) return -1;
            int v = 0;
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int code = base_code(b[p - 3 + j]);
                if (code > 3) return -1;
                v = (v << 2) | code;
            }
            return v;
        };
        for (int p0 = 0; p0 < L; p0 += 32) {
            const int v = window(p0 + lane);
            if (v >= 0) atomicAdd(&c[v], 1u);
        }
        __syncwarp();
        // inclusive prefix over the 256 buckets: lane owns 8 consecutive ones
        uint32_t loc[8], sum = 0;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            sum += c[lane * 8 + j];
            loc[j] = sum;
        }
        uint32_t incl = sum;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t o = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= d) incl += o;
        }
        const uint32_t before = incl - sum;
        __syncwarp();
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const uint32_t e = before + loc[j];
            c[lane * 8 + j] = e;
            R.pig[(size_t)r * 256 + lane * 8 + j] = (uint16_t)e;
        }
        __syncwarp();
        const uint32_t base16 = R.refoff16[r];
        uint16_t* out = R.pidx + R.off[r];
        for (int p0 = 0; p0 < L; p0 += 32) {
            const int p = p0 + lane;
            const int v = window(p);
            // invalid lanes get keys of their own
            const unsigned grp = __match_any_sync(0xffffffffu, v >= 0 ? v : 256 + lane);
            if (v >= 0) {
                const uint32_t rank = rn[v] + __popc(grp & lt);
                const uint32_t slot = c[v] - 1u - rank;
                out[slot] = (uint16_t)(base16 + (uint32_t)p);
            }
            __syncwarp();
            if (v >= 0 && (grp & lt) == 0) rn[v] += __popc(grp);
            __syncwarp();
        }
    }
}

void launch_planes(const DevReads& R, cudaStream_t s) {
    if (R.n <= 0) return;
    int grid = (R.n + 7) / 8;
    const int cap = num_sms() * 16;
    if (grid > cap) grid = cap;
    k_planes<<<grid, 256, 0, s>>>(R);
}

void launch_pigeon_index(const DevReads& R, cudaStream_t s) {
    if (R.n <= 0 || !R.pig) return;
    int grid = (R.n + kPigWarps - 1) / kPigWarps;
    const int cap = num_sms() * 8;
    if (grid > cap) grid = cap;
    k_pigeon_index<<<grid, kPigWarps * 32, 0, s>>>(R);
}

void launch_pack(const DevReads& R, float t, int k, cudaStream_t s) {
    if (R.n <= 0) return;
    int grid = (R.n + kPackWarps - 1) / kPackWarps;
    const int cap = num_sms() * 16;
    if (grid > cap) grid = cap;
    k_pack<<<grid, kPackWarps * 32, 0, s>>>(R, t, k);
}

// Word lengths 8..12 (createWords / sortWords / mergeWords, func.cu:405-653):
// the distinct k-mers of each read with their u16 multiplicities, counted in
// an open-addressing hash table of the CTA's own (global memory, L2
// resident).  The first thread that claims a slot records it in the CTA's
// slot list; after the read the listed slots are emitted (ids into R.kmer,
// counts into R.kcnt, in slot-claim order: the filters need the multiset, not
// an order) and cleared for the next read.
__global__ void __launch_bounds__(256) k_kmers_hash(DevReads R, int k) {
    const int S = R.khash_slots;  // a power of two, at least 2 x the longest read
    uint32_t* keys = R.khash + (size_t)blockIdx.x * 3 * S;
    uint32_t* cnt = keys + S;
    uint32_t* slots = cnt + S;
    __shared__ int nlist;
    const uint32_t mask = (k >= 16) ? 0xffffffffu : ((1u << (2 * k)) - 1u);
    const int shift = 32 - (31 - __clz(S));
    for (int r = blockIdx.x; r < R.n; r += gridDim.x) {
        if (threadIdx.x == 0) nlist = 0;
        __syncthreads();
        const int nk = R.len_gf[r] - k + 1;
        const uint32_t* pk = R.packed + R.pack_off[r];
        const uint32_t* bk = R.brk ? R.brk + R.pack_off[r] : nullptr;
        for (int p = threadIdx.x; p < nk; p += blockDim.x) {
            if (bk && window_broken(bk, p, k)) continue;
            const int w = p >> 4, o = p & 15;
            const uint64_t v = ((uint64_t)__ldg(pk + w) << 32) | __ldg(pk + w + 1);
            const uint32_t km = (uint32_t)(v >> (64 - 2 * o - 2 * k)) & mask;
            uint32_t h = (km * 0x9e3779b1u) >> shift;
            for (int probe = 0; probe < S; probe++) {
                const uint32_t old = atomicCAS(&keys[h], 0xffffffffu, km);
                if (old == 0xffffffffu) slots[atomicAdd(&nlist, 1)] = h;
                if (old == 0xffffffffu || old == km) {
                    atomicAdd(&cnt[h], 1u);
                    break;
                }
                h = (h + 1) & (uint32_t)(S - 1);
            }
        }
        __syncthreads();
        const int nl = nlist;
        uint32_t* ok = R.kmer + R.kmer_off[r];
        uint16_t* oc = R.kcnt + R.kmer_off[r];
        for (int i = threadIdx.x; i < nl; i += blockDim.x) {
            const uint32_t h = slots[i];
            ok[i] = keys[h];
            oc[i] = (uint16_t)(cnt[h] & 0xffffu);  // the reference's u16 multiplicity
            keys[h] = 0xffffffffu;
            cnt[h] = 0u;
        }
        for (int i = nl + threadIdx.x; i < ((nl + 3) & ~3); i += blockDim.x) {
            ok[i] = 0u;
            oc[i] = 0u;
        }
        if (threadIdx.x == 0) R.n_kmer[r] = nl;
        __syncthreads();
    }
}

__global__ void k_khash_init(DevReads R) {
    const int S = R.khash_slots;
    const size_t total = (size_t)R.khash_ctas * 3 * S;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (size_t)gridDim.x * blockDim.x) {
        const size_t part = (i / S) % 3;  // per CTA: keys, counts, slot list
        R.khash[i] = part == 0 ? 0xffffffffu : 0u;
    }
}

int launch_kmers(const DevReads& R, int k, cudaStream_t s) {
    if (R.n <= 0) return 0;
    if (k >= kWideK && R.khash) k_khash_init<<<num_sms() * 4, 256, 0, s>>>(R);
    switch (k) {
        case 4: return kmers_hist_launch<4>(R, s);
        case 5: return kmers_hist_launch<5>(R, s);
        case 6: return kmers_hist_launch<6>(R, s);
        case 7: return kmers_hist_launch<7>(R, s);
        default:
            if (k < kWideK || k > 12 || !R.khash) return 2;
            k_kmers_hash<<<R.khash_ctas, 256, 0, s>>>(R, k);
            return 0;
    }
}

}  // namespace gsdr
