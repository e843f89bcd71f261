// rounds.cu -- the greedy round loop on the device.
//
// Plain form: one representative per round, as the reference's clustering()
// (cuda-version/func.cu:1001-1066) and clusteringDrop() (func.cu:1068-1097).
// A round is four kernels that read their sizes from a RoundState in device
// memory, so rounds run back to back (and inside a CUDA graph) with no host
// round trip:
//   k_filter   kernel_preFilter + [kernel_pigeon] + kernel_makeTable/kernel_filter
//              (func.cu:712-826): warp-ballot over 32 candidates for the
//              composition bound, then one warp per survivor streams its
//              (k-mer, count) entries with 16-byte loads against the
//              representative's table staged in shared memory.  Survivors go
//              to an alignment queue (two length classes).
//   k_align_*  kernel_align (func.cu:828-999): warp-per-pair bit-parallel LCS,
//              marks cluster[j] = representative.
//   k_compact  updataRemain (func.cu:689-699): drops clustered reads from the
//              remain list (warp-aggregated atomics) and finds the smallest
//              unclustered index.
//   k_advance  updateRepresentative (func.cu:677-687): that index becomes the
//              next representative.
// Every decision is a pure function of (representative, candidate), so the
// order in which candidates are visited does not change any result.
#include <cuda_runtime.h>

#include "gsdr_device.cuh"
#include "lcs.cuh"

namespace gsdr {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kFilterThreads = 256;
constexpr int kAlignThreads = 128;
constexpr int kSmallWords = 128;  // pattern words handled by the small-class kernel (W <= 4)

__device__ __forceinline__ bool prefilter_pass(const int4 a, const int4 b, int cut) {
    const int s = min(a.x, b.x) + min(a.y, b.y) + min(a.z, b.z) + min(a.w, b.w);
    return !(s < cut);
}

// kernel_pigeon (cuda-version/func.cu:756-801), one warp per pair: lane l
// walks buckets l, l+32, ... with the reference's merge rule.
__device__ bool pigeon_pass_warp(const DevReads& R, float t, int rep, int q, int lane) {
    const uint16_t* p1 = R.pig + (size_t)rep * 256;
    const uint16_t* p2 = R.pig + (size_t)q * 256;
    const uint16_t* i1 = R.pig_idx + R.raw_off[rep];
    const uint16_t* i2 = R.pig_idx + R.raw_off[q];
    const int gap = (int)((float)R.len[rep] - ceilf(__fmul_rn((float)R.len[q], t)));
    int sum = 0;
    for (int b = lane; b < 256; b += 32) {
        int s1 = b > 0 ? p1[b - 1] : 0, e1 = p1[b];
        int s2 = b > 0 ? p2[b - 1] : 0, e2 = p2[b];
        while (s1 < e1 && s2 < e2) {
            const int one = i1[s1], two = i2[s2];
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
    return !(sum < R.cut_pig[q]);
}

template <int K, bool DROP, bool PIGEON>
__global__ void __launch_bounds__(kFilterThreads) k_filter(DevReads R, RoundState* st,
                                                           const int32_t* __restrict__ remain,
                                                           Pair* pairs, int pair_cap, float t) {
    extern __shared__ __align__(16) uint16_t table[];
    if (st->done) return;
    const int rep = st->rep;
    const int n = st->n_remain;
    if (n <= 0) return;
    constexpr int NB = DROP ? 0 : (1 << (2 * K));
    if (!DROP) {
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
        __syncthreads();
    }
    const int lane = threadIdx.x & 31;
    const int4 crep = R.comp[rep];
    const int rep_gf = R.len_gf[rep];
    unsigned long long n_pf = 0, n_wf = 0, n_al = 0, bytes = 0;
    while (true) {
        int base = 0;
        if (lane == 0) base = atomicAdd(&st->work_filter, 32);
        base = __shfl_sync(kFull, base, 0);
        if (base >= n) break;
        const int idx = base + lane;
        const int j = idx < n ? remain[idx] : -1;
        bool pass = false;
        if (j >= 0 && j != rep) {
            // kernel_preFilter (func.cu:738-754); lossless, so also used in drop mode.
            pass = prefilter_pass(crep, R.comp[j], R.cut_base[j]);
            n_pf++;
        }
        unsigned m = __ballot_sync(kFull, pass);
        while (m) {
            const int src = __ffs(m) - 1;
            m &= m - 1;
            const int q = __shfl_sync(kFull, j, src);
            bool ok = true;
            if (PIGEON) ok = pigeon_pass_warp(R, t, rep, q, lane);
            if (!DROP && ok) {
                // kernel_filter (func.cu:803-826): sum of min(table, count).
                const int ne = R.n_kmer[q];
                const int ne4 = (ne + 3) >> 2;
                const uint4* e4 = reinterpret_cast<const uint4*>(R.kmer + R.kmer_off[q]);
                int sum = 0;
                for (int i = lane; i < ne4; i += 32) {
                    const uint4 v = __ldcs(e4 + i);
                    sum += min((uint32_t)table[v.x >> 16], v.x & 0xffffu);
                    sum += min((uint32_t)table[v.y >> 16], v.y & 0xffffu);
                    sum += min((uint32_t)table[v.z >> 16], v.z & 0xffffu);
                    sum += min((uint32_t)table[v.w >> 16], v.w & 0xffffu);
                }
                sum = warp_sum_i(sum);
                ok = !(sum < R.cut_word[q]);
                if (lane == 0) {
                    n_wf++;
                    bytes += 16ull * ne4;
                }
            }
            if (ok && lane == 0) {
                n_al++;
                const int qgf = R.len_gf[q];
                const int words = (qgf + 31) >> 5;
                (void)rep_gf;
                const int cls = words <= kSmallWords ? 0 : 1;
                const int half = pair_cap >> 1;
                const int slot = atomicAdd(&st->n_pairs[cls], 1);
                if (slot < half) pairs[cls * half + slot] = Pair{rep, q};
                else st->pair_overflow = 1;
            }
        }
    }
    // per-warp statistics
    n_pf = __reduce_add_sync(kFull, (unsigned)n_pf);
    if (lane == 0) {
        atomicAdd(&st->cnt_prefilter, n_pf);
        if (n_wf) atomicAdd(&st->cnt_word, n_wf);
        if (n_al) atomicAdd(&st->cnt_aligned, n_al);
        if (bytes) atomicAdd(&st->filter_bytes, bytes + 0ull);
    }
}

// The pair decision shared by both alignment kernels.
template <bool SMALL>
__device__ bool align_pair(const DevReads& R, int rep, int q, int lane) {
    const int T = R.len_gf[rep];
    const int qn = R.len_gf[q];
    const int c = R.cut_base[q];
    if (T == 0) return false;   // the reference never decides such a pair
    if (c <= 0) return true;    // LCS >= 0 >= cutoff
    if (qn < c || T < c) return false;
    const uint32_t* pq = R.packed + R.pack_off[q];
    const uint32_t* pt = R.packed + R.pack_off[rep];
    const int words = (qn + 31) >> 5;
    if (SMALL) {
        if (words <= 32) return lcs_reaches_warp<1, true>(pq, qn, pt, T, c, lane);
        if (words <= 64) return lcs_reaches_warp<2, true>(pq, qn, pt, T, c, lane);
        return lcs_reaches_warp<4, true>(pq, qn, pt, T, c, lane);
    } else {
        if (words <= 256) return lcs_reaches_warp<8, false>(pq, qn, pt, T, c, lane);
        if (words <= 512) return lcs_reaches_warp<16, false>(pq, qn, pt, T, c, lane);
        return lcs_reaches_warp<32, false>(pq, qn, pt, T, c, lane);
    }
}

template <bool SMALL>
__global__ void __launch_bounds__(kAlignThreads) k_align(DevReads R, RoundState* st,
                                                         const Pair* __restrict__ pairs,
                                                         int pair_cap, int32_t* cluster,
                                                         int* work) {
    if (st->done) return;
    const int half = pair_cap >> 1;
    const int np = min(st->n_pairs[SMALL ? 0 : 1], half);
    if (np <= 0) return;
    const int lane = threadIdx.x & 31;
    const Pair* list = pairs + (SMALL ? 0 : half);
    unsigned long long acc = 0, cells = 0;
    while (true) {
        int i = 0;
        if (lane == 0) i = atomicAdd(work, 1);
        i = __shfl_sync(kFull, i, 0);
        if (i >= np) break;
        const Pair p = list[i];
        const bool ok = align_pair<SMALL>(R, p.rep, p.cand, lane);
        if (lane == 0) {
            cells += (unsigned long long)R.len_gf[p.rep] * (unsigned long long)R.len_gf[p.cand];
            if (ok) {
                cluster[p.cand] = p.rep;
                acc++;
            }
        }
    }
    if (lane == 0 && (acc || cells)) {
        atomicAdd(&st->cnt_accepted, acc);
        atomicAdd(&st->cells, cells);
    }
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

__global__ void k_advance(RoundState* st, int32_t* cluster, int* align_work) {
    if (st->done) return;
    st->rounds += 1;
    st->passes += 1;
    const int n = st->n_next;
    if (n == 0) {
        st->done = 1;
        return;
    }
    const int rep = st->next_min;
    cluster[rep] = rep;
    st->rep = rep;
    st->n_remain = n;
    st->n_next = 0;
    st->next_min = 0x7fffffff;
    st->n_pairs[0] = 0;
    st->n_pairs[1] = 0;
    st->work_filter = 0;
    align_work[0] = 0;
    align_work[1] = 0;
}

__global__ void k_init(RoundState* st, int32_t* cluster, int32_t* remain, int n, int* align_work) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        cluster[i] = i == 0 ? 0 : -1;
        if (i > 0) remain[i - 1] = i;
    }
    if (i == 0) {
        RoundState s = {};
        s.rep = 0;
        s.n_remain = n - 1;
        s.next_min = 0x7fffffff;
        s.done = n <= 0 ? 1 : 0;
        *st = s;
        align_work[0] = 0;
        align_work[1] = 0;
    }
}

template <int K, bool DROP, bool PIGEON>
void launch_filter_t(const DevReads& R, RoundBuffers& B, const int32_t* remain, float t,
                     cudaStream_t s) {
    const int smem = DROP ? 0 : (1 << (2 * K)) * 2;
    static int grid = 0;
    if (!grid) {
        if (smem > 48 * 1024)
            cudaFuncSetAttribute(k_filter<K, DROP, PIGEON>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_filter<K, DROP, PIGEON>,
                                                      kFilterThreads, smem);
        if (per_sm < 1) per_sm = 1;
        if (per_sm > 4) per_sm = 4;
        grid = num_sms() * per_sm;
    }
    k_filter<K, DROP, PIGEON><<<grid, kFilterThreads, smem, s>>>(R, B.st, remain, B.pairs,
                                                                 B.pair_cap, t);
}

template <bool DROP, bool PIGEON>
void launch_filter_k(const DevReads& R, RoundBuffers& B, const int32_t* remain, float t, int k,
                     cudaStream_t s) {
    switch (k) {
        case 4: launch_filter_t<4, DROP, PIGEON>(R, B, remain, t, s); break;
        case 5: launch_filter_t<5, DROP, PIGEON>(R, B, remain, t, s); break;
        case 6: launch_filter_t<6, DROP, PIGEON>(R, B, remain, t, s); break;
        default: launch_filter_t<7, DROP, PIGEON>(R, B, remain, t, s); break;
    }
}

}  // namespace

int filter_smem_bytes(int k, int drop) { return drop ? 0 : (1 << (2 * k)) * 2; }

// Device work counters for the two alignment kernels live right after the
// RoundState in the same allocation.
static int* align_work_of(RoundState* st) { return reinterpret_cast<int*>(st + 1); }

void init_rounds(const DevReads& R, RoundBuffers& B, cudaStream_t s) {
    const int n = R.n;
    const int threads = 256;
    const int blocks = n > 0 ? (n + threads - 1) / threads : 1;
    k_init<<<blocks, threads, 0, s>>>(B.st, B.cluster, B.remain[0], n, align_work_of(B.st));
}

void launch_plain_round(const DevReads& R, RoundBuffers& B, float t, int drop, int pigeon,
                        int parity, cudaStream_t s, long long* count, cudaEvent_t* ev4) {
    const int32_t* rin = B.remain[parity];
    int32_t* rout = B.remain[parity ^ 1];
    if (ev4) cudaEventRecord(ev4[0], s);
    if (drop) {
        launch_filter_k<true, false>(R, B, rin, t, R.k, s);
    } else if (pigeon) {
        launch_filter_k<false, true>(R, B, rin, t, R.k, s);
    } else {
        launch_filter_k<false, false>(R, B, rin, t, R.k, s);
    }
    if (ev4) cudaEventRecord(ev4[1], s);
    static int grid_small = 0, grid_large = 0;
    if (!grid_small) {
        int a = 0, b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_align<true>, kAlignThreads, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_align<false>, kAlignThreads, 0);
        grid_small = num_sms() * (a > 0 ? a : 1);
        grid_large = num_sms() * (b > 0 ? b : 1);
    }
    int* aw = align_work_of(B.st);
    k_align<true><<<grid_small, kAlignThreads, 0, s>>>(R, B.st, B.pairs, B.pair_cap, B.cluster,
                                                       aw + 0);
    k_align<false><<<grid_large, kAlignThreads, 0, s>>>(R, B.st, B.pairs, B.pair_cap, B.cluster,
                                                        aw + 1);
    if (ev4) cudaEventRecord(ev4[2], s);
    k_compact<<<num_sms() * 4, 256, 0, s>>>(B.st, rin, rout, B.cluster);
    k_advance<<<1, 1, 0, s>>>(B.st, B.cluster, aw);
    if (ev4) cudaEventRecord(ev4[3], s);
    if (count) *count += 5;
}

}  // namespace gsdr
