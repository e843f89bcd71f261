// devparse.cu -- readFile, clustering and saveFile with the FASTA text on the
// device (gsdr_cluster_fasta, include/gsdr.h).
//
// The reference reads the file with std::getline (cuda-version/func.cu:94-117):
// the first line is a name whatever it holds, every later line starting with
// '>' opens a record, other non-empty lines are appended to the record's data
// verbatim ('\r' included), and the records are then sorted longest first
// with std::sort.  Here the file's bytes are copied to the device once:
//   k_nl_count / k_nl_write   newline positions in file order (per 4 KB chunk
//                             counts, exclusive scan, ordered scatter)
//   k_line_kind              per line: header flag
//   k_rec_head               per record: its first line and name span
//   k_rec_data               per record (one warp): data length, pieces, and
//                            the data's offset (single-line records point into
//                            the file; multi-line ones are copied end to end
//                            into a region after the file, k_rec_concat)
// Only the data lengths come back to the host, for the same std::sort call
// (the order of equal-length reads depends on its comparisons), then the job
// clusters the device-resident reads and k_out_copy formats the output records
// (name line, data line) on the device; only the output bytes come back.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "gsdr.h"
#include "devmem.h"
#include "gsdr_device.cuh"
#include "gsdr_host.h"
#include "nvtx_range.h"
#include "job.h"
#include "stdsort.h"

struct gsdr_result {
    std::vector<char> out;          // representative records, saveFile's bytes
    std::vector<int32_t> cluster;   // sorted order
    std::vector<int32_t> order;     // sorted position -> record in file order
    std::vector<int32_t> length;    // sorted order
};

namespace gsdr {
namespace {

constexpr int kChunk = 4096;  // bytes per newline-count chunk (one warp)
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;  // per thread: a CTA scans 4096 entries

#define DCUDA(call)                                                      \
    do {                                                                 \
        cudaError_t e_ = (call);                                         \
        if (e_ != cudaSuccess)                                           \
            return fail(e_ == cudaErrorMemoryAllocation ? GSDR_ENOMEM    \
                                                        : GSDR_EDEVICE,  \
                        cudaGetErrorString(e_));                         \
    } while (0)

__device__ __forceinline__ uint32_t nl_bytes(uint32_t w) {
    // 0x80 in every byte equal to '\n'
    const uint32_t x = w ^ 0x0a0a0a0au;
    return ~(((x & 0x7f7f7f7fu) + 0x7f7f7f7fu) | x | 0x7f7f7f7fu);
}

__global__ void k_nl_count(const uint8_t* __restrict__ b, int64_t n, int64_t n_chunks,
                           uint32_t* cnt) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t c = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); c < n_chunks;
         c += nw) {
        const int64_t base = c * kChunk;
        uint32_t k = 0;
        if (base + kChunk <= n) {
            // a whole chunk: 16 bytes per lane, all of the chunk's loads at once
            const uint4* v4 = reinterpret_cast<const uint4*>(b + base) + lane;
            uint4 v[kChunk / 512];
#pragma unroll
            for (int i = 0; i < kChunk / 512; i++) v[i] = __ldg(v4 + 32 * i);
#pragma unroll
            for (int i = 0; i < kChunk / 512; i++)
                k += __popc(nl_bytes(v[i].x)) + __popc(nl_bytes(v[i].y)) +
                     __popc(nl_bytes(v[i].z)) + __popc(nl_bytes(v[i].w));
        } else {
            for (int i = lane * 4; i < kChunk; i += 128) {
                const int64_t p = base + i;
                if (p + 4 <= n) {
                    k += __popc(nl_bytes(*reinterpret_cast<const uint32_t*>(b + p)));
                } else {
                    for (int64_t q = p; q < n && q < p + 4; q++) k += b[q] == '\n';
                }
            }
        }
        k = __reduce_add_sync(0xffffffffu, k);
        if (lane == 0) cnt[c] = k;
    }
}

// newline positions in file order: the r-th '\n' of chunk c goes to
// nl[base[c] + r]; within a chunk, lanes take 4 bytes in turn
__global__ void k_nl_write(const uint8_t* __restrict__ b, int64_t n, int64_t n_chunks,
                           const uint32_t* __restrict__ base, int64_t* nl) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t c = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); c < n_chunks;
         c += nw) {
        uint32_t at = base[c];
        if ((c + 1) * kChunk <= n) {
            // a whole chunk: 16 bytes per lane per step, the steps' loads at once
            const uint4* v4 = reinterpret_cast<const uint4*>(b + c * kChunk) + lane;
            uint4 v[kChunk / 512];
#pragma unroll
            for (int i = 0; i < kChunk / 512; i++) v[i] = __ldg(v4 + 32 * i);
#pragma unroll
            for (int i = 0; i < kChunk / 512; i++) {
                const int64_t p = c * kChunk + 512 * i + 16 * lane;
                const uint32_t w[4] = {v[i].x, v[i].y, v[i].z, v[i].w};
                uint32_t m = 0;  // bit j: byte p + j is '\n'
#pragma unroll
                for (int h = 0; h < 4; h++) {
                    const uint32_t f = nl_bytes(w[h]);
                    m |= (((f >> 7) & 1u) | ((f >> 14) & 2u) | ((f >> 21) & 4u) |
                          ((f >> 28) & 8u)) << (4 * h);
                }
                const uint32_t k = __popc(m);
                uint32_t incl = k;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const uint32_t o = __shfl_up_sync(0xffffffffu, incl, d);
                    if (lane >= d) incl += o;
                }
                uint32_t wpos = at + incl - k;
                while (m) {
                    const int j = __ffs(m) - 1;
                    m &= m - 1;
                    nl[wpos++] = p + j;
                }
                at += __shfl_sync(0xffffffffu, incl, 31);
            }
            continue;
        }
        for (int i = 0; i < kChunk; i += 128) {
            const int64_t p = c * kChunk + i + lane * 4;
            uint32_t m = 0;  // bit j: byte p + j is '\n'
            if (p + 4 <= n) {
                const uint32_t f = nl_bytes(*reinterpret_cast<const uint32_t*>(b + p));
                m = ((f >> 7) & 1u) | ((f >> 14) & 2u) | ((f >> 21) & 4u) | ((f >> 28) & 8u);
            } else {
                for (int j = 0; j < 4; j++)
                    if (p + j < n && b[p + j] == '\n') m |= 1u << j;
            }
            const uint32_t k = __popc(m);
            uint32_t incl = k;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t o = __shfl_up_sync(0xffffffffu, incl, d);
                if (lane >= d) incl += o;
            }
            uint32_t w = at + incl - k;
            while (m) {
                const int j = __ffs(m) - 1;
                m &= m - 1;
                nl[w++] = p + j;
            }
            at += __shfl_sync(0xffffffffu, incl, 31);
        }
    }
}

// ---- exclusive scan of u32 counts (three phases) ------------------------------

__device__ uint32_t block_scan(uint32_t v, uint32_t* warp_tot, uint32_t* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t o = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += o;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const uint32_t t = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0u;
        uint32_t ti = t;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t o = __shfl_up_sync(0xffffffffu, ti, d);
            if (lane >= d) ti += o;
        }
        warp_tot[lane] = ti - t;
        if (lane == 31) *total = ti;
    }
    __syncthreads();
    const uint32_t r = warp_tot[warp] + incl - v;
    __syncthreads();
    return r;
}

// phase 1 (sums only) and 3 (scan with block offsets): a CTA covers
// kScanThreads * kScanItems consecutive entries
template <bool WRITE>
__global__ void __launch_bounds__(kScanThreads) k_scan_blocks(const uint32_t* __restrict__ in,
                                                              int64_t n, uint32_t* block_sum,
                                                              const uint32_t* __restrict__ block_off,
                                                              uint32_t* out) {
    __shared__ uint32_t wt[32];
    __shared__ uint32_t tot;
    const int64_t base = ((int64_t)blockIdx.x * kScanThreads + threadIdx.x) * kScanItems;
    uint32_t v[kScanItems], s = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; j++) {
        v[j] = base + j < n ? in[base + j] : 0u;
        s += v[j];
    }
    const uint32_t ex = block_scan(s, wt, &tot);
    if (!WRITE) {
        if (threadIdx.x == 0) block_sum[blockIdx.x] = tot;
        return;
    }
    uint32_t run = block_off[blockIdx.x] + ex;
#pragma unroll
    for (int j = 0; j < kScanItems; j++) {
        if (base + j < n) out[base + j] = run;
        run += v[j];
    }
}

// phase 2: one CTA scans the block sums in place, total into *total
__global__ void __launch_bounds__(kScanThreads) k_scan_single(uint32_t* a, int64_t n,
                                                              uint32_t* total) {
    __shared__ uint32_t wt[32];
    __shared__ uint32_t tot;
    uint32_t carry = 0;
    for (int64_t b0 = 0; b0 < n; b0 += kScanThreads) {
        const int64_t i = b0 + threadIdx.x;
        const uint32_t v = i < n ? a[i] : 0u;
        const uint32_t ex = block_scan(v, wt, &tot);
        if (i < n) a[i] = carry + ex;
        carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

// exclusive scan of n u32 values into out (may alias in); returns the total
int scan_u32(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* tmp, uint32_t* d_total,
             cudaStream_t s, uint32_t* h_total) {
    if (n <= 0) {
        *h_total = 0;
        return GSDR_OK;
    }
    const int64_t per = (int64_t)kScanThreads * kScanItems;
    const int64_t nb = (n + per - 1) / per;
    k_scan_blocks<false><<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, tmp, nullptr, nullptr);
    k_scan_single<<<1, kScanThreads, 0, s>>>(tmp, nb, d_total);
    k_scan_blocks<true><<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, nullptr, tmp, out);
    DCUDA(cudaGetLastError());
    DCUDA(cudaMemcpyAsync(h_total, d_total, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    DCUDA(cudaStreamSynchronize(s));
    return GSDR_OK;
}

// ---- lines and records ---------------------------------------------------------

__device__ __forceinline__ int64_t line_start(const int64_t* nl, int64_t j) {
    return j == 0 ? 0 : nl[j - 1] + 1;
}
__device__ __forceinline__ int64_t line_end(const int64_t* nl, int64_t j, int64_t n_nl, int64_t n) {
    return j < n_nl ? nl[j] : n;
}

// hdr[j] = 1 for a line j > 0 that opens a record (non-empty, starts with '>')
__global__ void k_line_kind(const uint8_t* __restrict__ b, int64_t n, const int64_t* __restrict__ nl,
                            int64_t n_nl, int64_t n_lines, uint32_t* hdr) {
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n_lines;
         j += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = line_start(nl, j), e = line_end(nl, j, n_nl, n);
        hdr[j] = (j > 0 && e > s && b[s] == '>') ? 1u : 0u;
    }
}

// record r begins at line head[r] (line 0, then every header line); its name
// is that whole line
__global__ void k_rec_head(const int64_t* __restrict__ nl, int64_t n_nl, int64_t n,
                           int64_t n_lines, const uint32_t* __restrict__ hdr,
                           const uint32_t* __restrict__ hdr_ex, int64_t* head, int64_t* name_off,
                           int32_t* name_len) {
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n_lines;
         j += (int64_t)gridDim.x * blockDim.x) {
        if (j == 0 || hdr[j]) {
            const int64_t r = j == 0 ? 0 : hdr_ex[j] + 1;  // header lines before j, + line 0
            const int64_t s = line_start(nl, j);
            head[r] = j;
            name_off[r] = s;
            name_len[r] = (int32_t)(line_end(nl, j, n_nl, n) - s);
        }
    }
}

// one warp per record: the data lines (non-empty lines up to the next record)
__global__ void k_rec_data(const int64_t* __restrict__ nl, int64_t n_nl, int64_t n,
                           int64_t n_lines, const int64_t* __restrict__ head, int64_t n_rec,
                           int64_t* data_off, int64_t* data_len, int32_t* pieces) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < n_rec;
         r += nw) {
        const int64_t j0 = head[r] + 1, j1 = r + 1 < n_rec ? head[r + 1] : n_lines;
        int64_t len = 0, first = -1;
        int k = 0;
        for (int64_t j = j0 + lane; j < j1; j += 32) {
            const int64_t s = line_start(nl, j), e = line_end(nl, j, n_nl, n);
            if (e > s) {
                len += e - s;
                k++;
                if (first < 0) first = s;  // lowest j of this lane
            }
        }
        // the first data line of the record: the smallest lane-first over the
        // lowest iteration (lanes visit j0+lane, j0+lane+32, ...)
        long long f = first < 0 ? 0x7fffffffffffffffll : first;
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) {
            const long long o = __shfl_xor_sync(0xffffffffu, f, d);
            f = o < f ? o : f;
        }
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) {
            len += __shfl_xor_sync(0xffffffffu, len, d);
            k += __shfl_xor_sync(0xffffffffu, k, d);
        }
        if (lane == 0) {
            data_len[r] = len;
            pieces[r] = k;
            data_off[r] = k == 0 ? 0 : (int64_t)f;
        }
    }
}

// multi-line records: their data lines copied end to end into the region after
// the file at extra_off[r] (set when pieces[r] > 1)
__global__ void k_rec_concat(uint8_t* b, const int64_t* __restrict__ nl, int64_t n_nl, int64_t n,
                             int64_t n_lines, const int64_t* __restrict__ head, int64_t n_rec,
                             const int32_t* __restrict__ pieces, const int64_t* __restrict__ data_off) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < n_rec;
         r += nw) {
        if (pieces[r] <= 1) continue;
        const int64_t j0 = head[r] + 1, j1 = r + 1 < n_rec ? head[r + 1] : n_lines;
        int64_t at = data_off[r];
        for (int64_t j = j0; j < j1; j++) {
            const int64_t s = line_start(nl, j), e = line_end(nl, j, n_nl, n);
            for (int64_t i = lane; i < e - s; i += 32) b[at + i] = b[s + i];
            at += e - s;
        }
    }
}

// saveFile's records (func.cu:1099-1111) for the representatives, in sorted
// order: warp per read, out_off from an exclusive scan of the record sizes
__global__ void k_out_copy(const uint8_t* __restrict__ b, const int32_t* __restrict__ cluster,
                           const int32_t* __restrict__ order, const int64_t* __restrict__ name_off,
                           const int32_t* __restrict__ name_len, const int64_t* __restrict__ off,
                           const int32_t* __restrict__ len, const uint32_t* __restrict__ out_off,
                           int n, uint8_t* out, int64_t out_base) {
    const int lane = threadIdx.x & 31;
    const int nw = gridDim.x * (blockDim.x >> 5);
    for (int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += nw) {
        if (cluster[i] != i) continue;
        const int r = order[i];
        uint8_t* o = out + ((int64_t)out_off[i] - out_base);
        const int nlen = name_len[r], dlen = len[i];
        const uint8_t* nm = b + name_off[r];
        const uint8_t* dt = b + off[i];
        for (int k = lane; k < nlen; k += 32) o[k] = nm[k];
        if (lane == 0) o[nlen] = '\n';
        for (int k = lane; k < dlen; k += 32) o[nlen + 1 + k] = dt[k];
        if (lane == 0) o[nlen + 1 + dlen] = '\n';
    }
}

__global__ void k_out_sizes(const int32_t* __restrict__ cluster, const int32_t* __restrict__ order,
                            const int32_t* __restrict__ name_len, const int32_t* __restrict__ len,
                            int n, uint32_t* sz) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        sz[i] = cluster[i] == i ? (uint32_t)(name_len[order[i]] + len[i] + 2) : 0u;
}

int grid_of(int64_t items, int per_block, int cap) {
    int64_t g = (items + per_block - 1) / per_block;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (int)g;
}

// A device buffer from the library's pool, returned to it on the stream it
// was taken on when the buffer goes out of scope (devmem.h).
struct DevBuf {
    cudaStream_t s;
    void* p = nullptr;
    explicit DevBuf(cudaStream_t st) : s(st) {}
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { dev_free(p, s); }
    template <class T>
    T* as() const {
        return reinterpret_cast<T*>(p);
    }
};

}  // namespace

gsdr_result* new_result() { return new (std::nothrow) gsdr_result(); }

int64_t cluster_fasta_parse_bytes(int64_t n, int64_t records, int64_t newlines) {
    const int64_t n_chunks = (n + kChunk - 1) / kChunk + 1;
    const int64_t lines = newlines + 2;
    return (2 * n + 64)                                  // the file, concatenated records
           + 4 * (n / (kScanThreads * kScanItems) + 8) + 64 + 4 * n_chunks  // scans, counts
           + 8 * lines                                   // newline positions
           + 8 * lines                                   // line kinds
           + 40 * (records + 1)                          // record heads, names, data spans
           + 12 * (records + 1) + 48                     // output order, sizes, offsets
           + n + 16                                      // output records (at most the file)
           + (1 << 20);                                  // allocation rounding
}

int cluster_fasta(const char* fasta, int64_t n, const gsdr_opts* opts_in, gsdr_result* res,
                  gsdr_stats* stats, const std::function<int(int64_t)>* admit) {
    gsdr_opts o = *opts_in;
    int rc = gsdr_resolve_opts(&o, nullptr);
    if (rc) return rc;
    int dev_count = 0;
    if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count <= 0)
        return fail(GSDR_EDEVICE, "no CUDA device");
    if (o.device < 0 || o.device >= dev_count) return fail(GSDR_EINVAL, "bad device");
    DCUDA(cudaSetDevice(o.device));
    cudaStream_t s = nullptr;
    DCUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    struct StreamGuard {
        cudaStream_t s;
        ~StreamGuard() { cudaStreamDestroy(s); }
    } sg{s};
    const double t0 = now_ms();
    // GSDR_TRACE=1: host time at each phase's end (the stream synchronized
    // there, so the phases do not overlap), on stderr
    const char* tr = std::getenv("GSDR_TRACE");
    const bool trace = tr && tr[0] == '1';
    std::vector<std::pair<const char*, double>> marks;
    auto mark = [&](const char* what) {
        if (!trace) return;
        cudaStreamSynchronize(s);
        marks.emplace_back(what, now_ms() - t0);
    };
    struct TracePrint {
        const std::vector<std::pair<const char*, double>>& m;
        ~TracePrint() {
            if (m.empty()) return;
            std::string line = "gsdr trace: cluster_fasta";
            for (auto& x : m) line += " " + std::string(x.first) + " " + std::to_string(x.second);
            std::fprintf(stderr, "%s ms\n", line.c_str());
        }
    } tp{marks};
    NvtxRange range_read("gsdr: FASTA bytes to reads (device parse, host sort)");

    // the file on the device, with room for multi-line records' data after it
    // (at most the file's size) and 16 bytes of slack for word loads
    DevBuf file(s);
    DCUDA(dev_alloc(&file.p, (size_t)(2 * n + 64), s));
    DCUDA(cudaMemsetAsync(file.as<uint8_t>() + n, 0, 64, s));
    DCUDA(cudaMemcpyAsync(file.p, fasta, (size_t)n, cudaMemcpyHostToDevice, s));
    uint8_t* b = file.as<uint8_t>();
    mark("h2d");

    const int64_t n_chunks = (n + kChunk - 1) / kChunk;
    const int64_t per = (int64_t)kScanThreads * kScanItems;
    DevBuf scan_tmp(s), small(s);
    DCUDA(dev_alloc(&scan_tmp.p, sizeof(uint32_t) * (size_t)(std::max<int64_t>(n_chunks, 1) / per + 2 +
                                                              (n / per) + 2), s));
    DCUDA(dev_alloc(&small.p, 64, s));
    uint32_t* d_total = small.as<uint32_t>();
    uint32_t h_total = 0;

    DevBuf cnt(s);
    DCUDA(dev_alloc(&cnt.p, sizeof(uint32_t) * (size_t)std::max<int64_t>(n_chunks, 1), s));
    k_nl_count<<<grid_of(n_chunks, 8, 1 << 16), 256, 0, s>>>(b, n, n_chunks, cnt.as<uint32_t>());
    rc = scan_u32(cnt.as<uint32_t>(), cnt.as<uint32_t>(), n_chunks, scan_tmp.as<uint32_t>(), d_total,
                  s, &h_total);
    if (rc) return rc;
    const int64_t n_nl = h_total;
    // getline: a last line without '\n' still counts; "a\n" is one line
    const int64_t n_lines = n_nl + (n > 0 && fasta[n - 1] != '\n' ? 1 : 0);
    DevBuf nl(s);
    DCUDA(dev_alloc(&nl.p, sizeof(int64_t) * (size_t)std::max<int64_t>(n_nl, 1), s));
    k_nl_write<<<grid_of(n_chunks, 8, 1 << 16), 256, 0, s>>>(b, n, n_chunks, cnt.as<uint32_t>(),
                                                             nl.as<int64_t>());

    DevBuf hdr(s), hdr_ex(s);
    DCUDA(dev_alloc(&hdr.p, sizeof(uint32_t) * (size_t)std::max<int64_t>(n_lines, 1), s));
    DCUDA(dev_alloc(&hdr_ex.p, sizeof(uint32_t) * (size_t)std::max<int64_t>(n_lines, 1), s));
    k_line_kind<<<grid_of(n_lines, 256, 1 << 16), 256, 0, s>>>(b, n, nl.as<int64_t>(), n_nl, n_lines,
                                                                hdr.as<uint32_t>());
    rc = scan_u32(hdr.as<uint32_t>(), hdr_ex.as<uint32_t>(), n_lines, scan_tmp.as<uint32_t>(),
                  d_total, s, &h_total);
    if (rc) return rc;
    const int64_t n_rec = 1 + (int64_t)h_total;
    if (n_rec > INT32_MAX) return fail(GSDR_EUNSUPPORTED, "too many records");

    DevBuf head(s), name_off(s), name_len(s), data_off(s), data_len(s), pieces(s);
    DCUDA(dev_alloc(&head.p, sizeof(int64_t) * n_rec, s));
    DCUDA(dev_alloc(&name_off.p, sizeof(int64_t) * n_rec, s));
    DCUDA(dev_alloc(&name_len.p, sizeof(int32_t) * n_rec, s));
    DCUDA(dev_alloc(&data_off.p, sizeof(int64_t) * n_rec, s));
    DCUDA(dev_alloc(&data_len.p, sizeof(int64_t) * n_rec, s));
    DCUDA(dev_alloc(&pieces.p, sizeof(int32_t) * n_rec, s));
    if (n_lines == 0) {
        // an empty file: one record with an empty name and no data
        DCUDA(cudaMemsetAsync(head.p, 0, sizeof(int64_t), s));
        DCUDA(cudaMemsetAsync(name_off.p, 0, sizeof(int64_t), s));
        DCUDA(cudaMemsetAsync(name_len.p, 0, sizeof(int32_t), s));
        DCUDA(cudaMemsetAsync(data_off.p, 0, sizeof(int64_t), s));
        DCUDA(cudaMemsetAsync(data_len.p, 0, sizeof(int64_t), s));
        DCUDA(cudaMemsetAsync(pieces.p, 0, sizeof(int32_t), s));
    } else {
        k_rec_head<<<grid_of(n_lines, 256, 1 << 16), 256, 0, s>>>(
            nl.as<int64_t>(), n_nl, n, n_lines, hdr.as<uint32_t>(), hdr_ex.as<uint32_t>(),
            head.as<int64_t>(), name_off.as<int64_t>(), name_len.as<int32_t>());
        k_rec_data<<<grid_of(n_rec, 8, 1 << 16), 256, 0, s>>>(
            nl.as<int64_t>(), n_nl, n, n_lines, head.as<int64_t>(), n_rec, data_off.as<int64_t>(),
            data_len.as<int64_t>(), pieces.as<int32_t>());
    }
    DCUDA(cudaGetLastError());
    mark("parse");
    // the record lengths, offsets and piece counts, in the thread's pinned
    // scratch (a direct copy; pageable memory would take a staged one)
    std::vector<int64_t> v_dlen, v_doff;
    std::vector<int32_t> v_pieces;
    int64_t* h_dlen = nullptr;
    int64_t* h_doff = nullptr;
    int32_t* h_pieces = nullptr;
    if (char* pin = static_cast<char*>(pinned_scratch(sizeof(int64_t) * 2 * n_rec +
                                                      sizeof(int32_t) * n_rec))) {
        h_dlen = reinterpret_cast<int64_t*>(pin);
        h_doff = h_dlen + n_rec;
        h_pieces = reinterpret_cast<int32_t*>(h_doff + n_rec);
    } else {
        v_dlen.resize(n_rec);
        v_doff.resize(n_rec);
        v_pieces.resize(n_rec);
        h_dlen = v_dlen.data();
        h_doff = v_doff.data();
        h_pieces = v_pieces.data();
    }
    DCUDA(cudaMemcpyAsync(h_dlen, data_len.p, sizeof(int64_t) * n_rec,
                          cudaMemcpyDeviceToHost, s));
    DCUDA(cudaMemcpyAsync(h_doff, data_off.p, sizeof(int64_t) * n_rec,
                          cudaMemcpyDeviceToHost, s));
    DCUDA(cudaMemcpyAsync(h_pieces, pieces.p, sizeof(int32_t) * n_rec,
                          cudaMemcpyDeviceToHost, s));
    DCUDA(cudaStreamSynchronize(s));
    // multi-line records: data placed end to end after the file
    int64_t extra = 0;
    bool multi = false;
    for (int64_t r = 0; r < n_rec; r++) {
        if (h_dlen[r] > INT32_MAX) return fail(GSDR_EUNSUPPORTED, "a record above 2^31 bytes");
        if (h_pieces[r] > 1) {
            h_doff[r] = n + 16 + extra;
            extra += h_dlen[r];
            multi = true;
        }
    }
    if (multi) {
        DCUDA(cudaMemcpyAsync(data_off.p, h_doff, sizeof(int64_t) * n_rec,
                              cudaMemcpyHostToDevice, s));
        k_rec_concat<<<grid_of(n_rec, 8, 1 << 16), 256, 0, s>>>(
            b, nl.as<int64_t>(), n_nl, n, n_lines, head.as<int64_t>(), n_rec,
            pieces.as<int32_t>(), data_off.as<int64_t>());
        DCUDA(cudaGetLastError());
    }
    // readFile's std::sort (func.cu:111-113) on the record indices (the same
    // permutation, its independent parts on several threads: stdsort.h)
    const int32_t nr = (int32_t)n_rec;
    res->order.resize(nr);
    std::iota(res->order.begin(), res->order.end(), 0);
    mark("records");
    // (the record lengths are below 2^31, so comparing them as 64-bit values
    // gives the comparator's outcomes, hence the permutation, of 32-bit ones)
    const int64_t* dlp = h_dlen;
    // (kept per thread between calls: a fresh array costs page faults and a
    // zero fill; every entry is written by the gather)
    static thread_local std::vector<int64_t> s_off;
    s_off.resize(nr);
    res->length.resize(nr);
    // offsets and lengths in sorted order, gathered by the sort's own threads
    // (one thread takes ~1 ms for the 200k-read workload: random reads of
    // arrays the copy wrote).  The same threads then lay out the job over the
    // reads each gathered (plan_chunks.h), so that Job::init skips its serial
    // pass over all reads (0.5 ms for the 200k-read workload).
    const int32_t* ord = res->order.data();
    const int64_t* doff = h_doff;
    int64_t* soff = s_off.data();
    int32_t* slen = res->length.data();
    const int n_threads = sort_threads();
    const int64_t view_bytes = n + 16 + extra;
    PlanPreset preset;
    preset.k = o.word_length;
    preset.drop = o.drop == 1;
    preset.pack_off.resize((size_t)nr + 1);
    preset.kmer_off.resize((size_t)nr + 1);
    preset.pack_off[0] = 0;
    preset.kmer_off[0] = 0;
    std::vector<PlanChunk> parts((size_t)std::max(n_threads, 1));
    std::atomic<int> arrived{0};
    int used = 0;  // threads that ran the gather (set by thread 0)
    int64_t* pk = preset.pack_off.data();
    int64_t* km = preset.kmer_off.data();
    PlanChunk* pp = parts.data();
    std::atomic<int>* arr = &arrived;
    int* usedp = &used;
    const int k_plan = preset.k;
    const bool drop_plan = preset.drop;
    const std::function<void(int, int)> gather = [=](int t, int T) {
        const int32_t lo = (int32_t)((int64_t)nr * t / T), hi = (int32_t)((int64_t)nr * (t + 1) / T);
        for (int32_t i = lo; i < hi; i++) {
            soff[i] = doff[ord[i]];
            slen[i] = (int32_t)dlp[ord[i]];
        }
        pp[t] = plan_chunk(soff, slen, view_bytes, lo, hi, k_plan, drop_plan, pk, km);
        // all T threads run this callback at once (stdsort.h): wait for the
        // others' sums, then add those of the parts before this one
        arr->fetch_add(1, std::memory_order_acq_rel);
        while (arr->load(std::memory_order_acquire) < T) std::this_thread::yield();
        int64_t pack_base = 0, kmer_base = 0;
        for (int u = 0; u < t; u++) {
            pack_base += pp[u].pack;
            kmer_base += pp[u].kmer;
        }
        plan_shift(lo, hi, pack_base, kmer_base, pk, km);
        if (t == 0) *usedp = T;
    };
    std_sort_threaded(res->order.begin(), res->order.end(),
                      [dlp](const int32_t& a, const int32_t& c) { return dlp[a] > dlp[c]; },
                      n_threads, gather);
    if (used > 0 && used <= (int)parts.size()) {
        PlanChunk all = parts[0];
        for (int u = 1; u < used; u++) {
            const int32_t lo = (int32_t)((int64_t)nr * u / used);
            const int32_t hi = (int32_t)((int64_t)nr * (u + 1) / used);
            const bool follows = lo >= hi || lo == 0 || slen[lo] <= slen[lo - 1];
            all = plan_join(all, parts[u], follows);
        }
        preset.sums = all;
    } else {
        preset.k = -1;  // not laid out: Job::init takes its own pass
    }
    const double t_parse = now_ms();
    mark("sort");
    range_read.end();

    // the clustering on the device-resident reads
    // (bytes: the device copy; the job reads only sizes from the view on the host)
    gsdr_reads view{reinterpret_cast<const char*>(b), n + 16 + extra, s_off.data(),
                    res->length.data(), nr};
    res->cluster.assign(nr > 0 ? nr : 1, 0);
    if (admit) {
        // the serving loop's admission by device footprint: it may block here
        const int64_t need = Job::footprint(&view, &o);
        if (need < 0) return fail(GSDR_EINVAL, "cluster_fasta: cannot size the job");
        rc = (*admit)(need);
        if (rc) return rc;
    }
    Job job;
    rc = job.init(&view, &o, s, &preset);
    mark("job_init");
    if (!rc) rc = job.upload(&view, b);
    mark("upload");
    if (!rc) rc = job.run();
    mark("run");
    if (rc) return rc;
    // the output records, formatted on the device
    NvtxRange range_out("gsdr: output records");
    DevBuf d_order(s), sz(s);
    DCUDA(dev_alloc(&d_order.p, sizeof(int32_t) * nr, s));
    DCUDA(dev_alloc(&sz.p, sizeof(uint32_t) * (size_t)nr + 16, s));
    DCUDA(cudaMemcpyAsync(d_order.p, res->order.data(), sizeof(int32_t) * nr,
                          cudaMemcpyHostToDevice, s));
    const DevReads& R = job.device_reads();
    k_out_sizes<<<grid_of(nr, 256, 1 << 14), 256, 0, s>>>(job.device_cluster(), d_order.as<int32_t>(),
                                                         name_len.as<int32_t>(), R.len, nr,
                                                         sz.as<uint32_t>());
    DevBuf sz_off(s);
    DCUDA(dev_alloc(&sz_off.p, sizeof(uint32_t) * (size_t)nr + 16, s));
    rc = scan_u32(sz.as<uint32_t>(), sz_off.as<uint32_t>(), nr, scan_tmp.as<uint32_t>(), d_total, s,
                  &h_total);
    if (rc) return rc;
    // (the output is smaller than the file, so 32-bit offsets hold for files
    // below 4 GiB; larger outputs are formatted on the host)
    DevBuf outd(s);
    const int64_t out_bytes = h_total;
    if (n < ((int64_t)1 << 32)) {
        DCUDA(dev_alloc(&outd.p, (size_t)out_bytes + 16, s));
        k_out_copy<<<grid_of(nr, 8, 1 << 16), 256, 0, s>>>(
            b, job.device_cluster(), d_order.as<int32_t>(), name_off.as<int64_t>(),
            name_len.as<int32_t>(), R.off, R.len, sz_off.as<uint32_t>(), nr, outd.as<uint8_t>(), 0);
        DCUDA(cudaGetLastError());
        res->out.resize((size_t)out_bytes);
        if (out_bytes)
            DCUDA(cudaMemcpyAsync(res->out.data(), outd.p, (size_t)out_bytes,
                                  cudaMemcpyDeviceToHost, s));
    } else {
        return fail(GSDR_EUNSUPPORTED, "device formatting of files above 4 GiB");
    }
    mark("output");
    rc = job.download(res->cluster.data());
    mark("download");
    if (rc) return rc;
    res->cluster.resize(nr);
    job.stats.ms_total = now_ms() - t0;
    job.stats.ms_prep += t_parse - t0;  // the parse and sort before the job's own preparation
    if (stats) *stats = job.stats;
    return GSDR_OK;
}

}  // namespace gsdr

using namespace gsdr;

extern "C" {

int gsdr_cluster_fasta(const char* fasta, int64_t n, const gsdr_opts* opts, gsdr_result** out,
                       gsdr_stats* stats) {
    if (!out || !opts || (!fasta && n > 0) || n < 0)
        return fail(GSDR_EINVAL, "gsdr_cluster_fasta: bad argument");
    *out = nullptr;
    gsdr_result* r = new (std::nothrow) gsdr_result();
    if (!r) return fail(GSDR_ENOMEM, "out of host memory");
    int rc = cluster_fasta(fasta, n, opts, r, stats);
    if (rc) {
        delete r;
        return rc;
    }
    *out = r;
    return GSDR_OK;
}

int gsdr_result_output(const gsdr_result* r, const char** data, int64_t* n) {
    if (!r || !data || !n) return GSDR_EINVAL;
    *data = r->out.data();
    *n = (int64_t)r->out.size();
    return GSDR_OK;
}

int32_t gsdr_result_count(const gsdr_result* r) { return r ? (int32_t)r->cluster.size() : 0; }

const int32_t* gsdr_result_cluster(const gsdr_result* r) { return r ? r->cluster.data() : nullptr; }

const int32_t* gsdr_result_order(const gsdr_result* r) { return r ? r->order.data() : nullptr; }

const int32_t* gsdr_result_lengths(const gsdr_result* r) { return r ? r->length.data() : nullptr; }

void gsdr_result_free(gsdr_result* r) { delete r; }

}  // extern "C"
