// noalloc.cu -- the alignment stage for callers that cannot allocate device
// memory (gsdr_lcs_decide_noalloc in include/gsdr.h).
//
// Some callers own every device allocation themselves: code running inside a
// framework's memory pool, a plug-in that must not grow the process's device
// footprint, or a caller that checks its memory budget up front.  They pass
// device buffers for the inputs and the output; the work space the alignment
// stage needs (round state, work counters, per-class pair queues, cutoffs and
// a decision slot per sequence) is the fixed array below, which every GPU
// that loads this library holds until the process exits.
//
// In host code `g_scratch` names a host-side stand-in, not the device array:
// its device address is fetched with cudaGetSymbolAddress once per device (on
// the first call made with that device current) and that address is what the
// kernels receive.  Every call reuses the same array, so each call first
// clears what must start at zero; two calls that overlap on the GPU (other
// streams, other host threads) race on it and give undefined results.  Each
// call reads two status words back and waits for its stream, so it returns
// with the stream idle and cannot be made while that stream is capturing.
// The address is kept for the life of the process: after a cudaDeviceReset
// of a device, the array's address there is not looked up again.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "gsdr.h"
#include "gsdr_device.cuh"
#include "gsdr_host.h"

namespace gsdr {

namespace {

constexpr int kNaMaxPairs = GSDR_NOALLOC_MAX_PAIRS;
constexpr int kNaClasses = 6;      // systolic classes 0..5: patterns of at most 1024 words
constexpr int kNaMaxWords = 1024;  // 32768 gap-free bases, the documented limit
constexpr int kNaMaxSeqs = GSDR_NOALLOC_MAX_SEQS;
constexpr int kNaMaxDevices = 64;

// Layout of the array (offsets in bytes, each 256-aligned).
constexpr size_t kOffState = 0;                                   // RoundState + counters
constexpr size_t kOffPairs = 1024;                                // kNaClasses x kNaMaxPairs
constexpr size_t kOffCut = kOffPairs + sizeof(Pair) * (size_t)kNaClasses * kNaMaxPairs;
constexpr size_t kOffCluster = kOffCut + sizeof(int32_t) * (size_t)kNaMaxSeqs;
constexpr size_t kScratchBytes = kOffCluster + sizeof(int32_t) * (size_t)kNaMaxSeqs;
static_assert(sizeof(RoundState) + 64 * sizeof(int) <= kOffPairs, "state area too small");
static_assert(kOffCut % 256 == 0 && kOffCluster % 256 == 0, "scratch areas must stay aligned");

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

std::mutex g_addr_mu;
void* g_addr[kNaMaxDevices] = {};

// Device address of g_scratch on the current device (looked up once).
int scratch_address(int dev, unsigned char** out) {
    std::lock_guard<std::mutex> lock(g_addr_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess || !p) return fail(GSDR_EDEVICE, "cudaGetSymbolAddress failed");
        g_addr[dev] = p;
    }
    *out = reinterpret_cast<unsigned char*>(g_addr[dev]);
    return GSDR_OK;
}

// Clears the round state and counters, marks every sequence undecided and
// computes the base cutoffs ceil(len * t) of kernel_createCutoff
// (cuda-version/func.cu:331-332).
__global__ void k_na_init(RoundState* st, int* work, int32_t* cluster, int32_t* cut,
                          const int32_t* __restrict__ len_raw, int n_seq, float t) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        RoundState s = {};
        s.pass = 1;
        s.n_tent = 1;
        s.R = 1;
        *st = s;
        for (int c = 0; c < 64; c++) work[c] = 0;
    }
    for (int j = i; j < n_seq; j += gridDim.x * blockDim.x) {
        cluster[j] = -1;
        cut[j] = (int)ceilf(__fmul_rn((float)len_raw[j], t));
    }
}

// Queues every pair in the alignment class of its pattern's length.  An index
// outside [0, n_seq), a pattern that appears in two pairs or a pattern longer
// than the limit sets the invalid-input flag instead (the call then fails).
__global__ void k_na_bucket(RoundState* st, Pair* pairs, int32_t* cluster,
                            const int32_t* __restrict__ len_gf,
                            const int32_t* __restrict__ pat, const int32_t* __restrict__ txt,
                            int n_pairs, int n_seq) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n_pairs;
         k += gridDim.x * blockDim.x) {
        const int p = pat[k], x = txt[k];
        if (p < 0 || p >= n_seq || x < 0 || x >= n_seq) {
            st->pair_overflow = 1;
            continue;
        }
        // one pair per pattern: the pattern's decision slot goes from -1
        // (cleared) to -2 (claimed); a second claim finds it taken
        if (atomicCAS(cluster + p, -1, -2) != -1) {
            st->pair_overflow = 1;
            continue;
        }
        const int words = (len_gf[p] + 31) >> 5;
        if (words > kNaMaxWords) {
            st->pair_overflow = 1;
            continue;
        }
        const int cls = words <= 32 ? 0 : words <= 64 ? 1 : words <= 128 ? 2 : words <= 256 ? 3
                                                                         : words <= 512 ? 4 : 5;
        const int slot = atomicAdd(&st->n_pairs[cls], 1);
        pairs[(size_t)cls * kNaMaxPairs + slot] = Pair{x, p};
    }
}

// accept[k] = 1 iff the alignment stage joined pattern pat[k] to text txt[k];
// a pair with an index outside [0, n_seq) reads nothing and gets 0 (the call
// reports it as invalid input).
__global__ void k_na_finish(const int32_t* __restrict__ cluster, const int32_t* __restrict__ pat,
                            const int32_t* __restrict__ txt, int n_pairs, int n_seq,
                            uint8_t* accept) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n_pairs;
         k += gridDim.x * blockDim.x) {
        const int p = pat[k];
        accept[k] = (p >= 0 && p < n_seq && cluster[p] == txt[k]) ? 1 : 0;
    }
}

}  // namespace
}  // namespace gsdr

using namespace gsdr;

extern "C" int gsdr_lcs_decide_noalloc(const uint32_t* d_packed, const int64_t* d_pack_off,
                                       const int32_t* d_len_raw, const int32_t* d_len_gf,
                                       int32_t n_seq, const int32_t* d_pat,
                                       const int32_t* d_txt, int32_t n_pairs, float t,
                                       uint8_t* d_accept, void* stream) {
    if (n_pairs < 0 || n_seq < 0) return fail(GSDR_EINVAL, "noalloc: negative size");
    if (n_pairs > kNaMaxPairs)
        return fail(GSDR_EINVAL, "noalloc: more pairs than GSDR_NOALLOC_MAX_PAIRS");
    if (n_seq > kNaMaxSeqs)
        return fail(GSDR_EINVAL, "noalloc: more sequences than GSDR_NOALLOC_MAX_SEQS");
    if (!(t >= 0.8f && t < 1.0f)) return fail(GSDR_EINVAL, "noalloc: threshold out of range");
    if (n_pairs == 0) return GSDR_OK;
    if (!d_packed || !d_pack_off || !d_len_raw || !d_len_gf || !d_pat || !d_txt || !d_accept)
        return fail(GSDR_EINVAL, "noalloc: null device pointer");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNaMaxDevices)
        return fail(GSDR_EDEVICE, "noalloc: no current CUDA device");
    unsigned char* base = nullptr;
    int rc = scratch_address(dev, &base);
    if (rc) return rc;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);

    DevReads R = {};
    R.n = n_seq;
    R.k = 0;
    R.len = d_len_raw;
    R.len_gf = const_cast<int32_t*>(d_len_gf);
    R.pack_off = d_pack_off;
    R.packed = const_cast<uint32_t*>(d_packed);
    R.cut_base = reinterpret_cast<int32_t*>(base + kOffCut);
    RoundBuffers B = {};
    B.st = reinterpret_cast<RoundState*>(base + kOffState);
    B.pairs = reinterpret_cast<Pair*>(base + kOffPairs);
    B.seg_cap = kNaMaxPairs;
    B.cluster = reinterpret_cast<int32_t*>(base + kOffCluster);
    int* work = reinterpret_cast<int*>(B.st + 1);

    // an error left by the caller's own earlier work is theirs: report it
    // without clearing it, before launching anything
    cudaError_t e = cudaPeekAtLastError();
    if (e != cudaSuccess)
        return fail(GSDR_EDEVICE, "noalloc: a CUDA error is pending from earlier work");
    const int threads = 256;
    const int grid = (n_seq > n_pairs ? n_seq : n_pairs) / threads + 1;
    k_na_init<<<grid < 1024 ? grid : 1024, threads, 0, s>>>(B.st, work, B.cluster, R.cut_base,
                                                           d_len_raw, n_seq, t);
    k_na_bucket<<<(n_pairs + threads - 1) / threads, threads, 0, s>>>(
        B.st, B.pairs, B.cluster, d_len_gf, d_pat, d_txt, n_pairs, n_seq);
    launch_align_stage(R, B, false, false, s);
    k_na_finish<<<(n_pairs + threads - 1) / threads, threads, 0, s>>>(B.cluster, d_pat, d_txt,
                                                                      n_pairs, n_seq, d_accept);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(GSDR_EDEVICE, cudaGetErrorString(e));
    // the flags of the state say whether every pair was valid and every wait ended
    int flags[2] = {0, 0};
    e = cudaMemcpyAsync(&flags[0], &B.st->pair_overflow, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&flags[1], &B.st->error, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(GSDR_EDEVICE, cudaGetErrorString(e));
    if (flags[0]) return fail(GSDR_EINVAL, "noalloc: index out of range, pattern in more than one pair, or pattern longer than 32768 bases");
    if (flags[1]) return fail(GSDR_ETIMEOUT, "noalloc: a device-side wait gave up");
    return GSDR_OK;
}
