// api.cu -- the C ABI: gsdr_cluster (the reference's copyData .. clustering
// sequence, cuda-version/main.cu:9-30) and gsdr_main (the CLI).
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gsdr.h"
#include "gsdr_device.cuh"
#include "gsdr_host.h"

namespace gsdr {

namespace {
thread_local std::string g_last_error;
}

int fail(int status, const char* msg) {
    g_last_error = msg ? msg : "";
    return status;
}

double now_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

namespace {

#define GSDR_CUDA(call)                                                             \
    do {                                                                            \
        cudaError_t e_ = (call);                                                    \
        if (e_ != cudaSuccess) {                                                    \
            std::string m_ = std::string(#call) + ": " + cudaGetErrorString(e_);    \
            rc = fail(e_ == cudaErrorMemoryAllocation ? GSDR_ENOMEM : GSDR_EDEVICE, \
                      m_.c_str());                                                  \
            goto done;                                                              \
        }                                                                           \
    } while (0)

inline int64_t round4(int64_t v) { return (v + 3) & ~(int64_t)3; }

// All device buffers of one clustering call, in one allocation.
struct JobMem {
    void* base = nullptr;
    size_t bytes = 0;
};

struct Carve {
    char* p;
    size_t used = 0;
    template <class T>
    T* take(size_t count) {
        size_t off = (used + 255) & ~(size_t)255;
        used = off + count * sizeof(T);
        return p ? reinterpret_cast<T*>(p + off) : nullptr;
    }
};

}  // namespace
}  // namespace gsdr

using namespace gsdr;

extern "C" {

const char* gsdr_strerror(int s) {
    switch (s) {
        case GSDR_OK: return "ok";
        case GSDR_EINVAL: return "invalid argument";
        case GSDR_ENOMEM: return "out of memory";
        case GSDR_EDEVICE: return "CUDA device error";
        case GSDR_ETIMEOUT: return "device wait timed out";
        case GSDR_EIO: return "I/O error";
        case GSDR_EUNSUPPORTED: return "unsupported input";
        case GSDR_EBUSY: return "busy";
        case GSDR_ENOTFOUND: return "not found";
        default: return "unknown status";
    }
}

const char* gsdr_last_error(void) { return g_last_error.c_str(); }

int gsdr_cluster(const gsdr_reads* reads, const gsdr_opts* opts_in, int32_t* cluster,
                 gsdr_stats* stats) {
    if (!reads || !opts_in || (!cluster && reads->n > 0))
        return fail(GSDR_EINVAL, "gsdr_cluster: null argument");
    gsdr_opts o = *opts_in;
    int rc = gsdr_resolve_opts(&o, nullptr);
    if (rc) return rc;
    const int n = reads->n;
    if (n < 0) return fail(GSDR_EINVAL, "gsdr_cluster: negative read count");
    gsdr_stats st_local;
    gsdr_stats& S = stats ? *stats : st_local;
    std::memset(&S, 0, sizeof(S));
    S.k = o.word_length;
    S.drop = o.drop;
    S.pigeon = o.pigeon;
    S.batch = 1;
    if (n == 0) return GSDR_OK;
    const int k = o.word_length;
    const bool drop = o.drop == 1;
    if (!drop && k > 7)
        return fail(GSDR_EUNSUPPORTED, "gsdr_cluster: word length above 7 is not built yet");
    if (o.pigeon == 1 && !drop)
        return fail(GSDR_EUNSUPPORTED, "gsdr_cluster: pigeon filter is not built yet");

    const double t_begin = now_ms();
    // Host-side layout: word and entry offsets from the raw lengths.
    std::vector<int64_t> pack_off(n + 1), kmer_off(n + 1);
    int64_t max_len = 0;
    pack_off[0] = 0;
    kmer_off[0] = 0;
    const int64_t kcap = (int64_t)1 << (2 * (k > 0 ? k : 1));
    for (int i = 0; i < n; i++) {
        const int64_t L = reads->length[i];
        if (L < 0) return fail(GSDR_EINVAL, "gsdr_cluster: negative length");
        if (reads->offset[i] < 0 || reads->offset[i] + L > reads->n_bytes)
            return fail(GSDR_EINVAL, "gsdr_cluster: read outside the byte buffer");
        if (L > max_len) max_len = L;
        pack_off[i + 1] = pack_off[i] + round4(L / 16 + 1);
        int64_t ents = drop ? 0 : L - k + 1;
        if (ents < 0) ents = 0;
        if (ents > kcap) ents = kcap;
        kmer_off[i + 1] = kmer_off[i] + round4(ents);
    }
    if (max_len > 32 * kMaxPatternWords)
        return fail(GSDR_EUNSUPPORTED, "gsdr_cluster: reads above 32768 bases are not built yet");

    int dev_count = 0;
    if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count <= 0)
        return fail(GSDR_EDEVICE, "gsdr_cluster: no CUDA device");
    if (o.device < 0 || o.device >= dev_count) return fail(GSDR_EINVAL, "gsdr_cluster: bad device");

    cudaStream_t s = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    cudaEvent_t ev[8] = {};
    int32_t* h_done = nullptr;
    RoundState* h_state = nullptr;
    void* dmem = nullptr;
    long long launches = 0;
    DevReads R = {};
    RoundBuffers B = {};
    {
        // Carve every buffer out of one allocation.
        Carve c{nullptr};
        auto plan = [&](Carve& cv) {
            R.n = n;
            R.k = drop ? 0 : k;
            R.bytes = cv.take<uint8_t>((size_t)reads->n_bytes + 64);
            R.off = cv.take<int64_t>(n);
            R.len = cv.take<int32_t>(n);
            R.len_gf = cv.take<int32_t>(n);
            R.pack_off = cv.take<int64_t>(n + 1);
            R.packed = cv.take<uint32_t>((size_t)pack_off[n] + 8);
            R.comp = cv.take<int4>(n);
            R.cut_word = cv.take<int32_t>(n);
            R.cut_base = cv.take<int32_t>(n);
            R.cut_pig = cv.take<int32_t>(n);
            R.kmer_off = cv.take<int64_t>(n + 1);
            R.n_kmer = cv.take<int32_t>(n);
            R.kmer = cv.take<uint32_t>((size_t)kmer_off[n] + 8);
            B.st = reinterpret_cast<RoundState*>(cv.take<char>(sizeof(RoundState) + 64));
            B.cluster = cv.take<int32_t>(n);
            B.remain[0] = cv.take<int32_t>(n);
            B.remain[1] = cv.take<int32_t>(n);
            B.pair_cap = 2 * n;
            B.pairs = cv.take<Pair>((size_t)B.pair_cap);
        };
        plan(c);
        const size_t total = c.used + 256;
        GSDR_CUDA(cudaSetDevice(o.device));
        GSDR_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        GSDR_CUDA(cudaMalloc(&dmem, total));
        Carve c2{reinterpret_cast<char*>(dmem)};
        plan(c2);
        GSDR_CUDA(cudaMallocHost(&h_done, sizeof(int32_t)));
        GSDR_CUDA(cudaMallocHost(&h_state, sizeof(RoundState)));
        for (auto& e : ev) GSDR_CUDA(cudaEventCreate(&e));

        // ---- copyData (func.cu:119-137): one H2D copy of the sequence bytes.
        GSDR_CUDA(cudaEventRecord(ev[0], s));
        GSDR_CUDA(cudaMemcpyAsync((void*)R.bytes, reads->bytes, (size_t)reads->n_bytes,
                                  cudaMemcpyHostToDevice, s));
        GSDR_CUDA(cudaMemcpyAsync((void*)R.off, reads->offset, sizeof(int64_t) * n,
                                  cudaMemcpyHostToDevice, s));
        GSDR_CUDA(cudaMemcpyAsync((void*)R.len, reads->length, sizeof(int32_t) * n,
                                  cudaMemcpyHostToDevice, s));
        GSDR_CUDA(cudaMemcpyAsync((void*)R.pack_off, pack_off.data(), sizeof(int64_t) * (n + 1),
                                  cudaMemcpyHostToDevice, s));
        GSDR_CUDA(cudaMemcpyAsync((void*)R.kmer_off, kmer_off.data(), sizeof(int64_t) * (n + 1),
                                  cudaMemcpyHostToDevice, s));
        GSDR_CUDA(cudaEventRecord(ev[1], s));

        // ---- baseToNumber + compressData + createCutoff + createPrefix
        GSDR_CUDA(cudaMemsetAsync(R.packed, 0, sizeof(uint32_t) * ((size_t)pack_off[n] + 8), s));
        launch_pack(R, o.threshold, k, s);
        launches += 1;
        GSDR_CUDA(cudaGetLastError());
        // ---- createWords + sortWords + mergeWords
        if (!drop) {
            int krc = launch_kmers(R, k, s);
            if (krc) {
                rc = fail(GSDR_EDEVICE, "k-mer kernel configuration failed");
                goto done;
            }
            launches += 1;
            GSDR_CUDA(cudaGetLastError());
        }
        GSDR_CUDA(cudaEventRecord(ev[2], s));

        // ---- clustering / clusteringDrop (func.cu:1001-1097)
        init_rounds(R, B, s);
        launches += 1;
        GSDR_CUDA(cudaGetLastError());
        if (o.stage_timing) {
            cudaEvent_t e4[4];
            for (auto& e : e4) GSDR_CUDA(cudaEventCreate(&e));
            int parity = 0;
            double fms = 0, ams = 0;
            while (true) {
                launch_plain_round(R, B, o.threshold, drop, o.pigeon, parity, s, &launches, e4);
                GSDR_CUDA(cudaGetLastError());
                GSDR_CUDA(cudaMemcpyAsync(h_done, &B.st->done, sizeof(int32_t),
                                          cudaMemcpyDeviceToHost, s));
                GSDR_CUDA(cudaStreamSynchronize(s));
                float a = 0, b = 0;
                cudaEventElapsedTime(&a, e4[0], e4[1]);
                cudaEventElapsedTime(&b, e4[1], e4[2]);
                fms += a;
                ams += b;
                parity ^= 1;
                if (*h_done) break;
            }
            S.ms_filter = fms;
            S.ms_align = ams;
            for (auto& e : e4) cudaEventDestroy(e);
        } else {
            const int unroll = 16;  // rounds per graph launch (even: remain buffers alternate)
            GSDR_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
            long long per_graph = 0;
            for (int r = 0; r < unroll; r++)
                launch_plain_round(R, B, o.threshold, drop, o.pigeon, r & 1, s, &per_graph,
                                   nullptr);
            GSDR_CUDA(cudaStreamEndCapture(s, &graph));
            GSDR_CUDA(cudaGraphInstantiate(&gexec, graph, 0));
            while (true) {
                GSDR_CUDA(cudaGraphLaunch(gexec, s));
                launches += per_graph;
                GSDR_CUDA(cudaMemcpyAsync(h_done, &B.st->done, sizeof(int32_t),
                                          cudaMemcpyDeviceToHost, s));
                GSDR_CUDA(cudaStreamSynchronize(s));
                if (*h_done) break;
            }
        }
        GSDR_CUDA(cudaEventRecord(ev[3], s));
        GSDR_CUDA(cudaMemcpyAsync(cluster, B.cluster, sizeof(int32_t) * n, cudaMemcpyDeviceToHost,
                                  s));
        GSDR_CUDA(cudaMemcpyAsync(h_state, B.st, sizeof(RoundState), cudaMemcpyDeviceToHost, s));
        GSDR_CUDA(cudaEventRecord(ev[4], s));
        GSDR_CUDA(cudaStreamSynchronize(s));
        GSDR_CUDA(cudaGetLastError());
        if (h_state->pair_overflow) {
            rc = fail(GSDR_EDEVICE, "alignment queue overflow");
            goto done;
        }
        float ms = 0;
        cudaEventElapsedTime(&ms, ev[0], ev[1]);
        S.ms_h2d = ms;
        cudaEventElapsedTime(&ms, ev[1], ev[2]);
        S.ms_prep = ms;
        cudaEventElapsedTime(&ms, ev[2], ev[3]);
        S.ms_cluster = ms;
        cudaEventElapsedTime(&ms, ev[3], ev[4]);
        S.ms_d2h = ms;
        S.rounds = h_state->rounds;
        S.passes = h_state->passes;
        S.pairs_prefilter = (int64_t)h_state->cnt_prefilter;
        S.pairs_word = (int64_t)h_state->cnt_word;
        S.pairs_aligned = (int64_t)h_state->cnt_aligned;
        S.pairs_accepted = (int64_t)h_state->cnt_accepted;
        S.cells = (double)h_state->cells;
        S.filter_bytes = (double)h_state->filter_bytes;
        S.kernel_launches = launches;
        rc = GSDR_OK;
    }
done:
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    for (auto& e : ev)
        if (e) cudaEventDestroy(e);
    if (dmem) cudaFree(dmem);
    if (h_done) cudaFreeHost(h_done);
    if (h_state) cudaFreeHost(h_state);
    if (s) cudaStreamDestroy(s);
    S.ms_total = now_ms() - t_begin;
    return rc;
}

// main (cuda-version/main.cu:3-36).
int gsdr_main(int argc, char** argv) {
    const double t0 = now_ms();
    gsdr_opts o;
    std::vector<char> in(4096), out(4096);
    if (gsdr_check_option(argc, argv, &o, in.data(), out.data(), (int64_t)in.size()) != GSDR_OK) {
        std::printf("Please check parameters.\n%s\n", gsdr_last_error());
        std::printf("cluster i inputFile o outputFile t threshold [w wordLength] [d 0|1] [p 0|1]\n");
        return 0;
    }
    o.verbose = 1;
    std::printf("input file:\t%s\noutput file:\t%s\nthreshold:\t%g\nword length:\t%d\ndrop filter\t%d\n",
                in.data(), out.data(), (double)o.threshold, o.word_length, o.drop);
    gsdr_fasta* f = nullptr;
    int rc = gsdr_fasta_read(in.data(), &f);
    if (rc) {
        std::printf("error: %s (%s)\n", gsdr_strerror(rc), gsdr_last_error());
        return 1;
    }
    gsdr_reads v;
    gsdr_fasta_view(f, &v);
    if (v.n > 0)
        std::printf("longest:\t%d\nshortest:\t%d\nreads count:\t%d\n", v.length[0],
                    v.length[v.n - 1], v.n);
    std::vector<int32_t> cl(v.n > 0 ? v.n : 1);
    gsdr_stats st;
    rc = gsdr_cluster(&v, &o, cl.data(), &st);
    if (rc) {
        std::printf("error: %s (%s)\n", gsdr_strerror(rc), gsdr_last_error());
        gsdr_fasta_free(f);
        return 1;
    }
    int64_t written = 0;
    rc = gsdr_fasta_write(out.data(), f, cl.data(), &written);
    gsdr_fasta_free(f);
    if (rc) {
        std::printf("error: %s (%s)\n", gsdr_strerror(rc), gsdr_last_error());
        return 1;
    }
    std::printf("cluster count:\t%lld\n", (long long)written);
    std::printf("time consuming:\t%.0fms\n", now_ms() - t0);
    return 0;
}

}  // extern "C"
