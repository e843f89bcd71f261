// api.cu -- the C ABI around gsdr::Job: gsdr_cluster (the reference's
// copyData .. clustering sequence, cuda-version/main.cu:9-30), the job entry
// points, and gsdr_main (the CLI).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "devmem.h"
#include "gsdr.h"
#include "gsdr_device.cuh"
#include "gsdr_host.h"
#include "nvtx_range.h"
#include "gsdr_testing.h"
#include "job.h"
#include "lcs_band.cuh"

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

int cuda_fail(cudaError_t e, const char* what) {
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    return fail(e == cudaErrorMemoryAllocation ? GSDR_ENOMEM : GSDR_EDEVICE, m.c_str());
}

#define JCUDA(call)                                   \
    do {                                              \
        cudaError_t e_ = (call);                      \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

// Sub-allocations of one device allocation, each 256-byte aligned.
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

// Layout plan shared by footprint() and plan_and_alloc().
struct Plan {
    std::vector<int64_t> pack_off, kmer_off;
    int64_t max_len = 0;
    int r_max = 1;          // largest R (tentatives per pass)
    int64_t idx_cap = 0;    // > 0: batched word filter by inverted index, postings capacity
    bool idx_smem = false;  // that index fits the filter's shared memory (16-bit copy)
    bool bits = false;      // batched word filter by k-mer presence bitmaps
    bool masks = false;     // batched word filter by tentative masks
    int mask_planes = 8;    // their count planes (10 where a read has over 255 entries)
    // pigeon filter (p 1): low 16 bits of each read's offset in the
    // reference's padded layout (copyData, func.cu:119-137: L/16*16 + 16 per read)
    std::vector<uint16_t> refoff16;
    int variant = 0;  // gsdr_opts::variant
};

constexpr int kSmemOptin = 227 * 1024;  // per-block shared memory limit of sm_100 / sm_103

// R_max of a job: the caller's batch, or 256 for the automatic choice (which
// make_plan raises for the table and index forms of the word filter).
int job_r_max(const gsdr_opts& o) {
    return o.batch == 0 ? 256 : (o.batch > kMaxBatch ? kMaxBatch : (o.batch < 1 ? 1 : o.batch));
}

// Sparse k-mer spaces (mean distinct k-mers per read at most 4^k /
// kIndexDensity), where almost every table lookup of the table form would
// read a zero, take the tentative masks when every read has at most
// kMaskMaxEntries k-mer entries, else the inverted index of the tentatives'
// k-mers.  GSDR_BFILTER=table|index|bits|masks forces a form.
constexpr int64_t kIndexDensity = 8;

int make_plan(const gsdr_reads* reads, const gsdr_opts& o, Plan& P, PlanPreset* pre) {
    const int n = reads->n;
    const bool drop = o.drop == 1;
    const int k = o.word_length;
    P.variant = o.variant;
    P.r_max = (o.batch == 1 || (!drop && k >= kWideK)) ? 1 : job_r_max(o);
    const int64_t kcap = (int64_t)1 << (2 * (k > 0 ? k : 1));
    // the per-read layout (plan_chunks.h): the caller's, when it computed it
    // for these options and every read was in range, else one pass here
    PlanChunk sums;
    if (pre && pre->k == k && pre->drop == drop && pre->sums.valid &&
        pre->pack_off.size() == (size_t)n + 1 && pre->kmer_off.size() == (size_t)n + 1) {
        P.pack_off.swap(pre->pack_off);
        P.kmer_off.swap(pre->kmer_off);
        sums = pre->sums;
    } else {
        P.pack_off.assign(n + 1, 0);
        P.kmer_off.assign(n + 1, 0);
        sums = plan_chunk(reads->offset, reads->length, reads->n_bytes, 0, n, k, drop,
                          P.pack_off.data(), P.kmer_off.data());
        if (!sums.valid)
            for (int i = 0; i < n; i++) {
                const int64_t L = reads->length[i];
                if (L < 0) return fail(GSDR_EINVAL, "negative read length");
                if (reads->offset[i] < 0 || reads->offset[i] + L > reads->n_bytes)
                    return fail(GSDR_EINVAL, "read outside the byte buffer");
            }
    }
    P.max_len = sums.max_len;
    const int64_t ents_sum = sums.ents_sum, ents_max = sums.ents_max;
    const bool sorted = sums.sorted;
    std::vector<int64_t> head;  // entries of the first kMaxBatch reads, prefix sums
    head.reserve(kMaxBatch + 1);
    head.push_back(0);
    for (int i = 0; i < n && i < kMaxBatch; i++)
        head.push_back(head.back() + plan_entries(reads->length[i], k, drop));
    if (o.pigeon == 1 && !drop) {
        P.refoff16.resize(n);
        int64_t ro = 0;
        for (int i = 0; i < n; i++) {
            P.refoff16[i] = (uint16_t)ro;
            ro += (int64_t)reads->length[i] / 16 * 16 + 16;
        }
    }
    if (o.batch != 1 && !drop && n > 0 && k < kWideK) {
        bool index = ents_sum * kIndexDensity <= kcap * (int64_t)n;
        // k <= 6: the two-level count bitmaps (measured faster than the
        // tables on every workload tried: 200k reads of 300-10,000 bp 50.2
        // against 53.3 ms, jobs of 150-5,000 bp 0.90 against 3.96 s at 200k
        // reads and 82 against 298 ms at 50k, 10k reads of 200-1,000 bp 7.0
        // against 8.4 ms)
        bool bits = !index && k <= kMaxBits2K;
        // sparse spaces with short reads: the tentative masks, whose counts
        // (8 or 10 bit planes) hold reads of at most kMaskMaxEntries k-mers
        const bool masks_ok = k <= kMaxBits2K && ents_max <= kMaskMaxEntries;
        P.mask_planes = ents_max <= kMaskEntries8 ? 8 : 10;
        bool masks = index && masks_ok;
        // the caller's choice (word_filter), else GSDR_BFILTER=table|index|bits|masks
        int form = o.word_filter;
        if (form == 0) {
            const char* f = std::getenv("GSDR_BFILTER");
            if (f && std::strcmp(f, "table") == 0) form = 1;
            if (f && std::strcmp(f, "index") == 0) form = 2;
            if (f && std::strcmp(f, "bits") == 0) form = 3;
            if (f && std::strcmp(f, "masks") == 0) form = 4;
        }
        if (form == 1) index = false, bits = false, masks = false;
        if (form == 2) index = true, bits = false, masks = false;
        if (form == 3) index = false, bits = k <= kMaxBits2K, masks = false;
        if (form == 4 && masks_ok) index = false, bits = false, masks = true;
        if (masks) index = false;
        P.bits = bits;
        P.masks = masks;
        // automatic R with the table and bitmap forms: the largest R for
        // k <= 6 (the table form measured 22.6 us per representative at
        // R_max 1024 against 25.5 at 256 on the 200k-read workload), 256 for
        // k = 7, whose tables and bitmaps are four times larger (200k reads of
        // 150-5,000 bp at t = 0.90: bitmaps 1.19 s at 256 against 1.72 s at
        // 1024, tables 3.7 against 4.4 s)
        if (o.batch == 0 && !index) P.r_max = k >= 7 && !masks ? 256 : kMaxBatch;
        if (index) {
            // a pass indexes at most R_max tentatives: for length-sorted reads
            // those hold at most the first R_max reads' entries
            auto cap_of = [&](int r) {
                const int m = std::min<int>(r, (int)head.size() - 1);
                return std::max<int64_t>(sorted ? head[m] : ents_max * r, 1);
            };
            if (o.batch == 0 && sorted) {
                // automatic R: the largest R_max (in steps of 64, at least the
                // default) whose index still fits the filter's shared memory
                for (int r = kMaxBatch; r > P.r_max; r -= 64)
                    if (index_in_smem(k, r, cap_of(r), kSmemOptin)) {
                        P.r_max = r;
                        break;
                    }
            }
            P.idx_cap = cap_of(P.r_max);
            P.idx_smem = index_in_smem(k, P.r_max, P.idx_cap, kSmemOptin);
        }
    }
    return GSDR_OK;
}

size_t carve_all(char* base, int n, int64_t n_bytes, const Plan& P, bool drop, int k, DevReads& R,
                 RoundBuffers& B) {
    Carve c{base};
    R.n = n;
    R.k = drop ? 0 : k;
    R.bytes = c.take<uint8_t>((size_t)n_bytes + 64);
    R.off = c.take<int64_t>(n);
    R.len = c.take<int32_t>(n);
    R.len_gf = c.take<int32_t>(n);
    R.pack_off = c.take<int64_t>(n + 1);
    R.packed = c.take<uint32_t>((size_t)P.pack_off[n] + 8);
    R.comp = c.take<int4>(n);
    R.cut_word = c.take<int32_t>(n);
    R.cut_base = c.take<int32_t>(n);
    R.cut_pig = c.take<int32_t>(n);
    R.kmer_off = c.take<int64_t>(n + 1);
    R.n_kmer = c.take<int32_t>(n);
    R.kmer = c.take<uint32_t>((size_t)P.kmer_off[n] + 8);
    R.bm = c.take<uint32_t>(2 * (size_t)P.pack_off[n] + 8);
    R.variant = P.variant;
    R.strict = P.variant == 1 ? 1 : 0;
    R.brk = P.variant == 1 && !drop ? c.take<uint32_t>((size_t)P.pack_off[n] + 8) : nullptr;
    // presence bitmaps: for the plain filter's bound (k <= 6) and for the
    // batched two-level filter (k <= 7)
    const bool bits = !drop && (k <= kMaxBitsK || P.bits);
    const size_t nbw = bits ? ((size_t)1 << (2 * k)) / 32 : 0;
    R.kbits = bits ? c.take<uint32_t>((size_t)n * nbw) : nullptr;
    R.kextra = bits ? c.take<int32_t>(n) : nullptr;
    R.kbits2 = P.bits ? c.take<uint32_t>((size_t)n * nbw) : nullptr;
    R.kextra3 = P.bits ? c.take<int32_t>(n) : nullptr;
    B.st = reinterpret_cast<RoundState*>(c.take<char>(sizeof(RoundState) + 4 * 64));
    B.cluster = c.take<int32_t>(n);
    B.remain[0] = c.take<int32_t>(n);
    B.remain[1] = c.take<int32_t>(n);
    B.seg_cap = n > (1 << 16) ? n : (1 << 16);
    B.pairs = c.take<Pair>((size_t)B.seg_cap * kAlignClasses);
    B.tent = c.take<int32_t>(kMaxBatch);
    B.tidx = c.take<uint32_t>(n);
    B.best = c.take<uint32_t>(n);
    B.tt = c.take<uint32_t>((size_t)kMaxBatch * kTTWords);
    B.ttrow = c.take<uint32_t>(kTTWords);
    B.survive = c.take<uint32_t>(kTTWords);
    B.acc_cap = 2 * B.seg_cap;
    B.acc = c.take<Pair>((size_t)B.acc_cap);
    B.r_max = P.r_max;
    B.idx_cap = P.idx_cap;
    B.idx_off = P.idx_cap > 0 ? c.take<uint32_t>(((size_t)1 << (2 * k)) + 1) : nullptr;
    B.idx_post = P.idx_cap > 0 ? c.take<uint32_t>((size_t)P.idx_cap) : nullptr;
    // 16-byte copies read whole: both rounded up to 8 entries
    B.idx_off16 = P.idx_smem ? c.take<uint16_t>(((size_t)1 << (2 * k)) + 8) : nullptr;
    B.idx_post16 = P.idx_smem ? c.take<uint16_t>((size_t)P.idx_cap + 8) : nullptr;
    // (four alignment queues' worth: a pass whose open pairs overflow it is redone)
    B.amb_cap = P.bits || P.masks ? 4 * B.seg_cap : 0;
    B.amb = P.bits || P.masks ? c.take<Pair>((size_t)B.amb_cap) : nullptr;
    B.amb2 = P.bits || P.masks ? c.take<Pair>((size_t)B.amb_cap) : nullptr;
    B.amb_idx = P.bits || P.masks ? c.take<int32_t>(4 * (size_t)(kMaxBatch + 1)) : nullptr;
    B.tmask_rwq = P.masks ? (P.r_max + 127) / 128 : 0;
    B.tmask_planes = P.mask_planes;
    B.tmask = P.masks ? c.take<uint4>(((size_t)1 << (2 * k)) * B.tmask_rwq) : nullptr;
    B.tmask_ex = P.masks ? c.take<int32_t>(kMaxBatch) : nullptr;
    // word lengths 8..12: k-mer ids and counts apart, the global table, the
    // per-CTA hash scratch (slots: a power of two >= 2 x the longest read)
    const bool wide = !drop && k >= kWideK;
    R.kcnt = wide ? c.take<uint16_t>((size_t)P.kmer_off[n] + 8) : nullptr;
    R.gtab = wide ? c.take<uint16_t>((size_t)1 << (2 * k)) : nullptr;
    // (a read holds at most 4^k distinct k-mers; very long reads leave fewer
    // CTAs counting, each with a larger table, within 256 MB of scratch)
    int64_t distinct = std::min<int64_t>(P.max_len, (int64_t)1 << (2 * k));
    int slots = 1024;
    while (wide && slots < 2 * distinct) slots <<= 1;
    R.khash_slots = wide ? slots : 0;
    R.khash_ctas = wide ? (int)std::max<int64_t>(
                              1, std::min<int64_t>(kHashCtas, (256ll << 20) / (12ll * slots)))
                        : 0;
    R.khash = wide ? c.take<uint32_t>((size_t)R.khash_ctas * 3 * slots) : nullptr;
    // patterns longer than one systolic group: chunk carries of k_align_long
    B.long_words = P.max_len > 32 * kMaxPatternWords ? (int)((P.max_len + 62) / 32 + 2) : 0;
    B.long_carry =
        B.long_words ? c.take<uint32_t>((size_t)num_sms() * 2 * B.long_words) : nullptr;
    const bool pig = !P.refoff16.empty();
    R.pig = pig ? c.take<uint16_t>((size_t)n * 256) : nullptr;
    R.pidx = pig ? c.take<uint16_t>((size_t)n_bytes + 8) : nullptr;
    R.refoff16 = pig ? c.take<uint16_t>(n) : nullptr;
    R.pig_cap = pig ? 4 * B.seg_cap : 0;
    R.pig_q = pig ? c.take<Pair>((size_t)R.pig_cap) : nullptr;
    return c.used + 256;
}

int validate(const gsdr_reads* reads, const gsdr_opts* opts_in, gsdr_opts& o) {
    if (!reads || !opts_in) return fail(GSDR_EINVAL, "null argument");
    if (reads->n < 0) return fail(GSDR_EINVAL, "negative read count");
    if (reads->n > 0 && (!reads->offset || !reads->length || (!reads->bytes && reads->n_bytes)))
        return fail(GSDR_EINVAL, "null read arrays");
    o = *opts_in;
    int rc = gsdr_resolve_opts(&o, nullptr);
    if (rc) return rc;
    return GSDR_OK;
}

}  // namespace

Job::~Job() {
    if (stream) cudaStreamSynchronize(stream);
    if (gexec_) cudaGraphExecDestroy(gexec_);
    if (graph_) cudaGraphDestroy(graph_);
    for (auto& e : ev_)
        if (e) cudaEventDestroy(e);
    // back to the library's pool after this job's own work (no device-wide wait)
    if (dmem_) dev_free(dmem_, stream);
    pinned_release(h_done_);
    pinned_release(h_state_);
    if (own_stream_ && stream) cudaStreamDestroy(stream);
}

int64_t Job::footprint(const gsdr_reads* reads, const gsdr_opts* opts) {
    gsdr_opts o;
    if (validate(reads, opts, o)) return -1;
    Plan P;
    if (make_plan(reads, o, P, nullptr)) return -1;
    DevReads R{};
    RoundBuffers B{};
    return (int64_t)carve_all(nullptr, reads->n, reads->n_bytes, P, o.drop == 1, o.word_length,
                              R, B);
}

int Job::init(const gsdr_reads* reads, const gsdr_opts* opts_in, cudaStream_t s,
               PlanPreset* preset) {
    const double t_start = now_ms();
    int rc = validate(reads, opts_in, opts);
    if (rc) return rc;
    const bool tuned = use_tune_cache && reads->n > 0 && apply_tuned(reads, opts);
    const double t_tuned = now_ms();
    n = reads->n;
    n_bytes_ = reads->n_bytes;
    std::memset(&stats, 0, sizeof(stats));
    stats.k = opts.word_length;
    stats.drop = opts.drop;
    stats.pigeon = opts.pigeon;
    stats.tuned = tuned ? 1 : 0;
    // word lengths 8..12 run one representative per round (the batched
    // filters keep the 4^k k-mer space on chip)
    batched_ = opts.batch != 1 && !(opts.drop == 0 && opts.word_length >= kWideK);
    {
        const char* tr = std::getenv("GSDR_TRACE");
        trace_ = tr && tr[0] == '1';
    }
    if (tuned && trace_)
        std::fprintf(stderr,
                     "gsdr trace: knobs from the tuning cache: batch %d word_filter %d "
                     "group_words %d band_serial %d align_blocks %d filter_blocks %d "
                     "graph_steps %d\n",
                     opts.batch, opts.word_filter, opts.group_words, opts.band_serial,
                     opts.align_blocks, opts.filter_blocks, opts.graph_steps);
    Plan P;
    rc = make_plan(reads, opts, P, preset);
    if (rc) return rc;
    const double t_plan = now_ms();
    // A read with 65,536 or more k-mers can reach a word-filter sum of 65,536,
    // which the batched filters' paired 16-bit sums do not hold: such jobs
    // run one representative per round (32-bit sums)
    if (batched_ && opts.drop == 0 && P.max_len - opts.word_length + 1 > 65535) {
        batched_ = false;
        P.r_max = 1;
        P.idx_cap = 0;
        P.idx_smem = false;
        P.bits = false;
        P.masks = false;
    }
    r_max_ = P.r_max;
    stats.batch = batched_ ? r_max_ : 1;
    if (P.max_len > kMaxReadBases)
        return fail(GSDR_EUNSUPPORTED, "reads above 16,777,216 bases are not built yet");
    int dev_count = 0;
    if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count <= 0)
        return fail(GSDR_EDEVICE, "no CUDA device");
    if (opts.device < 0 || opts.device >= dev_count) return fail(GSDR_EINVAL, "bad device");
    JCUDA(cudaSetDevice(opts.device));
    if (s) {
        stream = s;
    } else {
        JCUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        own_stream_ = true;
    }
    for (auto& e : ev_) JCUDA(cudaEventCreate(&e));
    static_assert(sizeof(RoundState) <= kPinnedSlot, "round state exceeds a pinned slot");
    h_done_ = static_cast<int32_t*>(pinned_slot());
    h_state_ = static_cast<RoundState*>(pinned_slot());
    if (!h_done_ || !h_state_) return fail(GSDR_ENOMEM, "pinned host memory");
    if (n == 0) return GSDR_OK;
    const double t_device = now_ms();
    dbytes_ = carve_all(nullptr, n, n_bytes_, P, opts.drop == 1, opts.word_length, R_, B_);
    JCUDA(dev_alloc(&dmem_, dbytes_, stream));
    carve_all(reinterpret_cast<char*>(dmem_), n, n_bytes_, P, opts.drop == 1, opts.word_length,
              R_, B_);
    if (trace_)
        std::fprintf(stderr,
                     "gsdr trace: job init: options and tuning cache %.3f plan %.3f device, "
                     "stream and events %.3f allocation %.3f ms\n",
                     t_tuned - t_start, t_plan - t_tuned, t_device - t_plan, now_ms() - t_device);
    stats.word_index = P.idx_cap > 0 ? 1 : P.bits ? 2 : P.masks ? 3 : 0;
    R_.threshold = opts.threshold;
    // band tiles of the banded alignment kernels (gsdr_opts; 0 = automatic,
    // where the environment may still override the defaults)
    R_.band_serial = opts.band_serial > 0   ? opts.band_serial
                     : opts.band_serial < 0 ? 0
                                            : kBandMaxSerial;
    if (opts.band_serial == 0)
        if (const char* bs = std::getenv("GSDR_BAND_SERIAL")) R_.band_serial = std::atoll(bs);
    R_.align_blocks = opts.align_blocks;
    R_.filter_blocks = opts.filter_blocks;
    R_.group_max_w = opts.group_words > 0 ? std::min(opts.group_words, kGroupMaxWords)
                                          : opts.group_words < 0 ? 0 : kGroupMaxWords;
    if (opts.group_words == 0)
        if (const char* gw = std::getenv("GSDR_GROUP_MAXW"))
            R_.group_max_w = std::min(std::max(std::atoi(gw), 0), kGroupMaxWords);
    refoff16_.swap(P.refoff16);
    pack_off_.swap(P.pack_off);
    kmer_off_.swap(P.kmer_off);
    return GSDR_OK;
}

int Job::upload(const gsdr_reads* reads, const void* dev_bytes) {
    if (n == 0) return GSDR_OK;
    JCUDA(cudaEventRecord(ev_[0], stream));
    // bytes already on the device are read in place (a copy of the 200k-read
    // workload's 300 MB took 0.2 ms); the carved copy stays unused
    if (dev_bytes)
        R_.bytes = static_cast<const uint8_t*>(dev_bytes);
    else
        JCUDA(cudaMemcpyAsync((void*)R_.bytes, reads->bytes, (size_t)reads->n_bytes,
                              cudaMemcpyHostToDevice, stream));
    JCUDA(cudaMemcpyAsync((void*)R_.off, reads->offset, sizeof(int64_t) * n,
                          cudaMemcpyHostToDevice, stream));
    JCUDA(cudaMemcpyAsync((void*)R_.len, reads->length, sizeof(int32_t) * n,
                          cudaMemcpyHostToDevice, stream));
    JCUDA(cudaMemcpyAsync((void*)R_.pack_off, pack_off_.data(), sizeof(int64_t) * (n + 1),
                          cudaMemcpyHostToDevice, stream));
    JCUDA(cudaMemcpyAsync((void*)R_.kmer_off, kmer_off_.data(), sizeof(int64_t) * (n + 1),
                          cudaMemcpyHostToDevice, stream));
    if (R_.refoff16)
        JCUDA(cudaMemcpyAsync((void*)R_.refoff16, refoff16_.data(), sizeof(uint16_t) * n,
                              cudaMemcpyHostToDevice, stream));
    JCUDA(cudaEventRecord(ev_[1], stream));
    JCUDA(cudaStreamSynchronize(stream));  // host buffers may be released after upload
    float ms = 0;
    cudaEventElapsedTime(&ms, ev_[0], ev_[1]);
    stats.ms_h2d = ms;
    return GSDR_OK;
}

// One round (plain) or one pass (batched) of the device loop.
void Job::launch_step(int parity, long long* count, cudaEvent_t* ev4) {
    if (batched_) launch_batch_pass(R_, B_, opts.drop, parity, stream, count, ev4);
    else launch_plain_round(R_, B_, opts.drop, parity, stream, count, ev4);
}

int Job::capture_graph() {
    if (gexec_) return GSDR_OK;
    // steps per graph launch (the staging depth); even, so the remain buffers alternate
    const int unroll = opts.graph_steps > 0 ? opts.graph_steps : (batched_ ? 4 : 16);
    JCUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeRelaxed));
    long long per = 0;
    for (int r = 0; r < unroll; r++) launch_step(r & 1, &per, nullptr);
    cudaError_t e = cudaStreamEndCapture(stream, &graph_);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    JCUDA(cudaGraphInstantiate(&gexec_, graph_, 0));
    graph_launches_per_ = per;
    return GSDR_OK;
}

int Job::loop_graph() {
    int rc = capture_graph();
    if (rc) return rc;
    while (true) {
        JCUDA(cudaGraphLaunch(gexec_, stream));
        stats.kernel_launches += graph_launches_per_;
        JCUDA(cudaMemcpyAsync(h_done_, &B_.st->done, sizeof(int32_t), cudaMemcpyDeviceToHost,
                              stream));
        JCUDA(cudaStreamSynchronize(stream));
        if (*h_done_) break;
    }
    return GSDR_OK;
}

int Job::loop_timed() {
    cudaEvent_t e4[4] = {};
    for (auto& e : e4) JCUDA(cudaEventCreate(&e));
    // One graph per remain-buffer parity holding one step's kernels with event
    // records between its stages (external event nodes): the step's launches
    // reach the device together, so the events time the device work alone and
    // not the host's launch calls.
    cudaGraph_t g[2] = {};
    cudaGraphExec_t gx[2] = {};
    long long per_step = 0;
    int rc = GSDR_OK;
    for (int p = 0; p < 2 && rc == GSDR_OK; p++) {
        long long per = 0;
        cudaError_t e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeRelaxed);
        if (e == cudaSuccess) {
            launch_step(p, &per, e4);
            e = cudaStreamEndCapture(stream, &g[p]);
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&gx[p], g[p], 0);
        if (e != cudaSuccess) rc = cuda_fail(e, "timed step capture");
        per_step = per;
    }
    int parity = 0;
    double fms = 0, ams = 0;
    long long launches = 0;
    unsigned long long fbytes_prev = 0;
    stats.filter_max_bytes = stats.filter_max_ms = 0;
    while (rc == GSDR_OK) {
        cudaError_t e = cudaGraphLaunch(gx[parity], stream);
        launches += per_step;
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(h_done_, &B_.st->done, sizeof(int32_t), cudaMemcpyDeviceToHost,
                                stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "timed round");
            break;
        }
        float a = 0, b = 0;
        cudaEventElapsedTime(&a, e4[0], e4[1]);
        cudaEventElapsedTime(&b, e4[1], e4[2]);
        fms += a;
        ams += b;
        // input bytes of this step's filter launch: the counter's growth
        unsigned long long fbytes = 0;
        if (cudaMemcpy(&fbytes, &B_.st->filter_bytes, sizeof(fbytes), cudaMemcpyDeviceToHost) ==
            cudaSuccess) {
            const double step_bytes = (double)(fbytes - fbytes_prev);
            if (step_bytes > stats.filter_max_bytes) {
                stats.filter_max_bytes = step_bytes;
                stats.filter_max_ms = a;
            }
            fbytes_prev = fbytes;
        }
        if (trace_) {
            // per-step trace on stderr: the state after the step
            RoundState h;
            if (cudaMemcpy(&h, B_.st, sizeof(h), cudaMemcpyDeviceToHost) == cudaSuccess) {
                // queues: systolic classes | lane-band classes | group-band classes
                std::string q;
                for (int c = 0; c < kAlignClasses; c++)
                    q += (c == kSysClasses || c == kSysClasses + kBandClasses ? " | " : " ") +
                         std::to_string(h.n_pairs[c]);
                std::fprintf(stderr,
                             "gsdr trace: step %lld rounds %lld tentatives %d R %d remain %d "
                             "aligned %llu filter %.3f ms align %.3f ms filter_bytes %llu "
                             "open %d queues%s\n",
                             (long long)h.passes, (long long)h.rounds, h.n_tent, h.R, h.n_remain,
                             (unsigned long long)h.cnt_aligned, a, b,
                             (unsigned long long)h.filter_bytes, h.n_amb, q.c_str());
            }
        }
        parity ^= 1;
        if (*h_done_) break;
    }
    stats.ms_filter = fms;
    stats.ms_align = ams;
    stats.kernel_launches += launches;
    for (int p = 0; p < 2; p++) {
        if (gx[p]) cudaGraphExecDestroy(gx[p]);
        if (g[p]) cudaGraphDestroy(g[p]);
    }
    for (auto& e : e4) cudaEventDestroy(e);
    return rc;
}

int Job::run(int pass_limit, const int32_t* resume) {
    if (n == 0) return GSDR_OK;
    NvtxRange range_run("gsdr: job run");
    const double t0 = now_ms();
    const int k = opts.word_length;
    const bool drop = opts.drop == 1;
    stats.kernel_launches = 0;
    stats.ms_filter = stats.ms_align = 0;
    stats.filter_max_bytes = stats.filter_max_ms = 0;
    JCUDA(cudaSetDevice(opts.device));
    JCUDA(cudaEventRecord(ev_[1], stream));
    NvtxRange range_prep("gsdr: preparation");
    // baseToNumber + compressData + createCutoff + createPrefix (func.cu:139-403)
    JCUDA(cudaMemsetAsync(R_.packed, 0, sizeof(uint32_t) * ((size_t)pack_off_[n] + 8), stream));
    if (R_.brk)
        JCUDA(cudaMemsetAsync(R_.brk, 0, sizeof(uint32_t) * ((size_t)pack_off_[n] + 8), stream));
    launch_pack(R_, opts.threshold, k, stream);
    launch_planes(R_, stream);
    stats.kernel_launches += 2;
    if (R_.pig) {
        // createPigeon (func.cu:252-270)
        launch_pigeon_index(R_, stream);
        stats.kernel_launches += 1;
    }
    JCUDA(cudaGetLastError());
    // createWords + sortWords + mergeWords (func.cu:405-653)
    if (R_.gtab)
        JCUDA(cudaMemsetAsync(R_.gtab, 0, sizeof(uint16_t) * ((size_t)1 << (2 * k)), stream));
    if (!drop) {
        if (launch_kmers(R_, k, stream)) return fail(GSDR_EDEVICE, "k-mer kernel configuration");
        stats.kernel_launches += 1;
        JCUDA(cudaGetLastError());
    }
    JCUDA(cudaEventRecord(ev_[2], stream));
    range_prep.end();
    // clustering / clusteringDrop (func.cu:1001-1097), from the start or from
    // a checkpoint's cluster array
    if (resume) {
        JCUDA(cudaMemcpyAsync(B_.cluster, resume, sizeof(int32_t) * n, cudaMemcpyHostToDevice,
                              stream));
        resume_rounds(R_, B_, batched_ ? 1 : 0, r_max_, stream, pass_limit);
        stats.kernel_launches += 3;
    } else {
        init_rounds(R_, B_, batched_ ? 1 : 0, r_max_, stream, pass_limit);
        stats.kernel_launches += 1;
    }
    JCUDA(cudaGetLastError());
    NvtxRange range_loop(batched_ ? "gsdr: batched passes" : "gsdr: rounds");
    int rc = opts.stage_timing ? loop_timed() : loop_graph();
    range_loop.end();
    if (rc) return rc;
    JCUDA(cudaEventRecord(ev_[3], stream));
    JCUDA(cudaMemcpyAsync(h_state_, B_.st, sizeof(RoundState), cudaMemcpyDeviceToHost, stream));
    JCUDA(cudaStreamSynchronize(stream));
    JCUDA(cudaGetLastError());
    if (h_state_->error == 2) return fail(GSDR_ENOMEM, "alignment queue overflow");
    if (h_state_->error == 3) return fail(GSDR_EDEVICE, "k-mer index capacity exceeded");
    if (h_state_->error) return fail(GSDR_ETIMEOUT, "a device-side wait gave up");
    if (!batched_ && h_state_->pair_overflow) return fail(GSDR_EDEVICE, "alignment queue overflow");
    float ms = 0;
    cudaEventElapsedTime(&ms, ev_[1], ev_[2]);
    stats.ms_prep = ms;
    cudaEventElapsedTime(&ms, ev_[2], ev_[3]);
    stats.ms_cluster = ms;
    const RoundState& h = *h_state_;
    stats.rounds = h.rounds;
    stats.passes = h.passes;
    stats.pairs_prefilter = (int64_t)h.cnt_prefilter;
    stats.pairs_word = (int64_t)h.cnt_word;
    stats.pairs_aligned = (int64_t)(h.cnt_aligned - h.cnt_pig_reject);
    stats.pairs_accepted = (int64_t)h.cnt_accepted;
    stats.cells = (double)h.cells;
    stats.cells_computed = (double)h.cells_done;
    stats.filter_bytes = (double)h.filter_bytes;
    stats.ms_total = now_ms() - t0;
    return GSDR_OK;
}

int Job::download(int32_t* cluster) {
    if (n == 0) return GSDR_OK;
    JCUDA(cudaEventRecord(ev_[4], stream));
    JCUDA(cudaMemcpyAsync(cluster, B_.cluster, sizeof(int32_t) * n, cudaMemcpyDeviceToHost,
                          stream));
    JCUDA(cudaEventRecord(ev_[5], stream));
    JCUDA(cudaStreamSynchronize(stream));
    float ms = 0;
    cudaEventElapsedTime(&ms, ev_[4], ev_[5]);
    stats.ms_d2h = ms;
    return GSDR_OK;
}

}  // namespace gsdr

using namespace gsdr;

struct gsdr_job {
    Job job;
};

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

int gsdr_job_create(const gsdr_reads* reads, const gsdr_opts* opts, gsdr_job** out) {
    if (!out) return fail(GSDR_EINVAL, "null output");
    *out = nullptr;
    gsdr_job* j = new (std::nothrow) gsdr_job();
    if (!j) return fail(GSDR_ENOMEM, "out of host memory");
    int rc = j->job.init(reads, opts);
    if (!rc) rc = j->job.upload(reads);
    if (rc) {
        delete j;
        return rc;
    }
    *out = j;
    return GSDR_OK;
}

int gsdr_job_run(gsdr_job* j, gsdr_stats* stats) {
    if (!j) return fail(GSDR_EINVAL, "null job");
    int rc = j->job.run();
    if (stats) *stats = j->job.stats;
    return rc;
}

int gsdr_job_run_limited(gsdr_job* j, int32_t max_passes, gsdr_stats* stats) {
    if (!j || max_passes < 1) return fail(GSDR_EINVAL, "gsdr_job_run_limited: bad argument");
    int rc = j->job.run(max_passes);
    if (stats) *stats = j->job.stats;
    return rc;
}

int gsdr_job_resume(gsdr_job* j, const int32_t* cluster, int32_t max_passes, gsdr_stats* stats) {
    if (!j || (!cluster && j->job.n > 0))
        return fail(GSDR_EINVAL, "gsdr_job_resume: null argument");
    const int n = j->job.n;
    // A state the greedy loop can reach: every read unclustered (-1) or joined
    // to a representative at or before it, and every representative before the
    // first unclustered read (representatives are taken in sorted order).
    int first_un = n, last_rep = -1;
    for (int i = 0; i < n; i++) {
        const int c = cluster[i];
        if (c == -1) {
            if (first_un == n) first_un = i;
            continue;
        }
        if (c < 0 || c > i || cluster[c] != c)
            return fail(GSDR_EINVAL, "gsdr_job_resume: not a clustering state (cluster[i] must "
                                     "be -1 or a representative at or before i)");
        if (c == i) last_rep = i;
    }
    if (last_rep > first_un)
        return fail(GSDR_EINVAL, "gsdr_job_resume: a representative after an unclustered read");
    int rc = j->job.run(max_passes > 0 ? max_passes : 0, cluster);
    if (stats) *stats = j->job.stats;
    return rc;
}

int gsdr_job_cluster(gsdr_job* j, int32_t* cluster) {
    if (!j || (!cluster && j->job.n > 0)) return fail(GSDR_EINVAL, "null argument");
    return j->job.download(cluster);
}

void gsdr_job_free(gsdr_job* j) { delete j; }

int gsdr_cluster(const gsdr_reads* reads, const gsdr_opts* opts, int32_t* cluster,
                 gsdr_stats* stats) {
    if (!reads || !opts || (!cluster && reads->n > 0))
        return fail(GSDR_EINVAL, "gsdr_cluster: null argument");
    const double t0 = now_ms();
    Job job;
    int rc = job.init(reads, opts);
    if (!rc) rc = job.upload(reads);
    if (!rc) rc = job.run();
    if (!rc) rc = job.download(cluster);
    job.stats.ms_total = now_ms() - t0;
    if (stats) *stats = job.stats;
    return rc;
}

// main (cuda-version/main.cu:3-36).
int gsdr_main(int argc, char** argv) {
    const double t0 = now_ms();
    gsdr_opts o;
    std::vector<char> in(4096), out(4096);
    // extension: "c <path>" also writes the cluster membership (.clstr text);
    // the other words go to checkOption unchanged
    std::string clstr;
    std::vector<char*> args;
    for (int i = 0; i < argc; i++) {
        const char* key = argv[i];
        while (i > 0 && i % 2 == 1 && *key == '-') key++;
        if (i > 0 && i % 2 == 1 && key[0] == 'c' && i + 1 < argc) {
            clstr = argv[i + 1];
            i++;
            continue;
        }
        args.push_back(argv[i]);
    }
    if (gsdr_check_option((int)args.size(), args.data(), &o, in.data(), out.data(),
                          (int64_t)in.size()) != GSDR_OK) {
        std::printf("Please check parameters.\n%s\n", gsdr_last_error());
        std::printf("cluster i inputFile o outputFile t threshold [w wordLength] [d 0|1] [p 0|1]"
                    " [v 0|1] [c clusterFile]\n");
        return 0;
    }
    o.verbose = 1;
    std::printf("input file:\t%s\noutput file:\t%s\nthreshold:\t%g\nword length:\t%d\ndrop filter\t%d\n",
                in.data(), out.data(), (double)o.threshold, o.word_length, o.drop);
    // readFile: the whole file into memory (an unreadable file reads as empty,
    // as the reference's ifstream does); parse, sort, clustering and output
    // formatting then run on the device (gsdr_cluster_fasta)
    std::vector<char> text;
    if (FILE* fp = std::fopen(in.data(), "rb")) {
        char chunk[1 << 16];
        size_t got;
        while ((got = std::fread(chunk, 1, sizeof(chunk), fp)) > 0)
            text.insert(text.end(), chunk, chunk + got);
        std::fclose(fp);
    }
    gsdr_result* res = nullptr;
    gsdr_stats st;
    int rc = gsdr_cluster_fasta(text.data(), (int64_t)text.size(), &o, &res, &st);
    if (rc) {
        std::printf("error: %s (%s)\n", gsdr_strerror(rc), gsdr_last_error());
        return 1;
    }
    const int32_t nr = gsdr_result_count(res);
    const int32_t* lens = gsdr_result_lengths(res);
    if (nr > 0)
        std::printf("longest:\t%d\nshortest:\t%d\nreads count:\t%d\n", lens[0], lens[nr - 1], nr);
    // saveFile (func.cu:1099-1111)
    const char* ob = nullptr;
    int64_t on = 0;
    gsdr_result_output(res, &ob, &on);
    FILE* fo = std::fopen(out.data(), "wb");
    bool ok = fo != nullptr;
    if (fo) {
        ok = std::fwrite(ob, 1, (size_t)on, fo) == (size_t)on;
        ok = std::fclose(fo) == 0 && ok;
    }
    int64_t written = 0;
    const int32_t* cl = gsdr_result_cluster(res);
    for (int32_t i = 0; i < nr; i++) written += cl[i] == i;
    if (ok && !clstr.empty()) {
        // the membership text needs the names: the host reader over the same bytes
        gsdr_fasta* f = nullptr;
        rc = gsdr_fasta_parse(text.data(), (int64_t)text.size(), &f);
        if (!rc) rc = gsdr_fasta_write_clusters(clstr.c_str(), f, cl, nullptr);
        if (f) gsdr_fasta_free(f);
        ok = rc == GSDR_OK;
    }
    gsdr_result_free(res);
    if (!ok) {
        std::printf("error: cannot write %s\n", out.data());
        return 1;
    }
    std::printf("cluster count:\t%lld\n", (long long)written);
    std::printf("time consuming:\t%.0fms\n", now_ms() - t0);
    return 0;
}

}  // extern "C"

// ---- testing: the alignment stage alone (include/gsdr_testing.h) ----------

namespace gsdr {

int Job::lcs_pairs(const int32_t* pat, const int32_t* txt, int n_pairs, int mapping, int greedy,
                   uint8_t* accept, double* ms) {
    if (n_pairs <= 0) return GSDR_OK;
    std::vector<int> seen(n, 0);
    std::vector<std::vector<Pair>> cls(kAlignClasses);
    std::vector<int32_t> gf(n);
    // gap-free lengths decide the class: prepare the reads first
    JCUDA(cudaSetDevice(opts.device));
    JCUDA(cudaMemsetAsync(R_.packed, 0, sizeof(uint32_t) * ((size_t)pack_off_[n] + 8), stream));
    launch_pack(R_, opts.threshold, opts.word_length, stream);
    launch_planes(R_, stream);
    JCUDA(cudaGetLastError());
    std::vector<int32_t> cut(n);
    JCUDA(cudaMemcpyAsync(gf.data(), R_.len_gf, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, stream));
    JCUDA(cudaMemcpyAsync(cut.data(), R_.cut_base, sizeof(int32_t) * n, cudaMemcpyDeviceToHost,
                          stream));
    JCUDA(cudaStreamSynchronize(stream));
    for (int k = 0; k < n_pairs; k++) {
        if (pat[k] < 0 || pat[k] >= n || txt[k] < 0 || txt[k] >= n || seen[pat[k]])
            return fail(GSDR_EINVAL, "lcs_pairs: bad or repeated pattern index");
        seen[pat[k]] = 1;
        int c = align_class_host((gf[pat[k]] + 31) >> 5);
        if (mapping == 2) {
            // the banded kernel where the band fits 32 words (as batched passes do)
            const int T = gf[txt[k]], q = gf[pat[k]], cb = cut[pat[k]];
            // (the serial-work limit of the passes is not applied: tests reach
            // every window class with any length)
            if (T > 0 && cb > 0 && q >= cb && T >= cb) {
                const int bw = band_words(T, q, cb);
                if (bw <= 32) c = kSysClasses + (bw <= 4 ? 0 : bw <= 8 ? 1 : bw <= 16 ? 2 : 3);
            }
        } else if (mapping == 3) {
            // the group-banded kernel where the band fits 128 words
            const int T = gf[txt[k]], q = gf[pat[k]], cb = cut[pat[k]];
            if (T > 0 && cb > 0 && q >= cb && T >= cb) {
                const int bw = band_words(T, q, cb);
                if (bw <= kGroupMaxWords) c = group_class(bw);
            }
        }
        cls[c].push_back(Pair{txt[k], pat[k]});
    }
    RoundState st{};
    for (int c = 0; c < kAlignClasses; c++) {
        if ((int)cls[c].size() > B_.seg_cap) return fail(GSDR_EINVAL, "lcs_pairs: too many pairs");
        st.n_pairs[c] = (int)cls[c].size();
        if (!cls[c].empty())
            JCUDA(cudaMemcpyAsync(B_.pairs + (size_t)c * B_.seg_cap, cls[c].data(),
                                  sizeof(Pair) * cls[c].size(), cudaMemcpyHostToDevice, stream));
    }
    st.pass = 1;
    st.n_tent = 1;
    st.R = 1;
    JCUDA(cudaMemcpyAsync(B_.st, &st, sizeof(st), cudaMemcpyHostToDevice, stream));
    JCUDA(cudaMemsetAsync(B_.st + 1, 0, 64 * sizeof(int), stream));
    JCUDA(cudaMemsetAsync(B_.cluster, 0xff, sizeof(int32_t) * n, stream));
    JCUDA(cudaMemsetAsync(B_.tidx, 0xff, sizeof(uint32_t) * n, stream));
    JCUDA(cudaEventRecord(ev_[2], stream));
    launch_align_stage(R_, B_, mapping >= 1, greedy != 0, stream);
    JCUDA(cudaGetLastError());
    JCUDA(cudaEventRecord(ev_[3], stream));
    JCUDA(cudaMemcpyAsync(h_state_, B_.st, sizeof(RoundState), cudaMemcpyDeviceToHost, stream));
    std::vector<int32_t> cl(n);
    JCUDA(cudaMemcpyAsync(cl.data(), B_.cluster, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, stream));
    JCUDA(cudaStreamSynchronize(stream));
    if (h_state_->error) return fail(GSDR_ETIMEOUT, "lcs_pairs: a device-side wait gave up");
    if (mapping >= 1) {
        const int na = h_state_->n_acc;
        if (na > B_.acc_cap) return fail(GSDR_ENOMEM, "lcs_pairs: accept list overflow");
        std::vector<Pair> acc(na);
        if (na)
            JCUDA(cudaMemcpy(acc.data(), B_.acc, sizeof(Pair) * na, cudaMemcpyDeviceToHost));
        for (const Pair& p : acc) cl[p.cand] = p.rep;
    }
    for (int k = 0; k < n_pairs; k++) accept[k] = cl[pat[k]] == txt[k] ? 1 : 0;
    float f = 0;
    cudaEventElapsedTime(&f, ev_[2], ev_[3]);
    if (ms) *ms = f;
    return GSDR_OK;
}

}  // namespace gsdr

extern "C" int gsdr_set_spin_limit(int32_t device, int32_t polls) {
    if (cudaSetDevice(device) != cudaSuccess) return fail(GSDR_EDEVICE, "no such CUDA device");
    if (set_spin_limit(polls)) return fail(GSDR_EDEVICE, "cannot set the spin limit");
    return GSDR_OK;
}

extern "C" int gsdr_lcs_decide(const char* bytes, int64_t n_bytes, const int64_t* off,
                               const int32_t* len, int32_t n_seq, const int32_t* pat,
                               const int32_t* txt, int32_t n_pairs, float t, int32_t mapping,
                               int32_t greedy, uint8_t* accept, double* ms) {
    if (!pat || !txt || (!accept && n_pairs > 0) || n_pairs < 0)
        return fail(GSDR_EINVAL, "gsdr_lcs_decide: null argument");
    gsdr_reads r{bytes, n_bytes, off, len, n_seq};
    gsdr_opts o;
    gsdr_default_opts(&o);
    o.threshold = t;
    o.drop = 1;
    o.batch = 1;
    Job job;
    int rc = job.init(&r, &o);
    if (!rc) rc = job.upload(&r);
    if (!rc) rc = job.lcs_pairs(pat, txt, n_pairs, mapping, greedy, accept, ms);
    return rc;
}
