// job.h -- one clustering job on one device: its device buffers, stream and
// round-loop graph.  gsdr_cluster, the job entry points and the serving loop
// all drive this object.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <functional>
#include <vector>

#include "gsdr.h"
#include "gsdr_device.cuh"
#include "plan_chunks.h"

namespace gsdr {

class Job {
public:
    ~Job();
    // Validates options and sizes, allocates device memory, creates the stream.
    // preset: the reads' layout, computed by the caller for the resolved word
    // length and drop mode (plan_chunks.h); init takes its arrays.
    int init(const gsdr_reads* reads, const gsdr_opts* opts, cudaStream_t stream = nullptr,
             PlanPreset* preset = nullptr);
    // Host -> device copy of the reads.  With dev_bytes, the job reads the
    // sequence bytes from that device buffer in place instead of reads->bytes:
    // its base 16-byte aligned, readable 16 bytes past reads->n_bytes, and
    // allocated and unchanged until the job's last kernel has run.
    int upload(const gsdr_reads* reads, const void* dev_bytes = nullptr);
    // Device views for kernels that follow the clustering (output formatting).
    const DevReads& device_reads() const { return R_; }
    const int32_t* device_cluster() const { return B_.cluster; }
    // Preparation kernels + the round loop; the cluster array stays on device.
    // pass_limit > 0 stops after that many passes or rounds (timing only: the
    // clustering is then unfinished).
    // resume (host, n entries): continue the clustering a checkpoint holds
    // (-1 = unclustered, else the read's representative) instead of starting it
    int run(int pass_limit = 0, const int32_t* resume = nullptr);
    // Device -> host copy of the cluster array (synchronous).
    int download(int32_t* cluster);
    // Testing: decisions of the alignment stage on given (pattern, text) pairs
    // (read indices); the job must have been initialised with drop = 1.
    int lcs_pairs(const int32_t* pat, const int32_t* txt, int n_pairs, int mapping, int greedy,
                  uint8_t* accept, double* ms);
    // Device bytes this job needs for its inputs (admission by footprint).
    static int64_t footprint(const gsdr_reads* reads, const gsdr_opts* opts);

    gsdr_opts opts{};
    gsdr_stats stats{};
    int n = 0;
    cudaStream_t stream = nullptr;
    // automatic jobs (batch 0) take the tuning cache's knobs for their
    // workload bucket (autotune.cu); the autotuner's own trials do not
    bool use_tune_cache = true;

private:
    int plan_and_alloc();
    int capture_graph();
    int loop_graph();
    int loop_timed();
    void launch_step(int parity, long long* count, cudaEvent_t* ev4);

    bool own_stream_ = false;
    bool batched_ = false;
    bool trace_ = false;  // GSDR_TRACE=1: per-step stage times on stderr (timed mode)
    int r_max_ = 1;
    int64_t n_bytes_ = 0;
    std::vector<int64_t> pack_off_, kmer_off_;
    std::vector<uint16_t> refoff16_;  // pigeon filter: padded-layout offsets (low 16 bits)
    void* dmem_ = nullptr;
    size_t dbytes_ = 0;
    int32_t* h_done_ = nullptr;
    RoundState* h_state_ = nullptr;
    cudaEvent_t ev_[6] = {};
    cudaGraph_t graph_ = nullptr;
    cudaGraphExec_t gexec_ = nullptr;
    long long graph_launches_per_ = 0;
    DevReads R_{};
    RoundBuffers B_{};
};

// devparse.cu: gsdr_cluster_fasta's path (device parse, host sort, clustering,
// device formatting) on its own stream.  admit (may be null) is called with
// the job's device footprint once the reads are known and before the job's
// memory is taken; a non-zero return ends the call with that status (the
// serving loop blocks there until the job fits its memory budget).
int cluster_fasta(const char* fasta, int64_t n, const gsdr_opts* opts, gsdr_result* res,
                  gsdr_stats* stats, const std::function<int(int64_t)>* admit = nullptr);
// An empty result for cluster_fasta (nullptr without host memory); released
// with gsdr_result_free.
gsdr_result* new_result();
// Device bytes gsdr_cluster_fasta takes beside the job's own for a file of n
// bytes with at most `records` records and `newlines` newlines (the file
// twice, the line and record arrays, the output records): an upper bound.
int64_t cluster_fasta_parse_bytes(int64_t n, int64_t records, int64_t newlines);

// autotune.cu: the tuning cache's knobs for this workload's bucket on this
// GPU, applied to every knob `o` leaves automatic (only when o.batch == 0);
// true when the cache held the bucket.
bool apply_tuned(const gsdr_reads* reads, gsdr_opts& o);

}  // namespace gsdr
