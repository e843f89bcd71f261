/* gsdr.h -- C ABI of the GB300 greedy exact-identity clustering library.
 *
 * The reference program (JuZhenCS/gene-sequences-de-redundancy, cuda-version)
 * has no library interface: main() calls free functions in a fixed order
 * (cuda-version/main.cu:3-36).  Each entry point below replaces one of those
 * functions, with the same argument meaning, and returns a status code where
 * the reference printed a message and exited.  Plain pointers and sizes only.
 *
 *   gsdr_check_option   <- checkOption        cuda-version/func.cu:10-92
 *   gsdr_fasta_read     <- readFile           cuda-version/func.cu:94-117
 *   gsdr_cluster        <- copyData .. mergeWords, clustering / clusteringDrop
 *                          cuda-version/func.cu:119-653, 1001-1097
 *                          (the declarations in cuda-version/func.h:55-77)
 *   gsdr_fasta_write    <- saveFile           cuda-version/func.cu:1099-1111
 *   gsdr_main           <- main               cuda-version/main.cu:3-36
 *
 * A representative is the longest still-unclustered read; every later
 * unclustered read whose gap-free LCS with it reaches ceil(len * t) (after the
 * reference's base-composition prefilter, optional pigeon filter and k-mer
 * word filter) joins it.  Results are bit-identical to the reference.
 */
#ifndef GSDR_H
#define GSDR_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define GSDR_OK 0
#define GSDR_EINVAL 1       /* bad argument; the reference prints usage and exits (func.cu:4-8,43-84) */
#define GSDR_ENOMEM 2       /* host or device allocation failed */
#define GSDR_EDEVICE 3      /* CUDA error, no usable device, or missing CUDA code */
#define GSDR_ETIMEOUT 4     /* a bounded device-side wait gave up */
#define GSDR_EIO 5          /* file could not be written */
#define GSDR_EUNSUPPORTED 6 /* input outside what this build handles (message says which) */
#define GSDR_EBUSY 7        /* serving: queue full */
#define GSDR_ENOTFOUND 8    /* serving: unknown job id */

/* Options, as struct Option (cuda-version/func.h:9-16) plus execution knobs. */
typedef struct {
    float threshold;      /* t: 0.8 <= t < 1 (func.cu:43) */
    int32_t word_length;  /* k: 0 = derive from t as func.cu:49-58 does; else 4..12 */
    int32_t drop;         /* 0 = filters on, 1 = alignment only, 3 = derive from t (func.cu:67-72) */
    int32_t pigeon;       /* 0 or 1: the 4-mer position filter (func.cu:756-801) */
    int32_t batch;        /* tentative representatives per pass: 1 = one per round
                             (the reference's form); >1 = batched; 0 = automatic */
    int32_t device;       /* CUDA device ordinal */
    int32_t stage_timing; /* 1: time each stage with CUDA events (slower; for profiling) */
    int32_t verbose;      /* 1: print the reference's progress lines to stdout */
    int32_t word_filter;  /* batched word filter form: 0 automatic, 1 per-tentative k-mer
                             tables, 2 inverted k-mer index, 3 two-level k-mer count
                             bitmaps (k <= 7), 4 per-k-mer tentative masks (k <= 7,
                             reads of at most 1,023 k-mers; otherwise the automatic
                             form); the result is the same in every form */
    int32_t variant;      /* semantics: 0 = cuda-version (func.cu, the default);
                             1 = the top-level SYCL program (func.cpp): k from t by
                             func.cpp:36-45, w 4..8, no drop mode and no pigeon filter,
                             k-mers over the raw read skipping windows with a non-ACGT
                             byte (func.cpp:238-274), word cutoff in float without the
                             offset (func.cpp:339-373), accept iff LCS > ceil(len*t)
                             (func.cpp:671) */
    int32_t band_serial;  /* band tile of the lane-per-pair banded alignment kernel: the
                             largest serial work (text bases x window words) of a pair it
                             takes; 0 = automatic (16,384), -1 = none (those pairs go to
                             the other alignment kernels); the result is the same */
    int32_t group_words;  /* band tile of the group-banded alignment kernel: the widest
                             band window (32-bit words, 1..128) it takes; 0 = automatic
                             (128), -1 = none; the result is the same */
    int32_t align_blocks; /* block shape: resident CTAs per SM the alignment kernels are
                             launched with (1..8, capped by what fits; 0 = automatic: as
                             many as fit); the result is the same */
    int32_t filter_blocks; /* the same for the word-filter kernels */
    int32_t graph_steps;  /* staging depth: rounds (plain) or passes (batched) captured in
                             one CUDA graph, launched between two host checks of the done
                             flag (even, 2..64; 0 = automatic: 16 plain, 4 batched) */
} gsdr_opts;

/* Reads in length-sorted order (the order readFile leaves them in).  Read i is
 * bytes[offset[i] .. offset[i] + length[i]) -- verbatim sequence bytes, any
 * letters; bytes outside A/C/G/T/U (either case) are gaps (func.cu:139-179). */
typedef struct {
    const char* bytes;
    int64_t n_bytes;
    const int64_t* offset;
    const int32_t* length;
    int32_t n;
} gsdr_reads;

typedef struct {
    int64_t rounds;           /* representatives taken (one per round in the plain form) */
    int64_t passes;           /* device passes (batched: one per batch of tentatives) */
    int64_t pairs_prefilter;  /* (representative, candidate) pairs that reached the prefilter */
    int64_t pairs_word;       /* pairs that reached the word filter (word_index = 1: pairs
                                 that passed it, word_index = 3: pairs its bounds did not
                                 reject; those forms apply the word filter first) */
    int64_t pairs_aligned;    /* pairs that reached the alignment */
    int64_t pairs_accepted;
    double cells;             /* sum over aligned pairs of gap-free q x T (full-DP cells) */
    double filter_bytes;      /* input bytes of the filter stage: per launch, each remaining
                                 candidate's 28 bytes of composition, cutoffs and index and
                                 its (k-mer, count) list (word_index = 2: its k-mer bitmap);
                                 the plain form counts the list only where the filter
                                 reads it (composition bound passed), the batched forms
                                 once per launch (re-reads by other tentatives not counted) */
    double ms_h2d, ms_prep, ms_cluster, ms_d2h, ms_total;
    double ms_filter, ms_align; /* with stage_timing only */
    int32_t k, drop, pigeon, batch;
    int64_t kernel_launches;  /* kernels launched by the library during the call */
    int32_t word_index;       /* form of the batched word filter: 0 per-tentative k-mer
                                 tables, 1 per-pass inverted k-mer index (reads holding
                                 few of the 4^k k-mers), 2 k-mer count bitmaps with an
                                 exact sum for the pairs their bound leaves open, 3
                                 per-k-mer tentative masks (short reads in a sparse
                                 k-mer space) with the same exact sum */
    double filter_max_bytes;  /* with stage_timing only: input bytes of the filter launch
                                 that read the most, and its time (filter_max_ms) */
    double filter_max_ms;
    double cells_computed;    /* DP cells the alignment kernels actually stepped: per block
                                 of 32 text bases, the 32-bit pattern or band-window words
                                 a warp or lane held x 32 bits x 32 bases (early exits,
                                 bands and the greedy bound make it smaller than cells) */
    int32_t tuned;            /* 1: an automatic job (batch 0) took its knobs from the
                                 tuning cache written by gsdr_autotune */
} gsdr_stats;

/* Fill `o` with the reference defaults (t 0.95, derived k/drop, pigeon 0). */
void gsdr_default_opts(gsdr_opts* o);

/* Derive k and drop from t exactly as checkOption does and validate ranges.
 * Returns GSDR_OK or GSDR_EINVAL (with a message in *msg if msg != NULL). */
int gsdr_resolve_opts(gsdr_opts* o, const char** msg);

/* checkOption (cuda-version/func.cu:10-92): argv holds letter/value pairs
 * i o t w d p; only the first character of a key counts, and a leading '-'
 * is also accepted.  Extensions: b (batch), g (device), v (variant: 0 or 1;
 * with v 1 the keys d and p are refused, as func.cpp:6-32 refuses them).  Paths are copied into in_path/out_path (cap bytes each).
 * Returns GSDR_OK or GSDR_EINVAL (the reference's usage exit). */
int gsdr_check_option(int argc, char** argv, gsdr_opts* o, char* in_path, char* out_path,
                      int64_t cap);

/* readFile (cuda-version/func.cu:94-117).  Parses the FASTA file with the
 * reference's getline rules and sorts reads longest first with the same
 * std::sort call, so that ties come out in the same order.  An unreadable
 * file behaves like an empty one, as in the reference. */
typedef struct gsdr_fasta gsdr_fasta;
int gsdr_fasta_read(const char* path, gsdr_fasta** out);
/* Same, from a buffer already in memory (copied). */
int gsdr_fasta_parse(const char* data, int64_t n, gsdr_fasta** out);
int32_t gsdr_fasta_count(const gsdr_fasta* f);
/* View of the sorted reads (valid while f lives). */
int gsdr_fasta_view(const gsdr_fasta* f, gsdr_reads* view);
/* order[i] = file position of sorted read i (n entries, valid while f lives). */
const int32_t* gsdr_fasta_order(const gsdr_fasta* f);
/* Name line (verbatim, with its '>') of sorted read i. */
const char* gsdr_fasta_name(const gsdr_fasta* f, int32_t i, int64_t* len);
/* saveFile (cuda-version/func.cu:1099-1111): for each sorted read i with
 * cluster[i] == i write "name\n" and "sequence\n". */
int gsdr_fasta_write(const char* path, const gsdr_fasta* f, const int32_t* cluster,
                     int64_t* n_written);
/* The same bytes into a caller buffer; returns the size needed in *need. */
int gsdr_fasta_format(const gsdr_fasta* f, const int32_t* cluster, char* buf, int64_t cap,
                      int64_t* need);
void gsdr_fasta_free(gsdr_fasta* f);

/* Cluster membership (no counterpart in the reference, which keeps cluster[]
 * in memory only; the FASTA output is unaffected), CD-HIT-like text:
 *   >Cluster <k>                      clusters numbered in output-FASTA order
 *   <m>\t<length>nt, <name line>... *  the representative (m = 0)
 *   <m>\t<length>nt, <name line>...    each member, in sorted order
 * <length> is the raw sequence length in bytes, <name line> the header with
 * its '>'.  No identity is printed: the decision LCS >= cutoff does not compute
 * one.  GSDR_EINVAL unless cluster[] is a finished clustering (cluster[i] <= i
 * and cluster[cluster[i]] == cluster[i]). */
int gsdr_fasta_format_clusters(const gsdr_fasta* f, const int32_t* cluster, char* buf,
                               int64_t cap, int64_t* need);
int gsdr_fasta_write_clusters(const char* path, const gsdr_fasta* f, const int32_t* cluster,
                              int64_t* n_clusters);

/* The clustering path (cuda-version/func.cu:119-653 preparation and the loop
 * of func.cu:1001-1097).  cluster[i] receives the representative of sorted
 * read i (cluster[i] == i for representatives).  Host buffers in and out;
 * device memory is managed by the library.  `stats` may be NULL. */
int gsdr_cluster(const gsdr_reads* reads, const gsdr_opts* opts, int32_t* cluster,
                 gsdr_stats* stats);

/* readFile + clustering + saveFile on the device for a FASTA file already in
 * host memory (the whole reference program, cuda-version/main.cu:3-36, minus
 * the file I/O): the bytes are copied to the device once; record boundaries
 * (the getline rules of func.cu:94-117) are found there; only the data
 * lengths return to the host for the same std::sort call; the representative
 * records are formatted on the device and only they return.  The result holds
 * the output bytes (saveFile's), the cluster array in sorted order, the sort
 * permutation and the sorted lengths. */
typedef struct gsdr_result gsdr_result;
int gsdr_cluster_fasta(const char* fasta, int64_t n, const gsdr_opts* opts, gsdr_result** out,
                       gsdr_stats* stats);
int gsdr_result_output(const gsdr_result* r, const char** data, int64_t* n);
int32_t gsdr_result_count(const gsdr_result* r);
const int32_t* gsdr_result_cluster(const gsdr_result* r);  /* sorted order */
const int32_t* gsdr_result_order(const gsdr_result* r);    /* sorted -> file position */
const int32_t* gsdr_result_lengths(const gsdr_result* r);  /* sorted order */
void gsdr_result_free(gsdr_result* r);

/* The same path in three steps, for callers that keep a job's data on the
 * device between calls (and for timing the device part alone):
 *   gsdr_job_create  copyData (func.cu:119-137): device allocation + H2D copy
 *   gsdr_job_run     preparation kernels and the round loop (func.cu:139-653,
 *                    1001-1097) on the device-resident reads
 *   gsdr_job_cluster the cluster array back to the host
 * gsdr_job_run may be called again on the same job; it recomputes from the
 * uploaded reads. */
typedef struct gsdr_job gsdr_job;
int gsdr_job_create(const gsdr_reads* reads, const gsdr_opts* opts, gsdr_job** out);
int gsdr_job_run(gsdr_job* job, gsdr_stats* stats);
int gsdr_job_cluster(gsdr_job* job, int32_t* cluster);
void gsdr_job_free(gsdr_job* job);

/* Checkpoint / resume.  The whole state the reference's round loop carries
 * from one round to the next is cluster[] (func.cu:1001-1066): the next
 * representative is the smallest unclustered read.  So a checkpoint is the
 * cluster array of an unfinished run -- gsdr_job_cluster after a run stopped
 * early (gsdr_job_run_limited, include/gsdr_testing.h), -1 for unclustered
 * reads -- which the caller may save anywhere.  gsdr_job_resume continues
 * that clustering on a job over the same reads and options (the same or
 * another job, in this or another process) for up to max_passes more passes
 * or rounds (<= 0: to the end); the finished result equals an uninterrupted
 * run's.  GSDR_EINVAL unless every cluster[i] is -1 or a representative
 * c <= i with cluster[c] == c, and no representative comes after an
 * unclustered read. */
int gsdr_job_resume(gsdr_job* job, const int32_t* cluster, int32_t max_passes,
                    gsdr_stats* stats);

/* The alignment-stage decision for callers that cannot allocate device memory.
 * No counterpart in the reference.  Some callers own every device allocation:
 * code inside a framework's memory pool or a plug-in that must not grow the
 * process's device footprint.  This entry point calls no cudaMalloc, cudaFree
 * or allocating library routine.  The caller passes device buffers for the
 * inputs and the output.  The work space lives in one fixed array of the
 * library of about 1.3 MB, which every GPU that loads the library holds until
 * the process exits.  That bounds the work per call: at most
 * GSDR_NOALLOC_MAX_PAIRS pairs over at most GSDR_NOALLOC_MAX_SEQS sequences of
 * at most 32768 gap-free bases; larger calls return GSDR_EINVAL.
 *
 * Inputs (device memory): packed 2-bit sequences (16 bases per uint32, first
 * base in bits 31:30, sequence i from word d_pack_off[i], readable one word
 * past its last base word), the raw length (for the cutoff ceil(len * t)) and
 * gap-free length of each sequence, and n_pairs (pattern, text) index pairs.
 * A pattern index may appear in at most one pair.  Output: d_accept[k] = 1 iff
 * LCS(pattern, text) >= ceil(raw length of the pattern * t).  An index outside
 * [0, n_seq), a pattern index in two pairs or a pattern above 32768 gap-free
 * bases makes the call return GSDR_EINVAL (no out-of-range access is made).
 *
 * The first call on a device, made with that device current, looks up the
 * array's device address and keeps it for the life of the process (a
 * cudaDeviceReset of that device is not followed).  Every call reuses the same
 * array and clears what it needs at the start, so calls that overlap on the
 * GPU (other streams, other host threads) race and give undefined results:
 * the caller serialises them.  Each call reads its status back and waits for
 * `stream` (a cudaStream_t, or NULL): it returns with that stream idle, and it
 * must not be called while the stream is being captured.  A CUDA error still
 * pending from the caller's earlier work is reported (GSDR_EDEVICE) and left
 * in place, before anything is launched. */
#define GSDR_NOALLOC_MAX_PAIRS 16384
#define GSDR_NOALLOC_MAX_SEQS 65536
int gsdr_lcs_decide_noalloc(const uint32_t* d_packed, const int64_t* d_pack_off,
                            const int32_t* d_len_raw, const int32_t* d_len_gf, int32_t n_seq,
                            const int32_t* d_pat, const int32_t* d_txt, int32_t n_pairs,
                            float t, uint8_t* d_accept, void* stream);

/* Autotuner: no counterpart in the reference, which has no execution knobs.
 * Times settings of the knobs of gsdr_opts that change only the time -- R_max
 * (batch), the batched word filter's form, the two band tiles, the block shape
 * (align_blocks, filter_blocks) and the staging depth (graph_steps) -- by
 * running the job on its first `reps` representatives (<= 0: min(8192,
 * reads/20), at least 256), `runs` timed runs each (<= 0: 2), in four stages
 * of coordinate descent; *best receives the fastest setting (the other fields
 * as in *opts).  The result is stored in the tuning cache, one line per (GPU
 * model and SM count, workload bucket: word length, drop mode, variant, pigeon
 * filter, threshold, log2 of the read count and of the mean read length):
 * at cache_path, or with cache_path NULL at $GSDR_TUNE_CACHE, else
 * $XDG_CACHE_HOME/gsdr/tune.tsv, else $HOME/.cache/gsdr/tune.tsv; "" stores
 * nothing.  Every later job with batch 0 in a bucket the cache holds (on the
 * same GPU model) takes the stored knobs for each knob it leaves at 0, the
 * `cluster` executable included (gsdr_stats.tuned = 1).  `report` (cap bytes,
 * may be NULL) receives a JSON text of every trial; *need its size. */
int gsdr_autotune(const gsdr_reads* reads, const gsdr_opts* opts, int32_t reps, int32_t runs,
                  const char* cache_path, gsdr_opts* best, char* report, int64_t cap,
                  int64_t* need);

/* main (cuda-version/main.cu:3-36): the `cluster` command line.  Returns the
 * process exit status (0 also for the usage exit, as in the reference). */
int gsdr_main(int argc, char** argv);

const char* gsdr_strerror(int status);
/* Text of the last error on this thread (more detail than gsdr_strerror). */
const char* gsdr_last_error(void);

/* ---- Serving: continuous batching of independent clustering jobs ----------
 * No counterpart in the reference.  Jobs are admitted by device-memory
 * footprint, run concurrently on separate CUDA streams, and each job's result
 * equals what gsdr_cluster returns for it alone.  When a slot frees, the
 * smallest queued job starts (a job that has waited 1 s or more goes first);
 * a job with a threshold checkOption refuses finishes with GSDR_EINVAL at
 * submission. */
typedef struct gsdr_server gsdr_server;
typedef struct {
    int32_t device;
    int32_t max_inflight;     /* concurrent jobs on the device (streams) */
    int64_t mem_budget;       /* device bytes for job data; 0 = 80% of free memory */
    int32_t batch;            /* as gsdr_opts.batch */
    int64_t express_bytes;    /* one slot beyond max_inflight takes only jobs of at most
                                 this many FASTA bytes; 0 = 4 MiB, -1 = no such slot */
} gsdr_server_opts;
int gsdr_server_create(const gsdr_server_opts* so, gsdr_server** out);
/* Submit a job: the FASTA bytes are copied; t as in gsdr_opts.  Returns the
 * job id in *job. */
int gsdr_server_submit(gsdr_server* s, const char* fasta, int64_t n, float threshold,
                       int64_t* job);
/* Wait up to timeout_ms (-1 = forever) for a finished job; returns its id,
 * status and timing.  GSDR_ETIMEOUT when none finished in time. */
int gsdr_server_wait(gsdr_server* s, int64_t timeout_ms, int64_t* job, int32_t* job_status,
                     double* latency_ms);
/* Result of a finished job: representative FASTA bytes (caller buffer; *need
 * receives the size) and the cluster array in sorted order (may be NULL). */
int gsdr_server_result(gsdr_server* s, int64_t job, char* buf, int64_t cap, int64_t* need,
                       int32_t* cluster, int32_t* n_reads);
/* Timing of a finished job: submission to the start of its run on a worker
 * (parse, sort, admission wait) and the run itself (device work and output
 * formatting), host wall clock.  The sum of run_ms over jobs divided by the
 * stream's wall time is the number of jobs running at once on average. */
int gsdr_server_times(gsdr_server* s, int64_t job, double* queued_ms, double* run_ms);
int gsdr_server_release(gsdr_server* s, int64_t job);
void gsdr_server_destroy(gsdr_server* s);

#ifdef __cplusplus
}
#endif
#endif
