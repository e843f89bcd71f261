// autotune.cu -- empirical choice of the execution knobs (gsdr_autotune in
// include/gsdr.h) and the tuning cache the library reads for automatic jobs.
//
// No counterpart in the reference, which has no execution knobs.  Every knob
// changes only the time: R_max (tentative representatives per pass), the
// batched word filter's form, the two band tiles, the block shape (CTAs per
// SM of the alignment and filter kernels) and the staging depth (passes per
// CUDA-graph launch).  Each candidate setting runs the job itself on the
// device-resident reads for its first representatives only (Job::run with a
// pass limit): the early passes, where every read is still a candidate, cost
// the most, and a sample of the reads would not show their cost.  Settings
// are compared by device time per representative.  The search is coordinate
// descent in four stages (R_max x form, band tiles, block shape, staging
// depth), each stage starting from the best setting so far.
//
// The result is kept in a text cache, one line per (GPU model, SM count,
// workload bucket): a later job with batch = 0 whose bucket is in the cache
// takes the tuned values for every knob it leaves automatic.  The bucket is
// word length, drop mode, variant, pigeon filter, threshold (percent), and
// log2 of the read count and of the mean read length, rounded.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "gsdr.h"
#include "gsdr_host.h"
#include "job.h"

namespace gsdr {

namespace {

std::mutex g_cache_mu;

std::string default_cache_path() {
    if (const char* p = std::getenv("GSDR_TUNE_CACHE")) return p;
    if (const char* x = std::getenv("XDG_CACHE_HOME"); x && *x)
        return std::string(x) + "/gsdr/tune.tsv";
    if (const char* h = std::getenv("HOME"); h && *h) return std::string(h) + "/.cache/gsdr/tune.tsv";
    return "";
}

// "<model>/<SMs>sm" of a device (looked up once per device).
std::string gpu_key(int device) {
    static std::mutex mu;
    static std::vector<std::string> known;
    std::lock_guard<std::mutex> lock(mu);
    if (device < 0 || device >= 64) return "";
    if ((int)known.size() <= device) known.resize(device + 1);
    if (known[device].empty()) {
        cudaDeviceProp p{};
        if (cudaGetDeviceProperties(&p, device) != cudaSuccess) return "";
        known[device] = std::string(p.name) + "/" + std::to_string(p.multiProcessorCount) + "sm";
    }
    return known[device];
}

int log2_round(double x) { return x > 1 ? (int)std::lround(std::log2(x)) : 0; }

// The knobs a cache line sets, in file order.
struct Knobs {
    int batch = 0, word_filter = 0, group_words = 0, band_serial = 0, align_blocks = 0,
        filter_blocks = 0, graph_steps = 0;
};

Knobs knobs_of(const gsdr_opts& o) {
    return Knobs{o.batch, o.word_filter, o.group_words, o.band_serial, o.align_blocks,
                 o.filter_blocks, o.graph_steps};
}

bool read_line(const std::string& line, std::string& gpu, std::string& bucket, Knobs& k) {
    if (line.empty() || line[0] == '#') return false;
    std::vector<std::string> f;
    std::stringstream ss(line);
    std::string x;
    while (std::getline(ss, x, '\t')) f.push_back(x);
    if (f.size() < 9) return false;
    gpu = f[0];
    bucket = f[1];
    k.batch = std::atoi(f[2].c_str());
    k.word_filter = std::atoi(f[3].c_str());
    k.group_words = std::atoi(f[4].c_str());
    k.band_serial = std::atoi(f[5].c_str());
    k.align_blocks = std::atoi(f[6].c_str());
    k.filter_blocks = std::atoi(f[7].c_str());
    k.graph_steps = std::atoi(f[8].c_str());
    return true;
}

}  // namespace

std::string tune_bucket(const gsdr_reads* reads, const gsdr_opts& o) {
    const double mean = reads->n > 0 ? (double)reads->n_bytes / reads->n : 0;
    char b[160];
    std::snprintf(b, sizeof(b), "k%d d%d v%d p%d t%d n2^%d len2^%d", o.word_length, o.drop,
                  o.variant, o.pigeon, (int)std::lround(o.threshold * 100), log2_round(reads->n),
                  log2_round(mean));
    return b;
}

// The tuned knobs of this workload's bucket on this GPU, for every knob `o`
// leaves automatic (0).  Returns true when the cache had the bucket.
bool apply_tuned(const gsdr_reads* reads, gsdr_opts& o) {
    if (o.batch != 0) return false;
    const std::string path = default_cache_path();
    if (path.empty()) return false;
    const std::string gpu = gpu_key(o.device), bucket = tune_bucket(reads, o);
    std::lock_guard<std::mutex> lock(g_cache_mu);
    std::ifstream in(path);
    if (!in) return false;
    std::string line, g, b;
    Knobs k;
    bool found = false;
    while (std::getline(in, line)) {
        Knobs t;
        if (read_line(line, g, b, t) && g == gpu && b == bucket) {
            k = t;
            found = true;
        }
    }
    if (!found) return false;
    o.batch = k.batch;
    if (!o.word_filter) o.word_filter = k.word_filter;
    if (!o.group_words) o.group_words = k.group_words;
    if (!o.band_serial) o.band_serial = k.band_serial;
    if (!o.align_blocks) o.align_blocks = k.align_blocks;
    if (!o.filter_blocks) o.filter_blocks = k.filter_blocks;
    if (!o.graph_steps) o.graph_steps = k.graph_steps;
    return true;
}

namespace {

int store_tuned(const std::string& path, const std::string& gpu, const std::string& bucket,
                const gsdr_opts& best, double us_per_rep) {
    std::lock_guard<std::mutex> lock(g_cache_mu);
    std::vector<std::string> keep;
    {
        std::ifstream in(path);
        std::string line, g, b;
        Knobs t;
        while (std::getline(in, line)) {
            if (read_line(line, g, b, t) && g == gpu && b == bucket) continue;
            if (!line.empty()) keep.push_back(line);
        }
    }
    if (keep.empty())
        keep.push_back("# gsdr tuning cache: gpu, bucket, batch, word_filter, group_words, "
                       "band_serial, align_blocks, filter_blocks, graph_steps, us per "
                       "representative");
    char row[512];
    const Knobs k = knobs_of(best);
    std::snprintf(row, sizeof(row), "%s\t%s\t%d\t%d\t%d\t%d\t%d\t%d\t%d\t%.3f", gpu.c_str(),
                  bucket.c_str(), k.batch, k.word_filter, k.group_words, k.band_serial,
                  k.align_blocks, k.filter_blocks, k.graph_steps, us_per_rep);
    keep.push_back(row);
    // the directory of the default path may not exist yet
    const size_t slash = path.rfind('/');
    if (slash != std::string::npos && slash > 0) {
        std::error_code ec;
        std::filesystem::create_directories(path.substr(0, slash), ec);
    }
    const std::string tmp = path + ".tmp";
    {
        std::ofstream out(tmp, std::ios::trunc);
        if (!out) return fail(GSDR_EIO, "autotune: cannot write the tuning cache");
        for (auto& l : keep) out << l << "\n";
        if (!out) return fail(GSDR_EIO, "autotune: short write on the tuning cache");
    }
    if (std::rename(tmp.c_str(), path.c_str()) != 0)
        return fail(GSDR_EIO, "autotune: cannot replace the tuning cache");
    return GSDR_OK;
}

struct Trial {
    gsdr_opts o{};
    std::string stage;
    double ms = 0;      // median device time of the limited run
    double us_per_rep = 0;
    int64_t reps = 0;
    int passes = 0;
    int word_index = -1;
    bool ok = false;
    std::string error;
};

// Passes of a run whose R grows from 1 to r_max until about `reps`
// representatives are taken (adaptive R doubles per pass).
int passes_for(int r_max, int reps) {
    int ramp = 1;
    while ((1 << (ramp - 1)) < r_max) ramp++;
    return ramp + (reps + r_max - 1) / r_max;
}

void run_trial(const gsdr_reads* reads, Trial& t, int reps, int runs) {
    Job job;
    job.use_tune_cache = false;
    int rc = job.init(reads, &t.o);
    if (!rc) rc = job.upload(reads);
    const int r = job.stats.batch > 1 ? job.stats.batch : 1;
    t.passes = r > 1 ? passes_for(r, reps) : reps;
    if (!rc) rc = job.run(t.passes);  // warm-up: graph capture, first-touch
    std::vector<double> ms;
    for (int i = 0; !rc && i < runs; i++) {
        rc = job.run(t.passes);
        if (!rc) ms.push_back(job.stats.ms_prep + job.stats.ms_cluster);
    }
    if (rc) {
        t.error = gsdr_last_error();
        return;
    }
    std::sort(ms.begin(), ms.end());
    t.ms = ms[ms.size() / 2];
    t.reps = job.stats.rounds;
    t.word_index = job.stats.word_index;
    t.us_per_rep = 1e3 * t.ms / (double)(t.reps > 0 ? t.reps : 1);
    t.ok = true;
}

std::string json_of(const Trial& t) {
    char b[512];
    if (!t.ok) {
        std::string e;
        for (char c : t.error) e.push_back(c == '"' || c == '\\' ? '\'' : c);
        std::snprintf(b, sizeof(b),
                      "{\"stage\": \"%s\", \"batch\": %d, \"word_filter\": %d, \"error\": \"%s\"}",
                      t.stage.c_str(), t.o.batch, t.o.word_filter, e.c_str());
        return b;
    }
    std::snprintf(b, sizeof(b),
                  "{\"stage\": \"%s\", \"batch\": %d, \"word_filter\": %d, \"group_words\": %d, "
                  "\"band_serial\": %d, \"align_blocks\": %d, \"filter_blocks\": %d, "
                  "\"graph_steps\": %d, \"word_index\": %d, \"passes\": %d, "
                  "\"representatives\": %lld, \"ms\": %.4f, \"us_per_rep\": %.4f}",
                  t.stage.c_str(), t.o.batch, t.o.word_filter, t.o.group_words, t.o.band_serial,
                  t.o.align_blocks, t.o.filter_blocks, t.o.graph_steps, t.word_index, t.passes,
                  (long long)t.reps, t.ms, t.us_per_rep);
    return b;
}

}  // namespace

int autotune(const gsdr_reads* reads, const gsdr_opts* base_in, int reps, int runs,
             const char* cache_path, gsdr_opts* best_out, std::string* report) {
    gsdr_opts base = *base_in;
    int rc = gsdr_resolve_opts(&base, nullptr);
    if (rc) return rc;
    if (!reads || reads->n <= 0) return fail(GSDR_EINVAL, "autotune: no reads");
    if (runs <= 0) runs = 2;
    if (reps <= 0) reps = std::max(256, std::min(8192, reads->n / 20));
    const bool drop = base.drop == 1;
    // the mask form takes reads of at most kMaskMaxEntries k-mer entries: for
    // longer reads its trials would repeat the automatic form
    int64_t longest = 0;
    for (int i = 0; i < reads->n; i++) longest = std::max<int64_t>(longest, reads->length[i]);
    const bool masks_ok = base.word_length <= kMaxBits2K &&
                          longest - base.word_length + 1 <= kMaskMaxEntries;
    std::vector<Trial> trials;
    auto best_of = [&]() -> const Trial* {
        const Trial* b = nullptr;
        for (auto& t : trials)
            if (t.ok && (!b || t.us_per_rep < b->us_per_rep)) b = &t;
        return b;
    };
    auto run = [&](gsdr_opts o, const char* stage) {
        Trial t;
        t.o = o;
        t.stage = stage;
        run_trial(reads, t, reps, runs);
        // a form the job could not take (bitmaps above word length 7, masks
        // for reads above 255 k-mers) is not a setting
        if (t.ok && o.word_filter == 3 && t.word_index != 2) return;
        if (t.ok && o.word_filter == 4 && t.word_index != 3) return;
        trials.push_back(t);
    };
    // stage 1: R_max x word-filter form (the form only matters with the filters on)
    {
        gsdr_opts o = base;
        o.batch = 0;
        o.word_filter = 0;
        run(o, "R x form");
        const int rs[] = {64, 256, 1024};
        for (int form = drop ? 0 : 1; form <= (drop ? 0 : masks_ok ? 4 : 3); form++)
            for (int r : rs) {
                o.batch = r;
                o.word_filter = form;
                run(o, "R x form");
            }
    }
    const Trial* b = best_of();
    if (!b) return fail(GSDR_EDEVICE, "autotune: no setting ran");
    // stage 2: band tiles with the best of stage 1
    {
        const gsdr_opts at = b->o;
        const int tiles[][2] = {{-1, 0}, {32, 0}, {64, 0}, {0, -1}, {0, 4096}, {0, 65536}};
        for (auto& tl : tiles) {
            gsdr_opts o = at;
            o.group_words = tl[0];
            o.band_serial = tl[1];
            run(o, "band tiles");
        }
    }
    // stage 3: block shape (CTAs per SM of the alignment and the filter kernels)
    {
        const gsdr_opts at = best_of()->o;
        const int shapes[][2] = {{1, 0}, {2, 0}, {0, 2}, {0, 4}};
        for (auto& sh : shapes) {
            gsdr_opts o = at;
            o.align_blocks = sh[0];
            o.filter_blocks = sh[1];
            run(o, "block shape");
        }
    }
    // stage 4: staging depth (passes or rounds per graph launch)
    {
        const gsdr_opts at = best_of()->o;
        for (int g : {2, 8, 16}) {
            gsdr_opts o = at;
            o.graph_steps = g;
            run(o, "staging depth");
        }
    }
    b = best_of();
    const gsdr_opts best = b->o;  // batch 0: the automatic R_max won
    if (best_out) *best_out = best;
    if (report) {
        std::string r = "{\"reps\": " + std::to_string(reps) + ", \"best\": " + json_of(*b) +
                        ", \"trials\": [";
        for (size_t i = 0; i < trials.size(); i++) r += (i ? ", " : "") + json_of(trials[i]);
        r += "], \"bucket\": \"" + tune_bucket(reads, base) + "\", \"gpu\": \"" +
             gpu_key(base.device) + "\"";
        std::string path = cache_path ? cache_path : default_cache_path();
        r += ", \"cache\": \"" + path + "\"}";
        *report = r;
    }
    const std::string path = cache_path ? std::string(cache_path) : default_cache_path();
    if (!path.empty()) {
        rc = store_tuned(path, gpu_key(base.device), tune_bucket(reads, base), best,
                         b->us_per_rep);
        if (rc) return rc;
    }
    return GSDR_OK;
}

}  // namespace gsdr

using namespace gsdr;

extern "C" int gsdr_autotune(const gsdr_reads* reads, const gsdr_opts* opts, int32_t reps,
                             int32_t runs, const char* cache_path, gsdr_opts* best, char* report,
                             int64_t cap, int64_t* need) {
    if (!reads || !opts) return fail(GSDR_EINVAL, "gsdr_autotune: null argument");
    std::string rep;
    int rc = autotune(reads, opts, reps, runs, cache_path, best, &rep);
    if (rc) return rc;
    if (need) *need = (int64_t)rep.size() + 1;
    if (report && cap > 0) {
        const size_t n = std::min((size_t)cap - 1, rep.size());
        std::memcpy(report, rep.data(), n);
        report[n] = 0;
    }
    return GSDR_OK;
}
