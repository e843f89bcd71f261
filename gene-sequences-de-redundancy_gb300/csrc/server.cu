// server.cu -- serving: continuous batching of independent clustering jobs on
// one GPU (gsdr_server_* in include/gsdr.h; no counterpart in the reference).
//
// Jobs arrive as FASTA bytes with their own threshold.  Each job runs the
// gsdr_cluster_fasta path on a worker thread and its own CUDA stream: the
// file goes to the device once, records are found there, the lengths come
// back for the reference's std::sort, the job clusters the device-resident
// reads and the representative records are formatted on the device.  So jobs
// overlap on the device, the host work of one job (its sort) overlaps the
// device work of the others, and each result is exactly what
// gsdr_cluster_fasta returns for that job alone.
//
// Admission by device footprint, in two steps against the memory budget:
//   1. the scheduler thread admits a job to a free slot (max_inflight) when
//      an upper bound of its parse buffers (from its byte, record and newline
//      counts, taken at submission) fits the remaining budget;
//   2. once the worker knows the reads, the job's exact clustering footprint
//      must fit too; the worker waits for it while the job's parse buffers
//      are held.
// A job that does not fit waits until no other job is clustering and then
// runs alone, so every job is served.  Device memory comes from the library's
// stream-ordered pool (devmem.h): a finished job's release waits for nothing
// but its own stream.
//
// Order: when a slot is free the scheduler starts the smallest queued job (by
// bytes, the measure of its parse and filter work), unless the job that has
// waited longest has waited kAgeMs or more: then that one.  Short jobs no
// longer queue behind long ones, and no job waits behind an endless run of
// smaller ones.  A job whose threshold checkOption refuses is finished at
// submission.  One slot beyond max_inflight, the express slot, takes only
// jobs of at most express_bytes (4 MiB by default), so a short job need not
// wait while every regular slot holds a long one.  The order changes no result: the jobs are
// independent.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "gsdr.h"
#include "gsdr_host.h"
#include "job.h"

namespace gsdr {

struct ServerJob {
    int64_t id = 0;
    std::vector<char> fasta;
    int64_t records = 0, newlines = 0;  // upper bounds, counted at submission
    float threshold = 0.95f;
    double t_submit = 0, t_start = 0, t_done = 0;
    int status = GSDR_OK;
    std::string error;
    std::vector<int32_t> cluster;
    std::vector<char> out;
    int64_t parse_bytes = 0;  // step-1 reservation
    int64_t job_bytes = 0;    // step-2 reservation
    bool clustering = false;
    bool express = false;     // runs in the express slot
};

}  // namespace gsdr

using namespace gsdr;

struct gsdr_server {
    gsdr_server_opts so{};
    std::mutex mu;
    std::condition_variable cv_sched;  // queue changed or resources freed
    std::condition_variable cv_done;   // a job finished
    std::deque<std::shared_ptr<ServerJob>> queue;
    std::map<int64_t, std::shared_ptr<ServerJob>> jobs;
    std::deque<int64_t> finished;      // not yet returned by gsdr_server_wait
    std::deque<std::shared_ptr<ServerJob>> ready;  // admitted, waiting for a worker
    std::condition_variable cv_work;
    std::vector<std::thread> workers;  // max_inflight threads
    std::thread scheduler;
    bool workers_stop = false;
    int inflight = 0;
    int express = 0;                   // jobs in the express slot (0 or 1)
    int clustering = 0;                // jobs past step 2
    int64_t mem_used = 0;
    int64_t next_id = 1;
    bool stopping = false;
};

namespace {

void finish(gsdr_server* s, const std::shared_ptr<ServerJob>& j, int rc) {
    j->status = rc;
    j->t_done = now_ms();
    s->finished.push_back(j->id);
    s->cv_done.notify_all();
}

void run_job(gsdr_server* s, std::shared_ptr<ServerJob> j) {
    j->t_start = now_ms();
    gsdr_opts o;
    gsdr_default_opts(&o);
    o.threshold = j->threshold;
    o.device = s->so.device;
    o.batch = s->so.batch;
    // step 2 of the admission: the job's own footprint, once its reads are known
    const std::function<int(int64_t)> admit = [s, j](int64_t need) -> int {
        std::unique_lock<std::mutex> lock(s->mu);
        s->cv_sched.wait(lock, [&] {
            return s->stopping || s->mem_used + need <= s->so.mem_budget || s->clustering == 0;
        });
        if (s->stopping) return fail(GSDR_EBUSY, "server stopped");
        s->mem_used += need;
        j->job_bytes = need;
        j->clustering = true;
        s->clustering++;
        return GSDR_OK;
    };
    int rc = GSDR_OK;
    std::unique_ptr<gsdr_result, void (*)(gsdr_result*)> r(new_result(), gsdr_result_free);
    if (!r) rc = fail(GSDR_ENOMEM, "server: out of host memory");
    if (!rc)
        rc = cluster_fasta(j->fasta.data(), (int64_t)j->fasta.size(), &o, r.get(), nullptr,
                           &admit);
    if (!rc) {
        const char* data = nullptr;
        int64_t nb = 0;
        gsdr_result_output(r.get(), &data, &nb);
        j->out.assign(data, data + nb);
        const int32_t* cl = gsdr_result_cluster(r.get());
        j->cluster.assign(cl, cl + gsdr_result_count(r.get()));
    } else {
        j->error = gsdr_last_error();
    }
    r.reset();
    j->fasta.clear();
    j->fasta.shrink_to_fit();
    std::lock_guard<std::mutex> lock(s->mu);
    s->inflight--;
    if (j->express) s->express = 0;
    s->mem_used -= j->parse_bytes + j->job_bytes;
    if (j->clustering) s->clustering--;
    finish(s, j, rc);
    s->cv_sched.notify_all();
}

// A job that has waited this long goes before smaller ones.
constexpr double kAgeMs = 1000.0;
// Jobs of at most this many FASTA bytes may take the express slot (the
// default of gsdr_server_opts.express_bytes).
constexpr int64_t kExpressBytes = (int64_t)4 << 20;

using JobIt = std::deque<std::shared_ptr<ServerJob>>::iterator;

JobIt smallest_job(gsdr_server* s) {
    auto& q = s->queue;
    auto best = q.begin();
    for (auto it = q.begin(); it != q.end(); ++it)
        if ((*it)->fasta.size() < (*best)->fasta.size()) best = it;
    return best;
}

// The queued job to start now, or the queue's end: with a regular slot free
// the job that has waited kAgeMs or more (the queue is in submission order,
// so its front has waited longest), else the smallest; with only the express
// slot free the smallest, if it is short enough.
JobIt next_job(gsdr_server* s) {
    auto& q = s->queue;
    if (q.empty()) return q.end();
    if (s->inflight - s->express < s->so.max_inflight) {
        if (now_ms() - q.front()->t_submit >= kAgeMs) return q.begin();
        return smallest_job(s);
    }
    if (s->express == 0 && s->so.express_bytes > 0) {
        auto it = smallest_job(s);
        if ((int64_t)(*it)->fasta.size() <= s->so.express_bytes) return it;
    }
    return q.end();
}

void scheduler_loop(gsdr_server* s) {
    cudaSetDevice(s->so.device);
    while (true) {
        std::unique_lock<std::mutex> lock(s->mu);
        // the choice is made when a slot is free, among the jobs queued then
        s->cv_sched.wait(lock, [&] { return s->stopping || next_job(s) != s->queue.end(); });
        if (s->stopping && s->queue.empty()) return;
        std::shared_ptr<ServerJob> j;
        if (s->stopping) {
            j = s->queue.front();
            s->queue.pop_front();
        } else {
            auto it = next_job(s);
            j = *it;
            s->queue.erase(it);
            j->express = s->inflight - s->express >= s->so.max_inflight;
        }
        j->parse_bytes = cluster_fasta_parse_bytes((int64_t)j->fasta.size(), j->records,
                                                   j->newlines);
        // step 1: room for the parse buffers (or nothing running); the slot
        // was free when the job was chosen and only this thread takes slots
        s->cv_sched.wait(lock, [&] {
            return s->stopping ||
                   s->mem_used + j->parse_bytes <= s->so.mem_budget || s->inflight == 0;
        });
        if (s->stopping) {
            j->error = "server stopped";
            finish(s, j, GSDR_EBUSY);
            continue;
        }
        s->inflight++;
        if (j->express) s->express = 1;
        s->mem_used += j->parse_bytes;
        s->ready.push_back(j);
        s->cv_work.notify_one();
    }
}

void worker_loop(gsdr_server* s) {
    cudaSetDevice(s->so.device);
    while (true) {
        std::shared_ptr<ServerJob> j;
        {
            std::unique_lock<std::mutex> lock(s->mu);
            s->cv_work.wait(lock, [&] { return s->workers_stop || !s->ready.empty(); });
            if (s->ready.empty()) return;
            j = s->ready.front();
            s->ready.pop_front();
        }
        run_job(s, j);
    }
}

}  // namespace

extern "C" {

int gsdr_server_create(const gsdr_server_opts* so, gsdr_server** out) {
    if (!so || !out) return fail(GSDR_EINVAL, "server: null argument");
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0)
        return fail(GSDR_EDEVICE, "server: no CUDA device");
    if (so->device < 0 || so->device >= n) return fail(GSDR_EINVAL, "server: bad device");
    gsdr_server* s = new (std::nothrow) gsdr_server();
    if (!s) return fail(GSDR_ENOMEM, "server: out of host memory");
    s->so = *so;
    if (s->so.max_inflight <= 0) s->so.max_inflight = 4;
    if (s->so.express_bytes == 0) s->so.express_bytes = kExpressBytes;
    if (s->so.mem_budget <= 0) {
        size_t free_b = 0, total_b = 0;
        cudaSetDevice(so->device);
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
            delete s;
            return fail(GSDR_EDEVICE, "server: cudaMemGetInfo failed");
        }
        s->so.mem_budget = (int64_t)(free_b / 10 * 8);
    }
    // a worker per slot, the express slot included
    for (int w = 0; w <= s->so.max_inflight; w++) s->workers.emplace_back(worker_loop, s);
    s->scheduler = std::thread(scheduler_loop, s);
    *out = s;
    return GSDR_OK;
}

int gsdr_server_submit(gsdr_server* s, const char* fasta, int64_t n, float threshold,
                       int64_t* job) {
    if (!s || (!fasta && n > 0) || n < 0 || !job) return fail(GSDR_EINVAL, "server: bad submit");
    auto j = std::make_shared<ServerJob>();
    try {
        j->fasta.assign(fasta, fasta + n);
    } catch (const std::bad_alloc&) {
        return fail(GSDR_ENOMEM, "server: out of host memory");
    }
    // bounds for the parse buffers: every '>' may open a record (and the first
    // line always does), every newline ends a line
    j->records = (int64_t)std::count(j->fasta.begin(), j->fasta.end(), '>') + 1;
    j->newlines = (int64_t)std::count(j->fasta.begin(), j->fasta.end(), '\n');
    j->threshold = threshold;
    j->t_submit = now_ms();
    // t outside [0.8, 1): the job is refused as checkOption refuses it, at once
    gsdr_opts o;
    gsdr_default_opts(&o);
    o.threshold = threshold;
    o.batch = s->so.batch;
    const int refused = gsdr_resolve_opts(&o, nullptr);
    if (refused) {
        j->error = gsdr_last_error();
        j->fasta.clear();
        j->fasta.shrink_to_fit();
    }
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->stopping) return fail(GSDR_EBUSY, "server: stopping");
    j->id = s->next_id++;
    s->jobs[j->id] = j;
    *job = j->id;
    if (refused) {
        j->t_start = j->t_submit;
        finish(s, j, refused);
        return GSDR_OK;
    }
    s->queue.push_back(j);
    s->cv_sched.notify_all();
    return GSDR_OK;
}

int gsdr_server_wait(gsdr_server* s, int64_t timeout_ms, int64_t* job, int32_t* job_status,
                     double* latency_ms) {
    if (!s || !job) return fail(GSDR_EINVAL, "server: bad wait");
    std::unique_lock<std::mutex> lock(s->mu);
    auto ready = [&] { return !s->finished.empty(); };
    if (timeout_ms < 0) {
        s->cv_done.wait(lock, ready);
    } else if (!s->cv_done.wait_for(lock, std::chrono::milliseconds(timeout_ms), ready)) {
        return GSDR_ETIMEOUT;
    }
    const int64_t id = s->finished.front();
    s->finished.pop_front();
    auto& j = s->jobs[id];
    *job = id;
    if (job_status) *job_status = j->status;
    if (latency_ms) *latency_ms = j->t_done - j->t_submit;
    return GSDR_OK;
}

int gsdr_server_result(gsdr_server* s, int64_t job, char* buf, int64_t cap, int64_t* need,
                       int32_t* cluster, int32_t* n_reads) {
    if (!s) return fail(GSDR_EINVAL, "server: null server");
    std::shared_ptr<ServerJob> j;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        auto it = s->jobs.find(job);
        if (it == s->jobs.end()) return fail(GSDR_ENOTFOUND, "server: unknown job");
        j = it->second;
        if (j->t_done == 0) return fail(GSDR_EBUSY, "server: job not finished");
    }
    if (j->status != GSDR_OK) return fail(j->status, j->error.c_str());
    if (need) *need = (int64_t)j->out.size();
    if (n_reads) *n_reads = (int32_t)j->cluster.size();
    if (buf) {
        if (cap < (int64_t)j->out.size()) return fail(GSDR_EINVAL, "server: buffer too small");
        std::memcpy(buf, j->out.data(), j->out.size());
    }
    if (cluster) std::memcpy(cluster, j->cluster.data(), j->cluster.size() * sizeof(int32_t));
    return GSDR_OK;
}

int gsdr_server_times(gsdr_server* s, int64_t job, double* queued_ms, double* run_ms) {
    if (!s) return fail(GSDR_EINVAL, "server: null server");
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->jobs.find(job);
    if (it == s->jobs.end()) return fail(GSDR_ENOTFOUND, "server: unknown job");
    const ServerJob& j = *it->second;
    if (j.t_done == 0) return fail(GSDR_EBUSY, "server: job not finished");
    const double start = j.t_start > 0 ? j.t_start : j.t_done;  // refused before running
    if (queued_ms) *queued_ms = start - j.t_submit;
    if (run_ms) *run_ms = j.t_done - start;
    return GSDR_OK;
}

int gsdr_server_release(gsdr_server* s, int64_t job) {
    if (!s) return fail(GSDR_EINVAL, "server: null server");
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->jobs.find(job);
    if (it == s->jobs.end()) return fail(GSDR_ENOTFOUND, "server: unknown job");
    if (it->second->t_done == 0) return fail(GSDR_EBUSY, "server: job not finished");
    s->jobs.erase(it);
    return GSDR_OK;
}

void gsdr_server_destroy(gsdr_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stopping = true;
        s->cv_sched.notify_all();
    }
    if (s->scheduler.joinable()) s->scheduler.join();
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->workers_stop = true;
        s->cv_work.notify_all();
    }
    for (auto& w : s->workers)
        if (w.joinable()) w.join();
    delete s;
}

}  // extern "C"
