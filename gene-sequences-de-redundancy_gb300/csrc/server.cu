// server.cu -- serving: continuous batching of independent clustering jobs on
// one GPU (gsdr_server_* in include/gsdr.h; no counterpart in the reference).
//
// Jobs arrive as FASTA bytes with their own threshold.  A scheduler thread
// takes them in arrival order, parses each one (the reference's readFile rules
// and sort), computes its device footprint and admits it as soon as a slot is
// free (max_inflight) and its footprint fits the remaining memory budget.  An
// admitted job runs on its own worker thread and CUDA stream through the same
// gsdr::Job as gsdr_cluster, so jobs overlap on the device and each result is
// exactly what gsdr_cluster returns for that job alone.  A job larger than the
// whole budget waits until nothing else runs and then runs alone.
#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
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
    float threshold = 0.95f;
    double t_submit = 0, t_start = 0, t_done = 0;
    int status = GSDR_OK;
    std::string error;
    gsdr_fasta* parsed = nullptr;
    std::vector<int32_t> cluster;
    std::vector<char> out;
    int64_t footprint = 0;
    ~ServerJob() {
        if (parsed) gsdr_fasta_free(parsed);
    }
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
    int64_t mem_used = 0;
    int64_t next_id = 1;
    bool stopping = false;
};

namespace {

void run_job(gsdr_server* s, std::shared_ptr<ServerJob> j) {
    j->t_start = now_ms();
    gsdr_opts o;
    gsdr_default_opts(&o);
    o.threshold = j->threshold;
    o.device = s->so.device;
    o.batch = s->so.batch;
    gsdr_reads v;
    gsdr_fasta_view(j->parsed, &v);
    j->cluster.assign(v.n > 0 ? v.n : 1, 0);
    int rc = GSDR_OK;
    {
        Job job;
        rc = job.init(&v, &o);
        if (!rc) rc = job.upload(&v);
        if (!rc) rc = job.run();
        if (!rc) rc = job.download(j->cluster.data());
        if (rc) j->error = gsdr_last_error();
    }
    if (!rc) {
        int64_t need = 0;
        gsdr_fasta_format(j->parsed, j->cluster.data(), nullptr, 0, &need);
        j->out.resize((size_t)need);
        rc = gsdr_fasta_format(j->parsed, j->cluster.data(), j->out.data(), need, &need);
    }
    j->cluster.resize(v.n > 0 ? v.n : 0);
    std::lock_guard<std::mutex> lock(s->mu);
    j->status = rc;
    j->t_done = now_ms();
    s->inflight--;
    s->mem_used -= j->footprint;
    s->finished.push_back(j->id);
    s->cv_done.notify_all();
    s->cv_sched.notify_all();
}

void scheduler_loop(gsdr_server* s) {
    cudaSetDevice(s->so.device);
    while (true) {
        std::shared_ptr<ServerJob> j;
        {
            std::unique_lock<std::mutex> lock(s->mu);
            s->cv_sched.wait(lock, [&] { return s->stopping || !s->queue.empty(); });
            if (s->stopping && s->queue.empty()) return;
            j = s->queue.front();
            s->queue.pop_front();
        }
        // parse and size the job outside the lock
        gsdr_opts o;
        gsdr_default_opts(&o);
        o.threshold = j->threshold;
        o.batch = s->so.batch;
        int rc = gsdr_resolve_opts(&o, nullptr);
        if (!rc) rc = gsdr_fasta_parse(j->fasta.data(), (int64_t)j->fasta.size(), &j->parsed);
        if (!rc) {
            gsdr_reads v;
            gsdr_fasta_view(j->parsed, &v);
            j->footprint = Job::footprint(&v, &o);
            if (j->footprint < 0) rc = GSDR_EINVAL;
        }
        j->fasta.clear();
        j->fasta.shrink_to_fit();
        std::unique_lock<std::mutex> lock(s->mu);
        if (rc) {
            j->status = rc;
            j->error = gsdr_last_error();
            j->t_done = now_ms();
            s->finished.push_back(j->id);
            s->cv_done.notify_all();
            continue;
        }
        // admission: a free slot and room in the budget (or nothing running)
        s->cv_sched.wait(lock, [&] {
            return s->stopping || (s->inflight < s->so.max_inflight &&
                                   (s->mem_used + j->footprint <= s->so.mem_budget ||
                                    s->inflight == 0));
        });
        if (s->stopping) {
            j->status = GSDR_EBUSY;
            j->error = "server stopped";
            j->t_done = now_ms();
            s->finished.push_back(j->id);
            s->cv_done.notify_all();
            continue;
        }
        s->inflight++;
        s->mem_used += j->footprint;
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
    if (s->so.mem_budget <= 0) {
        size_t free_b = 0, total_b = 0;
        cudaSetDevice(so->device);
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
            delete s;
            return fail(GSDR_EDEVICE, "server: cudaMemGetInfo failed");
        }
        s->so.mem_budget = (int64_t)(free_b / 10 * 8);
    }
    for (int w = 0; w < s->so.max_inflight; w++) s->workers.emplace_back(worker_loop, s);
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
    j->threshold = threshold;
    j->t_submit = now_ms();
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->stopping) return fail(GSDR_EBUSY, "server: stopping");
    j->id = s->next_id++;
    s->jobs[j->id] = j;
    s->queue.push_back(j);
    *job = j->id;
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
