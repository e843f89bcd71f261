"""Serving: jobs of different sizes and thresholds submitted while others
run.  Each job's output (FASTA bytes and cluster array) must equal the output
of gsdr_cluster on that job alone (integer work: tolerance zero); t = 1.00 is
rejected as the reference rejects it (cuda-version/func.cu:43-48)."""
import numpy as np
import pytest

import gsdr
import oracle_binding as orc

pytestmark = pytest.mark.gpu

THRESHOLDS = [0.80, 0.85, 0.90, 0.95, 1.00]


def make_jobs(n_jobs, seed):
    rng = np.random.default_rng(seed)
    jobs = []
    for i in range(n_jobs):
        t = THRESHOLDS[i % len(THRESHOLDS)]
        lo, hi = (200, 1200) if t < 0.88 else (300, 6000)
        n = int(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        data = gsdr.synth_fasta(4, n_reads=n, seed=1000 + i, n_seeds=max(1, n // 5),
                                len_lo=150, len_hi=2000 if t < 0.88 else 5000)
        jobs.append((data, t))
    return jobs


def alone(data, t):
    f = gsdr.Fasta.parse(data)
    try:
        cl = gsdr.clustering(f, gsdr.default_opts(threshold=t))
        return f.format(cl), cl
    finally:
        f.close()


@pytest.mark.parametrize("budget,inflight", [(0, 4), (64 << 20, 3)])
def test_each_job_same_alone_and_in_the_mix(budget, inflight):
    jobs = make_jobs(12, seed=budget & 0xff)
    srv = gsdr.Server(max_inflight=inflight, mem_budget=budget)
    try:
        ids = {srv.submit(data, t): k for k, (data, t) in enumerate(jobs)}
        done = {}
        while len(done) < len(ids):
            r = srv.wait(120000)
            assert r is not None, "a job did not finish"
            jid, status, lat = r
            done[jid] = (status, lat)
        for jid, k in ids.items():
            data, t = jobs[k]
            status, lat = done[jid]
            assert lat > 0
            if t >= 1.0:
                assert status == gsdr.EINVAL
                continue
            assert status == gsdr.OK, gsdr.lib().gsdr_strerror(status)
            out, cl = srv.result(jid)
            want_out, want_cl = alone(data, t)
            np.testing.assert_array_equal(cl, want_cl)
            assert out == want_out
            srv.release(jid)
    finally:
        srv.close()


def test_serving_matches_oracle_small(tmp_path):
    srv = gsdr.Server(max_inflight=2)
    try:
        datas = [gsdr.synth_fasta(4, n_reads=400, seed=77 + i, n_seeds=80, len_hi=1500)
                 for i in range(3)]
        ids = [srv.submit(d, 0.95) for d in datas]
        for _ in ids:
            assert srv.wait(60000) is not None
        for jid, d in zip(ids, datas):
            out, cl = srv.result(jid)
            _, ocl, _, ofa = orc.run_bytes(d, tmp_path, name=f"j{jid}.fa", t=0.95)
            np.testing.assert_array_equal(cl, ocl)
            assert out == ofa
    finally:
        srv.close()


def test_smaller_jobs_start_first():
    # one slot: while a first job runs, a large job and then two small ones
    # queue; when the slot frees, the small ones go first (smallest queued
    # job, the large one not yet waiting 1 s), and every result is exact
    # (the first job runs long enough for the others to be copied in while it
    # runs, well under the 1 s after which a waiting job goes first)
    first = gsdr.synth_fasta(4, n_reads=40000, seed=2001, n_seeds=8000, len_lo=150,
                             len_hi=2000)
    large = gsdr.synth_fasta(4, n_reads=20000, seed=2002, n_seeds=4000, len_lo=150, len_hi=2000)
    small = [gsdr.synth_fasta(4, n_reads=400, seed=2003 + i, n_seeds=80, len_lo=150,
                              len_hi=2000) for i in range(2)]
    srv = gsdr.Server(max_inflight=1)
    try:
        j0 = srv.submit(first, 0.95)
        jl = srv.submit(large, 0.95)
        js = [srv.submit(d, 0.95) for d in small]
        j_refused = srv.submit(small[0], 1.0)
        order = []
        while len(order) < 5:
            r = srv.wait(120000)
            assert r is not None, "a job did not finish"
            order.append(r[0])
            if r[0] == j_refused:
                assert r[1] == gsdr.EINVAL
            else:
                assert r[1] == gsdr.OK
        # refused at submission (no time in the queue); the small jobs
        # before the large one
        assert srv.times(j_refused)[0] == 0.0
        assert order.index(js[0]) < order.index(jl)
        assert order.index(js[1]) < order.index(jl)
        for jid, data in [(j0, first), (jl, large)] + list(zip(js, small)):
            out, cl = srv.result(jid)
            want_out, want_cl = alone(data, 0.95)
            np.testing.assert_array_equal(cl, want_cl)
            assert out == want_out
    finally:
        srv.close()


@pytest.mark.parametrize("express", [0, -1])
def test_express_slot_takes_short_jobs(express):
    # one regular slot held by a long job: a short job submitted meanwhile
    # runs in the express slot (default on) and finishes first; with the
    # express slot off it waits for the long job
    import time

    long_job = gsdr.synth_fasta(4, n_reads=40000, seed=2101, n_seeds=8000, len_lo=150,
                                len_hi=2000)
    short = gsdr.synth_fasta(4, n_reads=300, seed=2102, n_seeds=60, len_lo=150, len_hi=2000)
    srv = gsdr.Server(max_inflight=1, express_bytes=express)
    try:
        jl = srv.submit(long_job, 0.95)
        time.sleep(0.02)
        js = srv.submit(short, 0.95)
        order = []
        while len(order) < 2:
            r = srv.wait(120000)
            assert r is not None and r[1] == gsdr.OK
            order.append(r[0])
        assert order == ([js, jl] if express == 0 else [jl, js])
        out, cl = srv.result(js)
        want_out, want_cl = alone(short, 0.95)
        np.testing.assert_array_equal(cl, want_cl)
        assert out == want_out
    finally:
        srv.close()
