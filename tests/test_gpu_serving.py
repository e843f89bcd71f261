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
