"""Checkpoint / resume (gsdr_job_resume): a clustering stopped after some
passes or rounds leaves its whole state in the cluster array (the reference's
loop carries only cluster[] between rounds, cuda-version/func.cu:1001-1066);
resuming from that array -- on the same job, on a new job, from a file, in the
other form, or in several legs -- gives exactly the uninterrupted result."""
import numpy as np
import pytest

import gsdr

pytestmark = pytest.mark.gpu


def _full(f, t, batch):
    return gsdr.clustering(f, gsdr.default_opts(threshold=t, batch=batch))


@pytest.mark.parametrize("cfg,n,t", [(0, 3000, 0.95), (1, 4000, 0.95), (0, 1200, 0.85)])
@pytest.mark.parametrize("batch,stop", [(1, 1), (1, 37), (64, 3), (0, 5)])
def test_resume_equals_uninterrupted(tmp_path, cfg, n, t, batch, stop):
    data = gsdr.synth_fasta(cfg, n_reads=n, seed=91 + cfg)
    f = gsdr.Fasta.parse(data)
    try:
        want = _full(f, t, batch)
        job = gsdr.Job(f, gsdr.default_opts(threshold=t, batch=batch))
        try:
            part = job.run(stop)
            cp = job.cluster()
        finally:
            job.close()
        assert (cp == -1).any(), "the stopped run must be unfinished"
        assert part.rounds > 0
        path = tmp_path / "checkpoint.npy"
        np.save(path, cp)
        # a new job over the same reads, from the saved array
        job2 = gsdr.Job(f, gsdr.default_opts(threshold=t, batch=batch))
        try:
            job2.resume(np.load(path))
            got = job2.cluster()
        finally:
            job2.close()
    finally:
        f.close()
    np.testing.assert_array_equal(got, want)


def test_resume_in_legs_and_across_forms():
    data = gsdr.synth_fasta(0, n_reads=2500, seed=95)
    f = gsdr.Fasta.parse(data)
    try:
        want = _full(f, 0.95, 1)
        plain = gsdr.Job(f, gsdr.default_opts(threshold=0.95, batch=1))
        batched = gsdr.Job(f, gsdr.default_opts(threshold=0.95, batch=32))
        try:
            plain.run(20)
            cp = plain.cluster()
            for _ in range(3):  # three batched legs of two passes each
                batched.resume(cp, 2)
                cp = batched.cluster()
            plain.resume(cp)  # the rest in the plain form
            got = plain.cluster()
        finally:
            plain.close()
            batched.close()
    finally:
        f.close()
    np.testing.assert_array_equal(got, want)


def test_resume_refuses_impossible_states():
    data = gsdr.synth_fasta(0, n_reads=500, seed=96)
    f = gsdr.Fasta.parse(data)
    try:
        job = gsdr.Job(f, gsdr.default_opts(threshold=0.95))
        try:
            n = f.n
            bad = []
            a = np.full(n, -1, dtype=np.int32)
            a[5] = 7  # joined to a later read
            bad.append(a)
            a = np.full(n, -1, dtype=np.int32)
            a[4] = 2  # joined to a read that is no representative
            bad.append(a)
            a = np.full(n, -1, dtype=np.int32)
            a[10] = 10  # a representative after unclustered reads
            bad.append(a)
            for a in bad:
                with pytest.raises(gsdr.GsdrError) as e:
                    job.resume(a)
                assert e.value.status == gsdr.EINVAL
            # the fresh state resumes to the full result
            job.resume(np.full(n, -1, dtype=np.int32))
            got = job.cluster()
        finally:
            job.close()
        want = _full(f, 0.95, 1)
    finally:
        f.close()
    np.testing.assert_array_equal(got, want)
