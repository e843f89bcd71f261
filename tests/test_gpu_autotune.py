"""The autotuner (gsdr_autotune, csrc/autotune.cu): every setting it tries
gives the same clusters, the setting it picks is one of those it timed, and a
later automatic job (batch 0) of the same workload bucket takes the stored
setting from the tuning cache by itself."""
import os

import numpy as np
import pytest

import gsdr
from gsdr.autotune import autotune, tuned_opts

pytestmark = pytest.mark.gpu


def test_autotune_picks_a_timed_setting_with_identical_results(tmp_path):
    data = gsdr.synth_fasta(0, n_reads=4000, seed=81)
    cache = str(tmp_path / "tune.tsv")
    res = autotune(data, 0.95, reps=600, runs=1, cache_path=cache)
    timed = [t for t in res["trials"] if "ms" in t]
    assert res["best"] in timed and len(timed) >= 10
    assert {t["stage"] for t in timed} >= {"R x form", "band tiles", "block shape",
                                           "staging depth"}
    assert all(t["representatives"] > 0 for t in timed)
    f = gsdr.Fasta.parse(data)
    try:
        a = gsdr.clustering(f, gsdr.default_opts(threshold=0.95))
        b = gsdr.clustering(f, tuned_opts(res, 0.95))
        c = gsdr.clustering(f, gsdr.default_opts(threshold=0.95, batch=1))
    finally:
        f.close()
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(a, c)
    with open(cache) as fh:
        rows = [ln for ln in fh if ln.strip() and not ln.startswith("#")]
    assert len(rows) == 1 and res["bucket"] in rows[0]


def test_automatic_job_reads_the_cache(tmp_path, monkeypatch):
    data = gsdr.synth_fasta(0, n_reads=3000, seed=84)
    cache = str(tmp_path / "tune.tsv")
    monkeypatch.setenv("GSDR_TUNE_CACHE", cache)
    f = gsdr.Fasta.parse(data)
    try:
        ref, st0 = gsdr.clustering(f, gsdr.default_opts(threshold=0.95), stats=True)
        assert st0.tuned == 0  # no cache yet
        res = autotune(data, 0.95, reps=400, runs=1)  # default path: $GSDR_TUNE_CACHE
        assert os.path.exists(cache) and res["cache"] == cache
        cl, st = gsdr.clustering(f, gsdr.default_opts(threshold=0.95), stats=True)
        assert st.tuned == 1
        if res["best"]["batch"] > 1:
            assert st.batch == res["best"]["batch"]
        # an explicit batch bypasses the cache
        _, st2 = gsdr.clustering(f, gsdr.default_opts(threshold=0.95, batch=64), stats=True)
        assert st2.tuned == 0
    finally:
        f.close()
    np.testing.assert_array_equal(cl, ref)


@pytest.mark.parametrize("knobs", [dict(align_blocks=1), dict(align_blocks=2, filter_blocks=1),
                                   dict(filter_blocks=3), dict(graph_steps=2),
                                   dict(graph_steps=64, batch=1), dict(graph_steps=8, batch=64)])
def test_block_shape_and_staging_depth_keep_the_result(knobs):
    data = gsdr.synth_fasta(0, n_reads=2500, seed=85)
    f = gsdr.Fasta.parse(data)
    try:
        ref = gsdr.clustering(f, gsdr.default_opts(threshold=0.95, batch=1))
        cl = gsdr.clustering(f, gsdr.default_opts(threshold=0.95, **knobs))
    finally:
        f.close()
    np.testing.assert_array_equal(cl, ref)


@pytest.mark.parametrize("form", [1, 2, 3])
def test_word_filter_option_selects_the_form(form):
    data = gsdr.synth_fasta(0, n_reads=1500, seed=82)
    f = gsdr.Fasta.parse(data)
    try:
        cl, st = gsdr.clustering(f, gsdr.default_opts(threshold=0.95, word_filter=form),
                                 stats=True)
        ref = gsdr.clustering(f, gsdr.default_opts(threshold=0.95, batch=1))
    finally:
        f.close()
    assert st.word_index == {1: 0, 2: 1, 3: 2}[form]
    np.testing.assert_array_equal(cl, ref)


def test_word_filter_option_selects_the_masks():
    # the mask form takes reads of at most 255 k-mers
    data = gsdr.synth_fasta(0, n_reads=2000, seed=84, len_lo=60, len_hi=240, n_seeds=300)
    f = gsdr.Fasta.parse(data)
    try:
        cl, st = gsdr.clustering(f, gsdr.default_opts(threshold=0.95, word_filter=4),
                                 stats=True)
        ref = gsdr.clustering(f, gsdr.default_opts(threshold=0.95, batch=1))
    finally:
        f.close()
    assert st.word_index == 3
    np.testing.assert_array_equal(cl, ref)


def test_limited_run_stops_early_and_full_run_is_unaffected():
    data = gsdr.synth_fasta(0, n_reads=3000, seed=83)
    f = gsdr.Fasta.parse(data)
    try:
        job = gsdr.Job(f, gsdr.default_opts(threshold=0.95, batch=64))
        try:
            part = job.run(5)
            assert part.passes == 5
            full = job.run()
            cl = job.cluster()
        finally:
            job.close()
        ref = gsdr.clustering(f, gsdr.default_opts(threshold=0.95, batch=1))
    finally:
        f.close()
    assert part.rounds < full.rounds
    np.testing.assert_array_equal(cl, ref)


def test_cluster_executable_uses_the_cache(tmp_path):
    """`cluster` with b 0 (automatic) takes the tuned knobs: same output."""
    import subprocess

    data = gsdr.synth_fasta(0, n_reads=2000, seed=86)
    inp = tmp_path / "in.fa"
    inp.write_bytes(data)
    cache = str(tmp_path / "tune.tsv")
    autotune(data, 0.95, reps=300, runs=1, cache_path=cache)
    env = dict(os.environ, GSDR_TUNE_CACHE=cache, GSDR_TRACE="1")
    outs, errs = [], []
    for tag, e in (("tuned", env), ("untuned", dict(env, GSDR_TUNE_CACHE=""))):
        out = tmp_path / f"{tag}.fa"
        r = subprocess.run([gsdr.CLI_PATH, "i", str(inp), "o", str(out), "t", "0.95"], env=e,
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        outs.append(out.read_bytes())
        errs.append(r.stderr)
    assert outs[0] == outs[1]
    assert "knobs from the tuning cache" in errs[0]
    assert "knobs from the tuning cache" not in errs[1]
