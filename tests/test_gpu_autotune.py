"""The autotuner (gsdr/autotune.py): every setting it tries gives the same
clusters, and the setting it picks is one of those it timed."""
import numpy as np
import pytest

import gsdr
from gsdr.autotune import autotune, tuned_opts

pytestmark = pytest.mark.gpu


def test_autotune_picks_a_timed_setting_with_identical_results():
    data = gsdr.synth_fasta(0, n_reads=4000, seed=81)
    res = autotune(data, 0.95, reps=600, r_values=(64, 256), runs=1)
    timed = [t for t in res["trials"] if "ms" in t]
    assert res["best"] in timed and len(timed) >= 5
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
