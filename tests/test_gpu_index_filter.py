"""Batched word filter forms against the oracle: the per-pass inverted k-mer
index (chosen for reads holding few of the 4^k k-mers, e.g. 150 bp reads at
k = 7), the k-mer presence bitmaps (k <= 6 otherwise) and the per-tentative
tables.  Identical cluster arrays and FASTA bytes in every form, at every R,
every word length, and for reads too short to hold a k-mer (the reference's
kernel_filter, cuda-version/func.cu:803-826)."""
import numpy as np
import pytest

import gsdr
import oracle_binding as orc

pytestmark = pytest.mark.gpu


def run_form(data, tmp_path, monkeypatch, t, batch, form, w=0, d=3):
    if form is None:
        monkeypatch.delenv("GSDR_BFILTER", raising=False)
    else:
        monkeypatch.setenv("GSDR_BFILTER", form)
    _, ocl, ost, ofa = orc.run_bytes(data, tmp_path, t=t, w=w, d=d)
    f = gsdr.Fasta.parse(data)
    opts = gsdr.default_opts(threshold=t, drop=d, batch=batch, word_length=w)
    cl, st = gsdr.clustering(f, opts, stats=True)
    out = f.format(cl)
    f.close()
    bad = np.nonzero(cl != ocl)[0]
    assert len(bad) == 0, f"{form} R={batch}: {len(bad)} reads differ, first {bad[:8]}"
    assert out == ofa
    assert st.rounds == ost.rounds
    assert st.pairs_accepted == ost.accepted
    return st, ost


@pytest.mark.parametrize("batch", [2, 64, 256, 1024, 0])
def test_c2_recipe_index_auto(tmp_path, monkeypatch, batch):
    data = gsdr.synth_fasta(2, n_reads=30000, seed=33)
    st, ost = run_form(data, tmp_path, monkeypatch, 0.90, batch, None)
    assert st.k == 7 and st.word_index == 1
    # the pairs sent to the alignment are the pairs passing both filters
    assert st.passes < st.rounds


def test_c2_recipe_same_pairs_both_forms(tmp_path, monkeypatch):
    data = gsdr.synth_fasta(2, n_reads=20000, seed=34)
    si, _ = run_form(data, tmp_path, monkeypatch, 0.90, 128, "index")
    stt, _ = run_form(data, tmp_path, monkeypatch, 0.90, 128, "table")
    assert si.word_index == 1 and stt.word_index == 0
    assert si.pairs_prefilter == stt.pairs_prefilter
    assert si.pairs_aligned == stt.pairs_aligned
    assert si.cells == stt.cells


@pytest.mark.parametrize("t", [0.88, 0.90, 0.93, 0.97])
def test_index_forced_word_lengths(tmp_path, monkeypatch, t):
    data = gsdr.synth_fasta(0, n_reads=2000, seed=35)
    st, ost = run_form(data, tmp_path, monkeypatch, t, 64, "index")
    assert st.word_index == 1 and st.k == ost.k


@pytest.mark.parametrize("w", [4, 5, 6, 7])
def test_index_forced_word_override(tmp_path, monkeypatch, w):
    data = gsdr.synth_fasta(0, n_reads=1500, seed=36)
    st, _ = run_form(data, tmp_path, monkeypatch, 0.95, 32, "index", w=w)
    assert st.k == w and st.word_index == 1


def test_index_long_reads(tmp_path, monkeypatch):
    data = gsdr.synth_fasta(1, n_reads=5000, seed=37)
    st, _ = run_form(data, tmp_path, monkeypatch, 0.95, 256, "index")
    assert st.word_index == 1


@pytest.mark.parametrize("form", ["index", "table"])
def test_very_short_reads(tmp_path, monkeypatch, form):
    # 3-48 bp reads at k = 7: reads of at most 6 bases hold no k-mer, and the
    # word cutoff is never below 1 (func.cu:312-337), so they are never aligned
    data = gsdr.synth_fasta(0, n_reads=3000, seed=38, len_lo=3, len_hi=40, n_seeds=400)
    lens = np.array([len(l) for l in data.split(b"\n")[1::2]])
    cw, _, _ = orc.cutoffs(lens, 0.90, 7)
    assert (lens <= 6).any() and (cw >= 1).all()
    st, _ = run_form(data, tmp_path, monkeypatch, 0.90, 64, form, w=7)
    assert st.word_index == (1 if form == "index" else 0)


def test_index_form_is_repeatable(monkeypatch):
    monkeypatch.setenv("GSDR_BFILTER", "index")
    data = gsdr.synth_fasta(2, n_reads=20000, seed=39)
    f = gsdr.Fasta.parse(data)
    opts = gsdr.default_opts(threshold=0.90, batch=0)
    job = gsdr.Job(f, opts)
    try:
        assert job.run().word_index == 1
        a = job.cluster()
        job.run()
        b = job.cluster()
    finally:
        job.close()
        f.close()
    assert np.array_equal(a, b)


# ---- k-mer presence bitmaps (k <= 6): bound D <= S <= D + min(excess), exact
# sum for the pairs it leaves open

@pytest.mark.parametrize("batch", [2, 64, 256, 0])
def test_c0_recipe_bits_auto(tmp_path, monkeypatch, batch):
    # 200-1000 bp reads hold a small part of the 4^6 k-mers: bitmaps chosen
    data = gsdr.synth_fasta(0, n_reads=4000, seed=40)
    st, _ = run_form(data, tmp_path, monkeypatch, 0.95, batch, None)
    assert st.k == 6 and st.word_index == 2


@pytest.mark.parametrize("batch", [2, 256])
def test_c1_recipe_bits_forced(tmp_path, monkeypatch, batch):
    # long reads: the bound leaves most pairs open (exact sums, queue refills)
    data = gsdr.synth_fasta(1, n_reads=8000, seed=41)
    st, _ = run_form(data, tmp_path, monkeypatch, 0.95, batch, "bits")
    assert st.k == 6 and st.word_index == 2


def test_c1_recipe_bits_auto(tmp_path, monkeypatch):
    # long reads too: the two-level bitmaps are the automatic form for k <= 6
    data = gsdr.synth_fasta(1, n_reads=8000, seed=41)
    st, _ = run_form(data, tmp_path, monkeypatch, 0.95, 0, None)
    assert st.k == 6 and st.word_index == 2


@pytest.mark.parametrize("batch", [2, 256])
def test_c1_recipe_tables_forced(tmp_path, monkeypatch, batch):
    data = gsdr.synth_fasta(1, n_reads=8000, seed=41)
    st, _ = run_form(data, tmp_path, monkeypatch, 0.95, batch, "table")
    assert st.k == 6 and st.word_index == 0


@pytest.mark.parametrize("w", [4, 5, 6, 7])
def test_bits_word_lengths(tmp_path, monkeypatch, w):
    data = gsdr.synth_fasta(0, n_reads=2000, seed=42)
    st, _ = run_form(data, tmp_path, monkeypatch, 0.95, 64, "bits", w=w)
    assert st.k == w and st.word_index == 2


@pytest.mark.parametrize("batch", [32, 0])
def test_bits_k7_long_reads(tmp_path, monkeypatch, batch):
    # t = 0.90 gives k = 7; reads of 150-5000 bp hold too many 7-mers for the
    # index: the two-level bitmaps (four times larger at k = 7) are automatic
    data = gsdr.synth_fasta(4, n_reads=3000, seed=45, n_seeds=600, len_lo=150, len_hi=5000)
    st, ost = run_form(data, tmp_path, monkeypatch, 0.90, batch, None)
    assert st.k == 7 and ost.k == 7 and st.word_index == 2


@pytest.mark.parametrize("t", [0.88, 0.93, 0.97])
def test_bits_thresholds(tmp_path, monkeypatch, t):
    data = gsdr.synth_fasta(0, n_reads=2000, seed=43)
    st, ost = run_form(data, tmp_path, monkeypatch, t, 128, "bits")
    assert st.k == ost.k
    if st.k <= 6:
        assert st.word_index == 2


def test_bits_same_pairs_as_tables(tmp_path, monkeypatch):
    # short reads: the bitmap bound decides almost every pair and no queue
    # overflows, so both forms take the same passes (same R sequence) and
    # send the same pairs on (where a queue overflows, a pass is redone with
    # a smaller R and the pair counts, not the clusters, differ)
    data = gsdr.synth_fasta(0, n_reads=3000, seed=44)
    sb, _ = run_form(data, tmp_path, monkeypatch, 0.95, 64, "bits")
    stt, _ = run_form(data, tmp_path, monkeypatch, 0.95, 64, "table")
    assert sb.word_index == 2 and stt.word_index == 0
    assert sb.pairs_prefilter == stt.pairs_prefilter
    assert sb.pairs_word == stt.pairs_word
    assert sb.pairs_aligned == stt.pairs_aligned
    assert sb.cells == stt.cells
