"""Batched word filter forms against the oracle: the per-k-mer tentative
masks (chosen for short reads holding few of the 4^k k-mers, e.g. 150 bp
reads at k = 7), the per-pass inverted k-mer index, the two-level k-mer count
bitmaps (k <= 7 otherwise) and the per-tentative tables.  Identical cluster
arrays and FASTA bytes in every form, at every R, every word length, and for
reads too short to hold a k-mer (the reference's kernel_filter,
cuda-version/func.cu:803-826)."""
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
def test_c2_recipe_masks_auto(tmp_path, monkeypatch, batch):
    data = gsdr.synth_fasta(2, n_reads=30000, seed=33)
    st, ost = run_form(data, tmp_path, monkeypatch, 0.90, batch, None)
    assert st.k == 7 and st.word_index == 3
    # the pairs sent to the alignment are the pairs passing both filters
    assert st.passes < st.rounds


@pytest.mark.parametrize("batch", [2, 64, 256, 1024])
def test_c2_recipe_index_forced(tmp_path, monkeypatch, batch):
    data = gsdr.synth_fasta(2, n_reads=30000, seed=33)
    st, ost = run_form(data, tmp_path, monkeypatch, 0.90, batch, "index")
    assert st.k == 7 and st.word_index == 1


def test_c2_recipe_same_pairs_every_form(tmp_path, monkeypatch):
    data = gsdr.synth_fasta(2, n_reads=20000, seed=34)
    si, _ = run_form(data, tmp_path, monkeypatch, 0.90, 128, "index")
    stt, _ = run_form(data, tmp_path, monkeypatch, 0.90, 128, "table")
    sm, _ = run_form(data, tmp_path, monkeypatch, 0.90, 128, "masks")
    assert si.word_index == 1 and stt.word_index == 0 and sm.word_index == 3
    for s in (si, sm):
        assert s.pairs_prefilter == stt.pairs_prefilter
        assert s.pairs_aligned == stt.pairs_aligned
        assert s.cells == stt.cells


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


@pytest.mark.parametrize("form", ["index", "table", "masks"])
def test_very_short_reads(tmp_path, monkeypatch, form):
    # 3-48 bp reads at k = 7: reads of at most 6 bases hold no k-mer, and the
    # word cutoff is never below 1 (func.cu:312-337), so they are never aligned
    data = gsdr.synth_fasta(0, n_reads=3000, seed=38, len_lo=3, len_hi=40, n_seeds=400)
    lens = np.array([len(l) for l in data.split(b"\n")[1::2]])
    cw, _, _ = orc.cutoffs(lens, 0.90, 7)
    assert (lens <= 6).any() and (cw >= 1).all()
    st, _ = run_form(data, tmp_path, monkeypatch, 0.90, 64, form, w=7)
    assert st.word_index == {"index": 1, "table": 0, "masks": 3}[form]


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


# ---- per-k-mer tentative masks: D1 <= S <= D1 + min(excess), bit-sliced
# counts, exact sums for the pairs the bound leaves open

# R values that take each row width: 1, 2, 4 and 8 lanes per row of
# 16-byte words, with partly used words (100, 129, 300, 513)
@pytest.mark.parametrize("batch", [2, 100, 129, 300, 513, 1024])
def test_masks_row_widths(tmp_path, monkeypatch, batch):
    data = gsdr.synth_fasta(2, n_reads=12000, seed=46)
    st, _ = run_form(data, tmp_path, monkeypatch, 0.90, batch, "masks")
    assert st.k == 7 and st.word_index == 3


@pytest.mark.parametrize("w", [4, 5, 6, 7])
def test_masks_word_lengths_ragged_reads(tmp_path, monkeypatch, w):
    # 20-240 bp seeds (copies with insertions run a few bases longer): below
    # 256 k-mer entries per read at k = 4
    data = gsdr.synth_fasta(0, n_reads=2500, seed=47, len_lo=20, len_hi=240, n_seeds=500)
    st, _ = run_form(data, tmp_path, monkeypatch, 0.95, 256, "masks", w=w)
    assert st.k == w and st.word_index == 3


@pytest.mark.parametrize("t", [0.88, 0.90, 0.93, 0.97])
def test_masks_thresholds(tmp_path, monkeypatch, t):
    data = gsdr.synth_fasta(0, n_reads=2500, seed=48, len_lo=60, len_hi=240, n_seeds=400)
    st, ost = run_form(data, tmp_path, monkeypatch, t, 0, "masks")
    assert st.k == ost.k
    if st.k <= 7:
        assert st.word_index == 3


def repeat_reads(rng, n_seeds=120, copies=12):
    """Low-complexity reads (tandem repeats of 1-12 bp units, 80-250 bp) and
    their copies with a few substitutions and indels: k-mer counts well above
    one, so the mask bound leaves pairs open for the exact sums."""
    recs = []
    for s in range(n_seeds):
        unit = rng.choice(list(b"ACGT"), size=int(rng.integers(1, 13))).astype(np.uint8)
        L = int(rng.integers(80, 251))
        seed = np.resize(unit, L)
        if s % 3 == 0:  # a random stretch inside the repeat
            a = int(rng.integers(0, L // 2))
            seed[a:a + L // 4] = rng.choice(list(b"ACGT"), size=len(seed[a:a + L // 4]))
        for c in range(copies):
            r = seed.copy()
            for _ in range(int(rng.integers(0, 6))):
                p = int(rng.integers(0, len(r)))
                op = int(rng.integers(0, 3))
                if op == 0:
                    r[p] = rng.choice(list(b"ACGT"))
                elif op == 1 and len(r) > 40:
                    r = np.delete(r, p)
                else:
                    r = np.insert(r, p, rng.choice(list(b"ACGT")))
            recs.append(bytes(r[:255]))
    order = rng.permutation(len(recs))
    return b"".join(b">r%d\n%s\n" % (i, recs[j]) for i, j in enumerate(order))


@pytest.mark.parametrize("t,batch", [(0.90, 64), (0.90, 0), (0.95, 512), (0.88, 1024)])
def test_masks_low_complexity_open_pairs(tmp_path, monkeypatch, t, batch):
    data = repeat_reads(np.random.default_rng(49))
    st, _ = run_form(data, tmp_path, monkeypatch, t, batch, "masks")
    assert st.word_index == 3


def test_masks_fall_back_for_long_reads(tmp_path, monkeypatch):
    # reads above 1,023 k-mers: the counts would not fit the masks' ten
    # planes, so the forced form falls back to the automatic one
    data = gsdr.synth_fasta(1, n_reads=1500, seed=50)
    st, _ = run_form(data, tmp_path, monkeypatch, 0.95, 64, "masks")
    assert st.word_index != 3


@pytest.mark.parametrize("w,batch", [(6, 64), (6, 1024), (7, 300), (5, 0)])
def test_masks_ten_planes(tmp_path, monkeypatch, w, batch):
    # 200-1000 bp reads: up to ~1,000 k-mer entries, counts in ten planes
    data = gsdr.synth_fasta(0, n_reads=2500, seed=51)
    st, _ = run_form(data, tmp_path, monkeypatch, 0.95, batch, "masks", w=w)
    assert st.k == w and st.word_index == 3


def test_masks_form_is_repeatable(monkeypatch):
    monkeypatch.delenv("GSDR_BFILTER", raising=False)
    data = gsdr.synth_fasta(2, n_reads=20000, seed=39)
    f = gsdr.Fasta.parse(data)
    job = gsdr.Job(f, gsdr.default_opts(threshold=0.90, batch=0))
    try:
        assert job.run().word_index == 3
        a = job.cluster()
        job.run()
        b = job.cluster()
    finally:
        job.close()
        f.close()
    assert np.array_equal(a, b)
