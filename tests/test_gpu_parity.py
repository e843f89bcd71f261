"""GPU path vs the oracle: cluster arrays and FASTA bytes must be identical.

All cases are integer work, so the tolerance is zero.  Inputs are seeded
synthetic workloads (the reference's own input file is not distributed) and
hand-made edge cases.
"""
import numpy as np
import pytest

import gsdr
import oracle_binding as orc

pytestmark = pytest.mark.gpu


def run_both(data: bytes, tmp_path, t=0.95, w=0, d=3, p=0, batch=1):
    order, ocl, ost, ofa = orc.run_bytes(data, tmp_path, t=t, w=w, d=d, p=p)
    f = gsdr.Fasta.parse(data)
    assert f.n == len(ocl)
    np.testing.assert_array_equal(f.order(), order)
    cl, st = gsdr.clustering(f, gsdr.default_opts(threshold=t, word_length=w, drop=d, pigeon=p,
                                                  batch=batch), stats=True)
    out = f.format(cl)
    f.close()
    return cl, ocl, out, ofa, st, ost


def assert_same(cl, ocl, out, ofa):
    bad = np.nonzero(cl != ocl)[0]
    assert len(bad) == 0, f"{len(bad)} reads differ, first {bad[:10]}: gpu {cl[bad[:10]]} oracle {ocl[bad[:10]]}"
    assert out == ofa


@pytest.mark.parametrize("n,seed", [(600, 1), (3000, 2)])
def test_c0_recipe(tmp_path, n, seed):
    data = gsdr.synth_fasta(0, n_reads=n, seed=seed)
    cl, ocl, out, ofa, st, ost = run_both(data, tmp_path, t=0.95)
    assert_same(cl, ocl, out, ofa)
    assert st.rounds == ost.rounds
    assert st.pairs_accepted == ost.accepted


def test_c0_full(tmp_path):
    data = gsdr.synth_fasta(0)
    cl, ocl, out, ofa, st, ost = run_both(data, tmp_path, t=0.95)
    assert_same(cl, ocl, out, ofa)
    assert st.pairs_word == ost.prefilter_pass
    assert st.pairs_aligned == ost.aligned


@pytest.mark.parametrize("t", [0.88, 0.90, 0.93, 0.97, 0.99])
def test_thresholds_word_lengths(tmp_path, t):
    data = gsdr.synth_fasta(0, n_reads=2000, seed=11)
    cl, ocl, out, ofa, st, ost = run_both(data, tmp_path, t=t)
    assert st.k == ost.k
    assert_same(cl, ocl, out, ofa)


@pytest.mark.parametrize("w", [4, 5, 6, 7, 8, 9, 10, 11, 12])
def test_word_length_override(tmp_path, w):
    data = gsdr.synth_fasta(0, n_reads=1500, seed=5)
    cl, ocl, out, ofa, st, ost = run_both(data, tmp_path, t=0.95, w=w)
    assert_same(cl, ocl, out, ofa)
    assert st.k == w
    assert st.pairs_word == ost.prefilter_pass
    assert st.pairs_aligned == ost.aligned


@pytest.mark.parametrize("w,t,p", [(8, 0.90, 0), (9, 0.95, 1), (12, 0.97, 0)])
def test_long_word_lengths_long_reads(tmp_path, w, t, p):
    # reads of a few thousand bases: the k-mer hash of a read takes more than
    # its smallest table; a batched request runs one representative per round
    data = gsdr.synth_fasta(1, n_reads=400, seed=21)
    cl, ocl, out, ofa, st, ost = run_both(data, tmp_path, t=t, w=w, p=p, batch=0)
    assert_same(cl, ocl, out, ofa)
    assert st.batch == 1
    assert st.pairs_word == ost.prefilter_pass


@pytest.mark.parametrize("t", [0.80, 0.85])
def test_drop_mode(tmp_path, t):
    data = gsdr.synth_fasta(0, n_reads=700, seed=3)
    cl, ocl, out, ofa, st, ost = run_both(data, tmp_path, t=t)
    assert ost.drop == 1 and st.drop == 1
    assert_same(cl, ocl, out, ofa)


def test_drop_forced_at_high_t(tmp_path):
    data = gsdr.synth_fasta(0, n_reads=600, seed=4)
    cl, ocl, out, ofa, st, ost = run_both(data, tmp_path, t=0.95, d=1)
    assert_same(cl, ocl, out, ofa)


def test_c1_recipe_slice(tmp_path):
    data = gsdr.synth_fasta(1, n_reads=20000, seed=21)
    cl, ocl, out, ofa, st, ost = run_both(data, tmp_path, t=0.95)
    assert_same(cl, ocl, out, ofa)
    assert st.cells == ost.cells


def test_c2_recipe_slice(tmp_path):
    # all reads 150 bp: the order is pure std::sort tie-breaking
    data = gsdr.synth_fasta(2, n_reads=30000, seed=31)
    cl, ocl, out, ofa, st, ost = run_both(data, tmp_path, t=0.90)
    assert_same(cl, ocl, out, ofa)


@pytest.mark.parametrize("cfg,n,t", [(2, 6000, 0.90), (0, 3000, 0.85), (1, 3000, 0.95)])
@pytest.mark.parametrize("group_words,band_serial", [(-1, -1), (8, 1 << 30), (32, 4096),
                                                     (128, 65536)])
def test_band_tiles_same_clusters(tmp_path, cfg, n, t, group_words, band_serial):
    # the band tiles only move pairs between alignment kernels
    data = gsdr.synth_fasta(cfg, n_reads=n, seed=51 + cfg)
    _, ocl, _, _ = orc.run_bytes(data, tmp_path, t=t)
    f = gsdr.Fasta.parse(data)
    try:
        cl = gsdr.clustering(f, gsdr.default_opts(threshold=t, group_words=group_words,
                                                  band_serial=band_serial))
    finally:
        f.close()
    np.testing.assert_array_equal(cl, ocl)


def test_c3_recipe_slice_drop(tmp_path):
    data = gsdr.synth_fasta(3, n_reads=120, seed=41)
    cl, ocl, out, ofa, st, ost = run_both(data, tmp_path, t=0.80)
    assert_same(cl, ocl, out, ofa)


def _mixed_edge_fasta(seed=9):
    rng = np.random.default_rng(seed)
    recs = []
    base = np.frombuffer(b"ACGT", dtype=np.uint8)[rng.integers(0, 4, 700)].tobytes()
    for i in range(60):
        s = bytearray(base[: rng.integers(150, 700)])
        for _ in range(rng.integers(0, 12)):
            s[rng.integers(0, len(s))] = int(rng.choice(list(b"ACGTNRYacgtnu")))
        if i % 7 == 0:
            s += b"\r"
        recs.append(b">r%d desc\n" % i + bytes(s) + b"\n")
    recs.append(b">short1\nACG\n")
    recs.append(b">short2\nACGTA\n")
    recs.append(b">multiline\n" + base[:100] + b"\n" + base[100:300] + b"\n\n" + base[300:400] + b"\n")
    recs.append(b">dup1\n" + base[:500] + b"\n")
    recs.append(b">dup2\n" + base[:500] + b"\n")
    return b"".join(recs)


@pytest.mark.parametrize("t", [0.95, 0.90, 0.85])
def test_edge_symbols_and_layout(tmp_path, t):
    data = _mixed_edge_fasta()
    cl, ocl, out, ofa, st, ost = run_both(data, tmp_path, t=t)
    assert_same(cl, ocl, out, ofa)


def test_all_n_read_drop_mode(tmp_path):
    data = b">a\n" + b"ACGT" * 50 + b"\n>n\n" + b"N" * 300 + b"\n>b\n" + b"ACGT" * 40 + b"\n>e\n\n"
    cl, ocl, out, ofa, st, ost = run_both(data, tmp_path, t=0.85)
    assert_same(cl, ocl, out, ofa)


def test_single_read_and_no_newline(tmp_path):
    data = b">only\nACGTACGTAC"
    cl, ocl, out, ofa, st, ost = run_both(data, tmp_path, t=0.95)
    assert_same(cl, ocl, out, ofa)
    assert out == b">only\nACGTACGTAC\n"


@pytest.mark.parametrize("batch", [1, 0])
def test_reads_above_32k_bases(tmp_path, batch):
    # 33-65 kbp reads: patterns of the 8-warp x 8-word class (up to 65,536 bases)
    rng = np.random.default_rng(91)
    codes = np.frombuffer(b"ACGT", dtype=np.uint8)
    recs = []
    for s in range(3):
        base = codes[rng.integers(0, 4, 65000)].tobytes()
        for c in range(4):
            L = int(rng.integers(33000, 65000))
            seq = bytearray(base[:L])
            for _ in range(int(rng.integers(0, L // 40))):
                seq[int(rng.integers(0, L))] = int(codes[rng.integers(0, 4)])
            recs.append(b">s%d_%d\n" % (s, c) + bytes(seq) + b"\n")
    data = b"".join(recs)
    cl, ocl, out, ofa, st, ost = run_both(data, tmp_path, t=0.95, batch=batch)
    assert_same(cl, ocl, out, ofa)
    assert st.pairs_accepted == ost.accepted


@pytest.mark.parametrize("batch", [1, 0])
def test_reads_above_65536_bases(tmp_path, batch):
    """Patterns above one systolic group's 65,536 rows run in chunks
    (k_align_long): near copies of a 140 kbp read and of a 70 kbp one, with
    the 140 kbp read's halves and some unrelated long reads."""
    rng = np.random.default_rng(17)
    codes = np.frombuffer(b"ACGT", dtype=np.uint8)
    recs = []
    for s, L in enumerate((140000, 70000, 66000)):
        base = bytearray(codes[rng.integers(0, 4, L)].tobytes())
        for c in range(3):
            seq = bytearray(base)
            for _ in range(int(rng.integers(0, L // 40))):
                seq[int(rng.integers(0, len(seq)))] = int(codes[rng.integers(0, 4)])
            for _ in range(int(rng.integers(0, 30))):
                p = int(rng.integers(0, len(seq)))
                if rng.random() < 0.5:
                    del seq[p]
                else:
                    seq.insert(p, int(codes[rng.integers(0, 4)]))
            recs.append(b">L%d_%d\n" % (s, c) + bytes(seq) + b"\n")
        if s == 0:
            recs.append(b">half\n" + bytes(base[:69000]) + b"\n")
    data = b"".join(recs)
    for t in (0.90, 0.97):
        cl, ocl, out, ofa, st, ost = run_both(data, tmp_path, t=t, batch=batch)
        assert_same(cl, ocl, out, ofa)
        assert st.pairs_accepted == ost.accepted
        assert st.batch == 1  # reads with 65,536+ k-mers: one representative per round
    # drop mode keeps the batched form (no word filter)
    cl, ocl, out, ofa, st, ost = run_both(data, tmp_path, t=0.85, batch=batch)
    assert_same(cl, ocl, out, ofa)


def test_reads_above_the_length_limit_are_refused():
    data = b">a\n" + b"ACGT" * (1 << 22) + b"A\n>b\nACGT\n"
    f = gsdr.Fasta.parse(data)
    try:
        with pytest.raises(gsdr.GsdrError) as e:
            gsdr.clustering(f, gsdr.default_opts(threshold=0.95))
        assert e.value.status == gsdr.EUNSUPPORTED
    finally:
        f.close()


# ---- variant 1: the SYCL program's semantics (func.cpp) --------------------

def run_both_sycl(data: bytes, tmp_path, t=0.95, w=0, batch=1):
    order, ocl, ost, ofa = orc.run_bytes(data, tmp_path, t=t, w=w, variant=1)
    f = gsdr.Fasta.parse(data)
    np.testing.assert_array_equal(f.order(), order)
    cl, st = gsdr.clustering(f, gsdr.default_opts(threshold=t, word_length=w, variant=1,
                                                  batch=batch), stats=True)
    out = f.format(cl)
    f.close()
    return cl, ocl, out, ofa, st, ost


def n_rich_fasta(seed, n_seeds=150, copies=6):
    """Seeds with near copies that carry non-ACGT bytes (single N, N runs,
    IUPAC letters, lower case): k-mer windows over such bytes are where the
    two programs' k-mer rules differ."""
    rng = np.random.default_rng(seed)
    codes = np.frombuffer(b"ACGT", dtype=np.uint8)
    recs = []
    for s in range(n_seeds):
        L = int(rng.integers(200, 1500))
        seed_seq = codes[rng.integers(0, 4, L)]
        for c in range(copies):
            seq = bytearray(seed_seq.tobytes())
            for _ in range(int(rng.integers(0, L // 60 + 1))):
                seq[int(rng.integers(0, L))] = int(codes[rng.integers(0, 4)])
            for _ in range(int(rng.integers(0, 4))):
                p = int(rng.integers(0, len(seq)))
                run = int(rng.integers(1, 4))
                seq[p:p + run] = bytes(rng.choice(list(b"NNNNRYSWKMn"), run))
            if rng.random() < 0.2:
                seq = seq.lower()
            recs.append(b">v%d_%d\n" % (s, c) + bytes(seq) + b"\n")
    order = rng.permutation(len(recs))
    return b"".join(recs[i] for i in order)


@pytest.mark.parametrize("batch", [1, 0])
@pytest.mark.parametrize("t", [0.80, 0.85, 0.90, 0.95, 0.97])
def test_sycl_variant_thresholds(tmp_path, t, batch):
    data = gsdr.synth_fasta(0, n_reads=2000, seed=61)
    cl, ocl, out, ofa, st, ost = run_both_sycl(data, tmp_path, t=t, batch=batch)
    assert st.k == ost.k and st.drop == 0
    assert_same(cl, ocl, out, ofa)
    if batch == 1:
        assert st.pairs_word == ost.prefilter_pass
        assert st.pairs_aligned == ost.word_pass
        assert st.pairs_accepted == ost.accepted


@pytest.mark.parametrize("w", [4, 5, 6, 7, 8])
def test_sycl_variant_word_lengths(tmp_path, w):
    data = n_rich_fasta(70 + w)
    cl, ocl, out, ofa, st, ost = run_both_sycl(data, tmp_path, t=0.93, w=w)
    assert_same(cl, ocl, out, ofa)
    assert st.pairs_word == ost.prefilter_pass
    assert st.pairs_aligned == ost.word_pass


@pytest.mark.parametrize("batch", [1, 0])
@pytest.mark.parametrize("t", [0.90, 0.95, 0.97])
def test_sycl_variant_n_rich(tmp_path, t, batch):
    data = n_rich_fasta(int(t * 100))
    cl, ocl, out, ofa, st, ost = run_both_sycl(data, tmp_path, t=t, batch=batch)
    assert_same(cl, ocl, out, ofa)
    if batch == 1:
        assert st.pairs_aligned == ost.word_pass


def test_sycl_variant_differs_from_cuda_version(tmp_path):
    # the same input clusters differently under the two programs' rules
    data = n_rich_fasta(5)
    cl1, ocl1, *_ = run_both_sycl(data, tmp_path, t=0.95)
    cl0, ocl0, *_ = run_both(data, tmp_path, t=0.95)
    assert (ocl0 != ocl1).any()
    np.testing.assert_array_equal(cl0, ocl0)
    np.testing.assert_array_equal(cl1, ocl1)
