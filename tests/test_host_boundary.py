"""Host side of the boundary (no GPU): FASTA reading with the reference's
line rules and std::sort tie order, the writer, and option parsing, each
against the oracle."""
import os

import numpy as np
import pytest

import gsdr
import oracle_binding as orc


def oracle_fasta_roundtrip(data, tmp_path):
    """Oracle output when every read is its own representative (t=0.99 on
    unrelated random reads keeps them all), to compare the writer bytes."""
    order, cl, st, fa = orc.run_bytes(data, tmp_path, t=0.99, d=1)
    return order, cl, fa


def test_tie_order_matches_std_sort(tmp_path):
    rng = np.random.default_rng(0)
    lens = rng.choice([50, 51, 52, 60], size=3000)
    recs = [b">x%d\n" % i + rng.choice(list(b"ACGT"), int(L)).tobytes() + b"\n"
            for i, L in enumerate(lens)]
    data = b"".join(recs)
    path = tmp_path / "ties.fa"
    path.write_bytes(data)
    order, _, _ = orc.run(str(path), None, t=0.99, d=1, max_rounds=0)
    f = gsdr.read_file(str(path))
    np.testing.assert_array_equal(f.order(), order)
    # same permutation as a plain stable sort would NOT give in general
    stable = np.argsort(-lens, kind="stable")
    assert not np.array_equal(stable, order)


@pytest.mark.parametrize("mode", ["two", "few", "lognormal"])
def test_tie_order_matches_std_sort_large(tmp_path, mode):
    # >= 65,536 records: the sort runs on a team of threads (partitions shared
    # by the team, then parts from a stack) and must still give std::sort's
    # permutation
    rng = np.random.default_rng(1)
    n = 120000
    if mode == "two":
        lens = rng.choice([30, 31], size=n)
    elif mode == "few":
        lens = rng.choice([20, 21, 22, 25], size=n)
    else:
        lens = np.clip(rng.lognormal(np.log(60), 0.5, size=n), 12, 300).astype(int)
    base = rng.choice(list(b"ACGT"), int(lens.max())).tobytes()
    data = b"".join(b">x%d\n" % i + base[:L] + b"\n" for i, L in enumerate(lens))
    path = tmp_path / "ties_large.fa"
    path.write_bytes(data)
    order, _, _ = orc.run(str(path), None, t=0.99, d=1, max_rounds=0)
    f = gsdr.read_file(str(path))
    np.testing.assert_array_equal(f.order(), order)


@pytest.mark.parametrize("data", [
    b"",
    b"ACGT\n>a\nAC\n",
    b">a\nAC\r\nGT\r\n>b\r\nA\n",
    b">a\n\n\nACGT\n\n>b\nAAAA",
    b">only",
    b"\n>a\nACGT\n",
    b">a\nAC\nGT\nNN\n>b\nACG\n>c\n",
])
def test_reader_layout_cases(tmp_path, data):
    path = tmp_path / "in.fa"
    path.write_bytes(data)
    order, cl, st = orc.run(str(path), str(tmp_path / "o.fa"), t=0.99, d=1)
    f = gsdr.read_file(str(path))
    np.testing.assert_array_equal(f.order(), order)
    out = f.format(cl)
    assert out == (tmp_path / "o.fa").read_bytes()


def test_missing_file_reads_as_empty(tmp_path):
    f = gsdr.read_file(str(tmp_path / "does_not_exist.fa"))
    assert f.n == 1
    assert f.format(np.array([0], dtype=np.int32)) == b"\n\n"


@pytest.mark.parametrize("argv", [
    ["t", "0.95"], ["t", "0.88"], ["t", "0.879"], ["t", "0.8"], ["t", "0.94"], ["t", "0.97"],
    ["t", "0.9", "w", "9"], ["t", "0.9", "d", "1"], ["t", "0.85", "d", "0"], ["p", "1"],
    ["t", "1.0"], ["t", "0.79"], ["w", "3"], ["w", "13"], ["d", "2"], ["p", "2"], ["x", "1"],
    ["t"], ["i", "a.fa", "o", "b.fa", "t", "0.91"],
])
def test_check_option_matches(argv):
    ref = orc.check_option(argv)
    try:
        o, _, _ = gsdr.check_option(argv)
        got = (o.threshold, o.word_length, o.drop, o.pigeon)
    except gsdr.GsdrError as e:
        assert e.status == gsdr.EINVAL
        got = None
    if ref is None:
        assert got is None
    else:
        assert got is not None
        assert np.float32(got[0]) == np.float32(ref[0]) and got[1:] == ref[1:]


def test_dash_spelling_accepted():
    o, i, out = gsdr.check_option(["-t", "0.9", "--i", "x.fa", "-o", "y.fa"])
    assert abs(o.threshold - 0.9) < 1e-7 and i == "x.fa" and out == "y.fa" and o.word_length == 7


# ---- cluster membership (.clstr) ----------------------------------------------

def _clusters_case(tmp_path):
    data = gsdr.synth_fasta(0, n_reads=400, seed=77)
    _, ocl, _, ofa = orc.run_bytes(data, tmp_path, t=0.95)
    return data, ocl, ofa


def test_clstr_lists_every_read_once(tmp_path):
    data, ocl, ofa = _clusters_case(tmp_path)
    f = gsdr.Fasta.parse(data)
    try:
        text = f.format_clusters(ocl)
        lens = f.lengths()
    finally:
        f.close()
    lines = text.decode().splitlines()
    heads = [l for l in lines if l.startswith(">Cluster ")]
    reps = [l for l in lines if l.endswith("... *")]
    members = [l for l in lines if not l.startswith(">Cluster ")]
    assert len(heads) == len(reps) == int((ocl == np.arange(len(ocl))).sum())
    assert len(members) == len(ocl)
    # representatives in output order: the same names as the FASTA output
    out_names = [l for l in ofa.decode().split("\n") if l.startswith(">")]
    rep_names = [l.split("nt, ", 1)[1][: -len("... *")] for l in reps]
    assert rep_names == out_names
    # lengths are the raw sequence lengths, members of a cluster in sorted order
    assert sorted(int(l.split("\t")[1].split("nt")[0]) for l in members) == sorted(lens.tolist())
    for k, h in enumerate(heads):
        assert h == f">Cluster {k}"


def test_clstr_rejects_unfinished_clustering(tmp_path):
    data, ocl, _ = _clusters_case(tmp_path)
    f = gsdr.Fasta.parse(data)
    try:
        bad = ocl.copy()
        bad[-1] = len(bad) + 5
        with pytest.raises(gsdr.GsdrError):
            f.format_clusters(bad)
        bad = ocl.copy()
        bad[1] = -1
        with pytest.raises(gsdr.GsdrError):
            f.format_clusters(bad)
    finally:
        f.close()


def test_clstr_file_matches_format(tmp_path):
    data, ocl, _ = _clusters_case(tmp_path)
    f = gsdr.Fasta.parse(data)
    try:
        n = gsdr.save_clusters(str(tmp_path / "o.clstr"), f, ocl)
        assert (tmp_path / "o.clstr").read_bytes() == f.format_clusters(ocl)
        assert n == int((ocl == np.arange(len(ocl))).sum())
    finally:
        f.close()


@pytest.mark.parametrize("knobs,ok", [
    (dict(align_blocks=2, filter_blocks=4, graph_steps=8), True),
    (dict(align_blocks=9), False), (dict(filter_blocks=-1), False),
    (dict(graph_steps=3), False), (dict(graph_steps=66), False), (dict(graph_steps=64), True),
])
def test_block_shape_and_staging_depth_ranges(knobs, ok):
    o = gsdr.default_opts(**knobs)
    if ok:
        gsdr.resolve_opts(o)
    else:
        with pytest.raises(gsdr.GsdrError) as e:
            gsdr.resolve_opts(o)
        assert e.value.status == gsdr.EINVAL


def test_word_filter_option_range():
    for bad in (5, -1):
        with pytest.raises(gsdr.GsdrError):
            gsdr.resolve_opts(gsdr.default_opts(word_filter=bad))
    assert gsdr.resolve_opts(gsdr.default_opts(word_filter=2)).word_filter == 2
    assert gsdr.resolve_opts(gsdr.default_opts(word_filter=4)).word_filter == 4


@pytest.mark.parametrize("kw", [{"group_words": 129}, {"group_words": -2},
                                {"band_serial": -2}])
def test_band_tile_option_range(kw):
    with pytest.raises(gsdr.GsdrError) as e:
        gsdr.resolve_opts(gsdr.default_opts(**kw))
    assert e.value.status == gsdr.EINVAL


def test_band_tile_options_default_to_automatic():
    o = gsdr.resolve_opts(gsdr.default_opts(group_words=-1, band_serial=4096))
    assert (o.group_words, o.band_serial) == (-1, 4096)
    d = gsdr.default_opts()
    assert (d.group_words, d.band_serial) == (0, 0)


# ---- variant 1: the SYCL program's option rules (func.cpp:6-56) ---------------

@pytest.mark.parametrize("argv", [
    ["t", "0.95"], ["t", "0.88"], ["t", "0.879"], ["t", "0.8"], ["t", "0.94"], ["t", "0.97"],
    ["t", "0.93"], ["t", "0.9", "w", "8"], ["t", "0.9", "w", "9"], ["w", "3"], ["t", "1.0"],
    ["t", "0.9", "d", "1"], ["t", "0.9", "d", "0"], ["p", "0"], ["i", "a.fa", "t", "0.91"],
])
def test_check_option_sycl_matches(argv):
    ref = orc.check_option_sycl(argv)
    try:
        o, _, _ = gsdr.check_option(argv + ["v", "1"])
        got = (o.threshold, o.word_length)
        assert o.variant == 1 and o.drop == 0 and o.pigeon == 0
    except gsdr.GsdrError as e:
        assert e.status == gsdr.EINVAL
        got = None
    if ref is None:
        assert got is None
    else:
        assert got is not None
        assert np.float32(got[0]) == np.float32(ref[0]) and got[1] == ref[1]


def test_sycl_cutoffs_are_float_formulas():
    # func.cpp:339-373 in float32 arithmetic, offset 1; and the cuda-version
    # formulas differ from them (double, the 1.1 - |t - 0.95| * 2 offset)
    lens = np.arange(1, 20001, 7, dtype=np.int32)
    for t in (0.8, 0.85, 0.9, 0.93, 0.95, 0.97, 0.99):
        for k in (4, 5, 6, 7, 8):
            w, b = orc.cutoffs_sycl(lens, t, k)
            tf = np.float32(t)
            slack = np.ceil(lens.astype(np.float32) * (np.float32(1) - tf))
            req = lens - k + 1 - (slack * np.float32(k)).astype(np.int32)
            np.testing.assert_array_equal(w, np.maximum(req, 1))
            np.testing.assert_array_equal(b, np.ceil(lens.astype(np.float32) * tf).astype(np.int32))
    w0, _, _ = orc.cutoffs(lens, 0.95, 6)
    w1, _ = orc.cutoffs_sycl(lens, 0.95, 6)
    assert (w0 != w1).any()


def test_sycl_kmers_skip_windows_over_non_acgt():
    seq = b"ACGTNACGTACGTRRACG"
    w, c = orc.kmers_raw(seq, 4)
    # windows of 4 raw bytes without N/R: ACGT; ACGT CGTA GTAC TACG ACGT; (none after RR but ACG is 3)
    words = {}
    codes = {ord("A"): 0, ord("C"): 1, ord("G"): 2, ord("T"): 3}
    for i in range(3, len(seq)):
        win = seq[i - 3:i + 1]
        if all(ch in codes for ch in win):
            v = sum(codes[win[3 - j]] << (2 * j) for j in range(4))
            words[v] = words.get(v, 0) + 1
    assert dict(zip(w.tolist(), c.tolist())) == words
    assert sum(c) == 6


def test_fasta_input_buffers():
    # gsdr_cluster_fasta takes the FASTA bytes from bytes or from a contiguous
    # uint8 array (for example a view of pinned host memory)
    data = b">a\nACGT\n"
    p1, n1 = gsdr._host_bytes(data)
    arr = np.frombuffer(data, dtype=np.uint8).copy()
    p2, n2 = gsdr._host_bytes(arr)
    assert n1 == n2 == len(data)
    assert p2.value == arr.ctypes.data
    for bad in (np.zeros(4, dtype=np.int32), np.zeros((2, 2), dtype=np.uint8),
                np.zeros(8, dtype=np.uint8)[::2]):
        with pytest.raises(TypeError):
            gsdr._host_bytes(bad)


def test_tuned_opts_carry_every_setting():
    from gsdr.autotune import KNOBS, tuned_opts

    best = {"batch": 512, "word_filter": 2, "group_words": 64, "band_serial": 4096,
            "align_blocks": 2, "filter_blocks": 4, "graph_steps": 8, "stage": "staging depth"}
    o = tuned_opts({"best": best}, 0.9)
    assert all(getattr(o, k) == best[k] for k in KNOBS)
    assert abs(o.threshold - 0.9) < 1e-6
    gsdr.resolve_opts(o)
