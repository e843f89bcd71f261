"""readFile + clustering + saveFile on the device (gsdr_cluster_fasta): the
FASTA text is parsed on the GPU (the reference's getline rules,
cuda-version/func.cu:94-117), only the lengths go back for the same std::sort
call, and the output records are formatted on the GPU.  The output bytes must
equal the reference's (golden cases) and the host path's, with the same
cluster array and sort permutation."""
import hashlib
import os
import sys

import numpy as np
import pytest

import gsdr

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import cases  # noqa: E402
from test_golden import GOLDEN, case_input  # noqa: E402

pytestmark = pytest.mark.gpu


def host_path(data, **kw):
    f = gsdr.Fasta.parse(data)
    try:
        cl = gsdr.clustering(f, gsdr.default_opts(**kw))
        return f.format(cl), cl, f.order()
    finally:
        f.close()


@pytest.mark.parametrize("batch", [1, 0])
@pytest.mark.parametrize("name", sorted(cases.CASES))
def test_device_parse_reproduces_reference(name, batch):
    data, o = case_input(name)
    out, cl, order = gsdr.cluster_fasta(
        data, threshold=float(o.get("t", 0.95)), word_length=int(o.get("w", 0)),
        drop=int(o.get("d", 3)), pigeon=int(o.get("p", 0)), batch=batch)
    assert hashlib.sha256(out).hexdigest() == GOLDEN[name]["output_sha256"]


@pytest.mark.parametrize("data", [
    b"",                                   # one empty record
    b"\n",
    b">only\n",
    b">a\nACGT",                           # no newline at the end
    b">a\r\nACGTACGT\r\n>b\r\nACGT\r\n",   # CRLF: the '\r' stays in names and data
    b"ACGT\n>b\nAC\n\nGT\n\n>c\n\n",       # first line is a name; empty lines skipped
    b">x\n" + b"ACGTTGCA\n" * 50 + b">y\n" + b"ACGTTGCA" * 50 + b"\n",  # multi-line vs one line
    b">n1\nNNNNACGT\n>n2\nacgtacgu\n>n3\n>n4\nACG\n",
])
def test_device_parse_edge_texts(data):
    out, cl, order = gsdr.cluster_fasta(data, threshold=0.9)
    hout, hcl, horder = host_path(data, threshold=0.9)
    assert out == hout
    np.testing.assert_array_equal(cl, hcl)
    np.testing.assert_array_equal(order, horder)


def test_device_parse_multiline_workload():
    # every record wrapped at 60 columns
    rng = np.random.default_rng(5)
    flat = gsdr.synth_fasta(0, n_reads=3000, seed=71)
    recs = flat.split(b"\n")
    wrapped = []
    for name, seq in zip(recs[0::2], recs[1::2]):
        wrapped.append(name)
        for i in range(0, len(seq), 60):
            wrapped.append(seq[i:i + 60])
    data = b"\n".join(wrapped) + b"\n"
    for batch in (1, 0):
        out, cl, order = gsdr.cluster_fasta(data, threshold=0.95, batch=batch)
        hout, hcl, horder = host_path(data, threshold=0.95, batch=batch)
        assert out == hout
        np.testing.assert_array_equal(cl, hcl)
    del rng


def test_device_parse_c2_slice_ties():
    # all reads 150 bp: the order is std::sort tie-breaking alone
    data = gsdr.synth_fasta(2, n_reads=20000, seed=72)
    out, cl, order, st = gsdr.cluster_fasta(data, threshold=0.90, stats=True)
    hout, hcl, horder = host_path(data, threshold=0.90)
    assert out == hout
    np.testing.assert_array_equal(order, horder)
    assert st.rounds > 0


def test_device_parse_large_ties_match_std_sort(tmp_path):
    # 100k reads of 150 bp (>= 65,536 records: the host sort runs threaded):
    # the order is std::sort's tie-breaking alone, checked against the oracle
    import oracle_binding as orc

    data = gsdr.synth_fasta(2, n_reads=100000, seed=73)
    path = tmp_path / "c2_100k.fa"
    path.write_bytes(data)
    oorder, _, _ = orc.run(str(path), None, t=0.99, d=1, max_rounds=0)
    out, cl, order = gsdr.cluster_fasta(data, threshold=0.90)
    hout, hcl, horder = host_path(data, threshold=0.90)
    np.testing.assert_array_equal(order, oorder)
    np.testing.assert_array_equal(horder, oorder)
    assert out == hout


def test_zero_copy_result_views_outlive_the_call():
    # copy=False: output and arrays are views of the library's result buffers;
    # they stay valid while any of them is referenced
    import gc

    data = gsdr.synth_fasta(0, n_reads=2000, seed=74)
    out, cl, order = gsdr.cluster_fasta(data, threshold=0.95)
    vout, vcl, vorder = gsdr.cluster_fasta(data, threshold=0.95, copy=False)
    del vout, vorder
    gc.collect()
    np.testing.assert_array_equal(vcl, cl)
    vout, _, vorder = gsdr.cluster_fasta(data, threshold=0.95, copy=False)
    gc.collect()
    assert vout.dtype == np.uint8 and vout.tobytes() == out
    np.testing.assert_array_equal(vorder, order)
