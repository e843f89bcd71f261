"""The GPU path on the named workloads at sizes the oracle takes minutes for:
the whole 200k-read workload, a 200k-read slice of the 2M-read 150 bp
workload and a 3k-read slice of the 2-30 kbp workload, against the oracle's
results recorded in tests/golden/oracle_outputs.json (made by
tests/golden/make_oracle_fixtures.py).  Cluster array, sort permutation and
output FASTA must be identical (integer work: no tolerance), in the batched
and the plain form.  A 20k-read slice of the 2-30 kbp workload, where the
oracle would take hours, checks plain == batched instead."""
import hashlib
import json
import os

import numpy as np
import pytest

import gsdr

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "oracle_outputs.json")) as _f:
    FIXTURES = json.load(_f)


def sha(b):
    return hashlib.sha256(b).hexdigest()


def _input(case):
    fx = FIXTURES[case]
    data = gsdr.synth_fasta(fx["config"], n_reads=fx["reads"], seed=fx["seed"])
    assert sha(data) == fx["input_sha256"], "generator output changed"
    return fx, data


@pytest.mark.parametrize("case", sorted(FIXTURES))
@pytest.mark.parametrize("batch", [0, 1])
def test_matches_oracle_fixture(case, batch):
    fx, data = _input(case)
    f = gsdr.Fasta.parse(data)
    try:
        assert f.n == fx["n"]
        assert sha(np.ascontiguousarray(f.order(), dtype="<i4").tobytes()) == fx["order_sha256"]
        cl, st = gsdr.clustering(f, gsdr.default_opts(threshold=fx["threshold"], batch=batch),
                                 stats=True)
        out = f.format(cl)
    finally:
        f.close()
    assert int((cl == np.arange(len(cl))).sum()) == fx["representatives"]
    assert st.rounds == fx["rounds"]
    assert st.pairs_accepted == fx["accepted"]
    assert sha(np.ascontiguousarray(cl, dtype="<i4").tobytes()) == fx["cluster_sha256"]
    assert sha(out) == fx["output_sha256"]


def test_c3_20k_plain_equals_batched():
    data = gsdr.synth_fasta(3, n_reads=20000, seed=47)
    f = gsdr.Fasta.parse(data)
    try:
        plain, sp = gsdr.clustering(f, gsdr.default_opts(threshold=0.80, batch=1), stats=True)
        batched, sb = gsdr.clustering(f, gsdr.default_opts(threshold=0.80, batch=0), stats=True)
    finally:
        f.close()
    assert sp.drop == 1 and sb.drop == 1
    np.testing.assert_array_equal(batched, plain)
    assert sb.rounds == sp.rounds
    assert sb.cells_computed > 0 and sb.cells_computed <= 2 * sb.cells
