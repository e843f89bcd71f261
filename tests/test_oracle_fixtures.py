"""The inputs of the oracle fixtures (tests/golden/oracle_outputs.json) are
rebuilt byte for byte by the workload generator on this machine, so the GPU
tests that compare against those fixtures compare like with like."""
import hashlib
import json
import os

import pytest

import gsdr

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "oracle_outputs.json")) as _f:
    FIXTURES = json.load(_f)


@pytest.mark.parametrize("case", sorted(FIXTURES))
def test_fixture_input_is_reproducible(case):
    fx = FIXTURES[case]
    data = gsdr.synth_fasta(fx["config"], n_reads=fx["reads"], seed=fx["seed"])
    assert len(data) == fx["input_bytes"]
    assert hashlib.sha256(data).hexdigest() == fx["input_sha256"]
    assert 0 < fx["representatives"] <= fx["n"]
