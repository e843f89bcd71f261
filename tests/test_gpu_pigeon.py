"""The pigeon filter (`p 1`, kernel_createPigeon1/2 and kernel_pigeon,
cuda-version/func.cu:188-270, 756-801) on the GPU against the oracle: the
same cluster arrays, FASTA bytes and pairs reaching the alignment, in the
plain and the batched form.  The reference binary's own outputs for `p 1`
are golden cases of tests/test_golden.py."""
import numpy as np
import pytest

import gsdr
import oracle_binding as orc
from test_gpu_parity import _mixed_edge_fasta, assert_same, run_both

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("batch", [1, 64, 0])
@pytest.mark.parametrize("t", [0.88, 0.90, 0.95, 0.97])
def test_pigeon_c0_recipe(tmp_path, t, batch):
    data = gsdr.synth_fasta(0, n_reads=2000, seed=61)
    cl, ocl, out, ofa, st, ost = run_both(data, tmp_path, t=t, p=1, batch=batch)
    assert ost.pigeon == 1
    assert_same(cl, ocl, out, ofa)
    assert st.pairs_accepted == ost.accepted
    if batch == 1:
        assert st.pairs_aligned == ost.aligned


@pytest.mark.parametrize("batch", [1, 0])
def test_pigeon_long_reads(tmp_path, batch):
    data = gsdr.synth_fasta(4, n_reads=1500, seed=62, n_seeds=300, len_lo=150, len_hi=5000)
    cl, ocl, out, ofa, st, ost = run_both(data, tmp_path, t=0.93, p=1, batch=batch)
    assert_same(cl, ocl, out, ofa)


@pytest.mark.parametrize("t", [0.95, 0.90])
def test_pigeon_edge_symbols(tmp_path, t):
    # N / IUPAC / lower case / \r: 4-mer windows holding a non-ACGT code are
    # skipped by the position index
    data = _mixed_edge_fasta(17)
    for batch in (1, 0):
        cl, ocl, out, ofa, st, ost = run_both(data, tmp_path, t=t, p=1, batch=batch)
        assert_same(cl, ocl, out, ofa)


def test_pigeon_filter_is_active(tmp_path):
    # on this input the pigeon stage removes pairs in the oracle (its count
    # of pairs passing it is below the composition bound's), and the GPU
    # sends exactly the oracle's pairs to the alignment
    data = gsdr.synth_fasta(4, n_reads=1500, seed=63, n_seeds=300, len_lo=150, len_hi=5000)
    cl, ocl, out, ofa, st, ost = run_both(data, tmp_path, t=0.93, p=1, batch=1)
    assert ost.pigeon_pass < ost.prefilter_pass
    assert_same(cl, ocl, out, ofa)
    assert st.pairs_aligned == ost.aligned
