"""Batched form (R tentative representatives per pass, greedy conflict
resolution) against the oracle: identical cluster arrays and FASTA bytes for
every R, since each pair decision is a pure function of the pair."""
import numpy as np
import pytest

import gsdr
import oracle_binding as orc

pytestmark = pytest.mark.gpu


def run_batched(data, tmp_path, t, batch, d=3):
    _, ocl, ost, ofa = orc.run_bytes(data, tmp_path, t=t, d=d)
    f = gsdr.Fasta.parse(data)
    cl, st = gsdr.clustering(f, gsdr.default_opts(threshold=t, drop=d, batch=batch), stats=True)
    out = f.format(cl)
    f.close()
    bad = np.nonzero(cl != ocl)[0]
    assert len(bad) == 0, f"R={batch}: {len(bad)} reads differ, first {bad[:8]}"
    assert out == ofa
    assert st.rounds == ost.rounds
    assert st.pairs_accepted == ost.accepted
    return st


@pytest.mark.parametrize("batch", [1, 2, 8, 64, 256, 0])
def test_c0_recipe_batched(tmp_path, batch):
    data = gsdr.synth_fasta(0, n_reads=3000, seed=12)
    st = run_batched(data, tmp_path, 0.95, batch)
    if batch not in (1,):
        assert st.passes <= st.rounds


@pytest.mark.parametrize("batch", [4, 1024])
def test_c1_recipe_batched(tmp_path, batch):
    data = gsdr.synth_fasta(1, n_reads=20000, seed=22)
    run_batched(data, tmp_path, 0.95, batch)


@pytest.mark.parametrize("t,batch", [(0.90, 64), (0.97, 16), (0.88, 32)])
def test_thresholds_batched(tmp_path, t, batch):
    data = gsdr.synth_fasta(0, n_reads=2000, seed=13)
    run_batched(data, tmp_path, t, batch)


@pytest.mark.parametrize("batch", [8, 128])
def test_drop_mode_batched(tmp_path, batch):
    data = gsdr.synth_fasta(0, n_reads=700, seed=14)
    run_batched(data, tmp_path, 0.85, batch)


def test_c2_recipe_batched(tmp_path):
    data = gsdr.synth_fasta(2, n_reads=30000, seed=32)
    run_batched(data, tmp_path, 0.90, 256)


def test_c3_recipe_batched_drop(tmp_path):
    data = gsdr.synth_fasta(3, n_reads=120, seed=42)
    run_batched(data, tmp_path, 0.80, 32)


def test_duplicates_all_ties_batched(tmp_path):
    # many identical reads: every tentative after the first is absorbed in-pass
    seq = b"ACGTTGCAAC" * 30
    data = b"".join(b">d%d\n%s\n" % (i, seq) for i in range(200))
    run_batched(data, tmp_path, 0.95, 64)
