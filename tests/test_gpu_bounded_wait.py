"""A device-side wait that runs out ends in a status, not a hang.

The multi-warp alignment kernels hand carry words from warp to warp through
shared memory; each wait for a neighbour is bounded (gsdr_set_spin_limit,
include/gsdr_testing.h).  With the limit at 0 polls every such wait gives up
at once: the kernel sets its error flag and returns, the call reports
GSDR_ETIMEOUT, and the context stays usable -- the next call with the default
limit decides the same pairs exactly as the oracle does.  The reference has no
device-side waits; it reads errors once at the end (checkError,
cuda-version/func.cu:1118-1123).  Nothing here can hang: lowering the limit
only shortens waits that are bounded already."""
import numpy as np
import pytest

import gsdr
import oracle_binding as orc

pytestmark = pytest.mark.gpu

CODES = np.frombuffer(b"ACGT", dtype=np.uint8)


def _pairs(rng, n, qlen, tlen):
    """Half mutated copies (accepted at t = 0.9), half unrelated pairs of
    similar length (rejected: a random pattern only embeds in a text several
    times longer)."""
    seqs, pairs = [], []
    for i in range(n):
        T = int(rng.integers(*tlen))
        q = int(rng.integers(*qlen))
        b = CODES[rng.integers(0, 4, T)].tobytes()
        if i % 2 == 0:
            a = np.frombuffer(b[:q], dtype=np.uint8).copy()
            hit = rng.random(q) < 0.03
            a[hit] = CODES[rng.integers(0, 4, int(hit.sum()))]
            a = a.tobytes()
        else:
            a = CODES[rng.integers(0, 4, q)].tobytes()
        seqs += [b, a]
        pairs.append((len(seqs) - 1, len(seqs) - 2))
    return seqs, pairs


# mapping 0 (the plain form's grouping): 3-4 kbp patterns need 2 warps of
# 2 words per lane; mapping 1 (the batched form's): 9-12 kbp patterns need
# 2 warps of 8 words per lane
@pytest.mark.parametrize("mapping,qlen,tlen", [(0, (3000, 4000), (4000, 4600)),
                                               (1, (9000, 12000), (12000, 13500))])
def test_wait_that_runs_out_reports_timeout(mapping, qlen, tlen):
    rng = np.random.default_rng(17 + mapping)
    seqs, pairs = _pairs(rng, 16, qlen, tlen)
    t = 0.90
    want = orc.lcs_decisions(seqs, pairs, t)
    assert 0 < want.sum() < len(pairs)
    try:
        gsdr.set_spin_limit(0)
        with pytest.raises(gsdr.GsdrError) as e:
            gsdr.lcs_decide(seqs, pairs, t, mapping=mapping, greedy=0)
        assert e.value.status == gsdr.ETIMEOUT
    finally:
        gsdr.set_spin_limit(None)
    got, _ = gsdr.lcs_decide(seqs, pairs, t, mapping=mapping, greedy=0)
    np.testing.assert_array_equal(got, want)
