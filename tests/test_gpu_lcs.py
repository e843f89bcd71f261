"""Alignment kernels alone against the oracle's LCS: the decision
LCS(pattern, text) >= ceil(len(pattern) * t) (kernel_align,
cuda-version/func.cu:828-999) for random, mutated and repetitive pairs in
every length class, with both warp groupings, with the banded one-pair-per-lane
kernel (mapping 2), the group-banded kernel (mapping 3) and with the greedy
bound."""
import numpy as np
import pytest

import gsdr
import oracle_binding as orc

pytestmark = pytest.mark.gpu

CODES = np.frombuffer(b"ACGT", dtype=np.uint8)


def rand_seq(rng, n):
    return CODES[rng.integers(0, 4, n)].tobytes()


def mutate(rng, s, rate, indel=0.2):
    out = bytearray()
    for ch in s:
        r = rng.random()
        if r < rate * (1 - indel):
            out.append(int(CODES[rng.integers(0, 4)]))
        elif r < rate * (1 - indel / 2):
            continue
        elif r < rate:
            out.append(ch)
            out.append(int(CODES[rng.integers(0, 4)]))
        else:
            out.append(ch)
    return bytes(out)


def expected(seqs, pairs, t):
    return orc.lcs_decisions(seqs, pairs, t)


def build_case(rng, n_pairs, qlen, tlen, kind):
    seqs, pairs = [], []
    for _ in range(n_pairs):
        q = int(rng.integers(*qlen))
        T = int(rng.integers(*tlen))
        if kind == "random":
            a, b = rand_seq(rng, q), rand_seq(rng, T)
        elif kind == "mutated":
            b = rand_seq(rng, T)
            a = mutate(rng, b[:q], rng.uniform(0.0, 0.12))
        elif kind == "repeats":
            unit = rand_seq(rng, int(rng.integers(1, 5)))
            b = (unit * (T // len(unit) + 1))[:T]
            a = mutate(rng, (unit * (q // len(unit) + 1))[:q], 0.03)
        else:  # embedding: short pattern, long text
            a, b = rand_seq(rng, q), rand_seq(rng, T)
        seqs.append(b)
        seqs.append(a)
        pairs.append((len(seqs) - 1, len(seqs) - 2))
    return seqs, pairs


@pytest.mark.parametrize("mapping", [0, 1, 2, 3])
@pytest.mark.parametrize("greedy", [0, 1])
@pytest.mark.parametrize("qlen,tlen,kind", [
    ((20, 1000), (20, 1200), "mutated"),        # classes 0-1
    ((1000, 4000), (1000, 4500), "mutated"),    # classes 1-3
    ((4000, 9000), (4000, 9500), "mutated"),    # classes 3-4
    ((16000, 20000), (16000, 21000), "mutated"),  # class 5
    ((300, 2500), (9000, 10000), "embed"),      # short pattern, long text
    ((1500, 5000), (3000, 10000), "random"),    # near-threshold rejects
    ((50, 3000), (50, 3000), "repeats"),
])
def test_lcs_decisions(mapping, greedy, qlen, tlen, kind):
    rng = np.random.default_rng(hash((qlen, tlen, kind)) & 0xffff)
    n = 24 if qlen[0] >= 16000 else 120
    seqs, pairs = build_case(rng, n, qlen, tlen, kind)
    for t in (0.80, 0.95):
        got, ms = gsdr.lcs_decide(seqs, pairs, t, mapping=mapping, greedy=greedy)
        want = expected(seqs, pairs, t)
        bad = np.nonzero(got != want)[0]
        assert len(bad) == 0, f"t={t}: {len(bad)} of {len(pairs)} differ, first {bad[:5]}"


def test_lcs_edge_lengths():
    rng = np.random.default_rng(7)
    seqs, pairs = [], []
    # lengths around word / lane / class boundaries, and N-containing patterns
    for q in (1, 2, 15, 16, 17, 31, 32, 33, 63, 64, 65, 1023, 1024, 1025, 2048, 2049, 3072,
              3073, 4096, 4097, 5120, 5121, 6144, 6145, 7168, 7169, 8192, 8193, 16384, 16385,
              32768, 32769, 50000, 65536, 65537, 70000, 131072, 131073):
        b = rand_seq(rng, q + int(rng.integers(0, 40)))
        a = mutate(rng, b[:q], 0.03)
        seqs.append(b)
        seqs.append(a)
        pairs.append((len(seqs) - 1, len(seqs) - 2))
    b = rand_seq(rng, 500)
    seqs.append(b)
    seqs.append(b[:200] + b"NNNNNNNNNN" + b[200:400])
    pairs.append((len(seqs) - 1, len(seqs) - 2))
    for mapping in (0, 1, 2, 3):
        for t in (0.8, 0.9, 0.95):
            got, _ = gsdr.lcs_decide(seqs, pairs, t, mapping=mapping, greedy=1)
            np.testing.assert_array_equal(got, expected(seqs, pairs, t))


@pytest.mark.parametrize("t", [0.80, 0.90, 0.95, 0.99])
@pytest.mark.parametrize("qlen", [(30, 400), (400, 3000), (3000, 12000)])
def test_band_near_threshold(t, qlen):
    """Pairs of similar length whose identity straddles t: every window class
    of the banded kernel (4 to 32 words) decides them as the full DP does."""
    rng = np.random.default_rng(int(t * 100) * 7 + qlen[0])
    seqs, pairs = [], []
    n = 40 if qlen[0] >= 3000 else 150
    for _ in range(n):
        T = int(rng.integers(*qlen))
        b = rand_seq(rng, T)
        a = mutate(rng, b, rng.uniform(0.0, 2.2 * (1 - t) + 0.005), indel=0.4)
        seqs.append(b)
        seqs.append(a)
        pairs.append((len(seqs) - 1, len(seqs) - 2))
    want = expected(seqs, pairs, t)
    assert 0 < want.sum() < len(pairs)
    for mapping in (2, 3):
        got, _ = gsdr.lcs_decide(seqs, pairs, t, mapping=mapping, greedy=0)
        bad = np.nonzero(got != want)[0]
        assert len(bad) == 0, f"mapping {mapping}: {len(bad)} of {len(pairs)} differ, first {bad[:5]}"


@pytest.mark.parametrize("t", [0.80, 0.95])
def test_group_band_every_class(t):
    """Pairs whose bands need 5 to 128 window words, at both ends of each
    group class (2, 4, 8, 16, 32 lanes x 4 words), near the threshold: the
    group-banded kernel decides them as the full DP does."""
    rng = np.random.default_rng(int(t * 1000))
    seqs, pairs = [], []
    # T - c + q - c + 62 spans window words 5 .. 128 through the lengths
    for T in (200, 260, 400, 520, 700, 900, 1300, 1800, 2600, 3400, 5000, 6500, 9000, 12000):
        for _ in range(6):
            b = rand_seq(rng, T)
            a = mutate(rng, b[: int(T * rng.uniform(0.9, 1.0))], rng.uniform(0.0, 2.0 * (1 - t)),
                       indel=0.4)
            seqs.append(b)
            seqs.append(a)
            pairs.append((len(seqs) - 1, len(seqs) - 2))
    want = expected(seqs, pairs, t)
    assert 0 < want.sum() < len(pairs)
    got, _ = gsdr.lcs_decide(seqs, pairs, t, mapping=3, greedy=0)
    bad = np.nonzero(got != want)[0]
    assert len(bad) == 0, f"{len(bad)} of {len(pairs)} differ, first {bad[:5]}"
