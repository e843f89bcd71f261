"""The alignment decision through gsdr_lcs_decide_noalloc, the entry point for
callers that cannot allocate device memory (a framework's memory pool owns
every buffer, or a plug-in may not grow the device footprint).  The test owns
the device buffers; the library works in its fixed array only.  Two calls in
a row must both match the oracle's LCS decision and the allocating entry point,
gsdr_lcs_decide, exactly (the decisions are integers: no tolerance).  Inputs
the entry point must refuse (an index out of range, a pattern in two pairs)
return GSDR_EINVAL without touching memory out of range, and a valid call after
them is still exact.  This file is collected last."""
import numpy as np
import pytest

import gsdr
import oracle_binding as orc

pytestmark = pytest.mark.gpu

CODES = np.frombuffer(b"ACGT", dtype=np.uint8)


def _pack(seqs):
    """Gap-free 2-bit packing (16 bases per word, first base in bits 31:30),
    one extra readable word after each sequence."""
    lut = np.full(256, 255, dtype=np.uint8)
    for i, ch in enumerate(b"ACGT"):
        lut[ch] = i
    words, off, gf = [], [], []
    pos = 0
    for s in seqs:
        c = lut[np.frombuffer(s, dtype=np.uint8)]
        c = c[c < 4].astype(np.uint32)
        nw = len(c) // 16 + 2
        w = np.zeros(nw, dtype=np.uint32)
        idx = np.arange(len(c))
        np.bitwise_or.at(w, idx // 16, c << (30 - 2 * (idx % 16)).astype(np.uint32))
        words.append(w)
        off.append(pos)
        gf.append(len(c))
        pos += nw
    return (np.concatenate(words), np.array(off, dtype=np.int64), np.array(gf, dtype=np.int32))


def _case(seed=5):
    rng = np.random.default_rng(seed)
    seqs, pairs = [], []
    for q, T, rate in [(150, 160, 0.05), (900, 1000, 0.03), (1800, 2100, 0.08),
                       (3500, 3900, 0.04), (7000, 8000, 0.02), (600, 9000, 0.0),
                       (12000, 12500, 0.03), (20000, 20500, 0.02)]:
        for _ in range(12 if q < 10000 else 3):
            text = CODES[rng.integers(0, 4, T)].tobytes()
            if rate == 0.0:
                pat = CODES[rng.integers(0, 4, q)].tobytes()  # embedding case
            else:
                a = np.frombuffer(text[:q], dtype=np.uint8).copy()
                hit = rng.random(q) < rate
                a[hit] = CODES[rng.integers(0, 4, hit.sum())]
                pat = a.tobytes()
            seqs.append(text)
            seqs.append(pat)
            pairs.append((len(seqs) - 1, len(seqs) - 2))
    return seqs, pairs


def _device_case(torch, seqs, pairs):
    words, off, gf = _pack(seqs)
    dev = torch.device("cuda:0")
    return {
        "packed": torch.from_numpy(words.view(np.int32)).to(dev),
        "off": torch.from_numpy(off).to(dev),
        "raw": torch.from_numpy(np.array([len(s) for s in seqs], dtype=np.int32)).to(dev),
        "gf": torch.from_numpy(gf).to(dev),
        "pat": torch.tensor([p for p, _ in pairs], dtype=torch.int32, device=dev),
        "txt": torch.tensor([x for _, x in pairs], dtype=torch.int32, device=dev),
        "n_seq": len(seqs),
    }


def _call(torch, d, t, n_pairs=None, pat=None):
    n = len(d["pat"]) if n_pairs is None else n_pairs
    acc = torch.full((max(n, 1),), 7, dtype=torch.uint8, device="cuda:0")
    torch.cuda.synchronize()
    p = d["pat"] if pat is None else pat
    gsdr.lcs_decide_noalloc(d["packed"].data_ptr(), d["off"].data_ptr(), d["raw"].data_ptr(),
                            d["gf"].data_ptr(), d["n_seq"], p.data_ptr(), d["txt"].data_ptr(),
                            n, t, acc.data_ptr(), None)
    return acc[:n].cpu().numpy()


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def test_noalloc_matches_oracle_and_allocating_entry():
    torch = _torch()
    seqs, pairs = _case()
    t = 0.95
    want = orc.lcs_decisions(seqs, pairs, t)
    alloc, _ = gsdr.lcs_decide(seqs, pairs, t, mapping=0, greedy=1)
    np.testing.assert_array_equal(alloc, want)
    d = _device_case(torch, seqs, pairs)
    for call in range(2):
        np.testing.assert_array_equal(_call(torch, d, t), want, err_msg=f"call {call}")
    assert 0 < want.sum() < len(pairs)


def test_noalloc_rejects_bad_indices_then_stays_exact():
    torch = _torch()
    seqs, pairs = _case(seed=8)
    t = 0.90
    want = orc.lcs_decisions(seqs, pairs, t)
    d = _device_case(torch, seqs, pairs)
    n = len(pairs)
    for bad_value in (-1, d["n_seq"], 1 << 30):
        bad = d["pat"].clone()
        bad[n // 2] = bad_value
        with pytest.raises(gsdr.GsdrError) as e:
            _call(torch, d, t, pat=bad)
        assert e.value.status == gsdr.EINVAL
    dup = d["pat"].clone()
    dup[1] = dup[0]  # the same pattern in two pairs
    with pytest.raises(gsdr.GsdrError) as e:
        _call(torch, d, t, pat=dup)
    assert e.value.status == gsdr.EINVAL
    np.testing.assert_array_equal(_call(torch, d, t), want)


def test_noalloc_rejects_oversized_calls():
    with pytest.raises(gsdr.GsdrError) as e:
        gsdr.lcs_decide_noalloc(0, 0, 0, 0, 10, 0, 0, gsdr.NOALLOC_MAX_PAIRS + 1, 0.95, 0,
                                None)
    assert e.value.status == gsdr.EINVAL
    with pytest.raises(gsdr.GsdrError) as e:
        gsdr.lcs_decide_noalloc(0, 0, 0, 0, gsdr.NOALLOC_MAX_SEQS + 1, 0, 0, 1, 0.95, 0, None)
    assert e.value.status == gsdr.EINVAL
