"""The alignment decision through gsdr_lcs_decide_noalloc, the entry point for
callers that cannot allocate device memory (a framework's memory pool owns
every buffer, or a plug-in may not grow the device footprint).  The test owns
the device buffers; the library works in its fixed array only.  Two calls in
a row must both match the allocating entry point, gsdr_lcs_decide, exactly
(the decisions are integers: no tolerance).  This file is collected last."""
import numpy as np
import pytest

import gsdr

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


def test_noalloc_matches_allocating_entry():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    seqs, pairs = _case()
    t = 0.95
    want, _ = gsdr.lcs_decide(seqs, pairs, t, mapping=0, greedy=1)
    words, off, gf = _pack(seqs)
    dev = torch.device("cuda:0")
    d_packed = torch.from_numpy(words.view(np.int32)).to(dev)
    d_off = torch.from_numpy(off).to(dev)
    d_raw = torch.from_numpy(np.array([len(s) for s in seqs], dtype=np.int32)).to(dev)
    d_gf = torch.from_numpy(gf).to(dev)
    d_pat = torch.tensor([p for p, _ in pairs], dtype=torch.int32, device=dev)
    d_txt = torch.tensor([x for _, x in pairs], dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    for call in range(2):
        d_acc = torch.full((len(pairs),), 7, dtype=torch.uint8, device=dev)
        torch.cuda.synchronize()
        gsdr.lcs_decide_noalloc(d_packed.data_ptr(), d_off.data_ptr(), d_raw.data_ptr(),
                                d_gf.data_ptr(), len(seqs), d_pat.data_ptr(), d_txt.data_ptr(),
                                len(pairs), t, d_acc.data_ptr(), None)
        got = d_acc.cpu().numpy()
        np.testing.assert_array_equal(got, want, err_msg=f"call {call}")
    assert want.sum() > 0 and want.sum() < len(pairs)


def test_noalloc_rejects_oversized_calls():
    with pytest.raises(gsdr.GsdrError) as e:
        gsdr.lcs_decide_noalloc(0, 0, 0, 0, 10, 0, 0, gsdr_max_pairs() + 1, 0.95, 0, None)
    assert e.value.status == gsdr.EINVAL


def gsdr_max_pairs():
    return 16384
