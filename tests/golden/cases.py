"""Inputs of the golden cases: every input is rebuilt byte for byte from
these definitions (the synthetic generator and numpy's PCG64 are the same on
every platform; the recorded input sha256 guards that)."""
import gzip
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _edge_mixed(seed=9):
    rng = np.random.default_rng(seed)
    codes = np.frombuffer(b"ACGT", dtype=np.uint8)
    base = codes[rng.integers(0, 4, 700)].tobytes()
    recs = []
    for i in range(60):
        s = bytearray(base[: rng.integers(150, 700)])
        for _ in range(rng.integers(0, 12)):
            s[rng.integers(0, len(s))] = int(rng.choice(list(b"ACGTNRYacgtnu")))
        if i % 7 == 0:
            s += b"\r"
        recs.append(b">r%d desc\n" % i + bytes(s) + b"\n")
    recs.append(b">short1\nACG\n")
    recs.append(b">short2\nACGTA\n")
    recs.append(b">multiline\n" + base[:100] + b"\n" + base[100:300] + b"\n\n" + base[300:400] + b"\n")
    recs.append(b">dup1\n" + base[:500] + b"\n")
    recs.append(b">dup2\n" + base[:500] + b"\n")
    return b"".join(recs)


def _ties(seed=4):
    rng = np.random.default_rng(seed)
    codes = np.frombuffer(b"ACGT", dtype=np.uint8)
    seeds = [codes[rng.integers(0, 4, 120)].tobytes() for _ in range(40)]
    recs = []
    for i in range(1500):
        s = bytearray(seeds[i % 40])
        for _ in range(rng.integers(0, 6)):
            s[rng.integers(0, 120)] = int(codes[rng.integers(0, 4)])
        recs.append(b">t%d\n" % i + bytes(s) + b"\n")
    return b"".join(recs)


def _reference_result():
    return reference_result("cuda")


def reference_result(which):
    """The reference's own output file: "cuda" = cuda-version/result.fasta,
    "sycl" = the SYCL program's top-level result.fasta (both at t = 0.95 on
    the same input, which the reference does not distribute)."""
    with gzip.open(os.path.join(HERE, f"ref_{which}_result.fasta.gz"), "rb") as f:
        return f.read()


def records(data):
    """(name line, sequence) pairs of a file with one sequence line per record."""
    lines = data.split(b"\n")
    return [(lines[i], lines[i + 1]) for i in range(0, len(lines) - 1, 2)]


def union_of_results(first):
    """The records of both result files, longest first; among equal lengths the
    records of result file `first` come first, in that file's order.  Every
    record of the other file only was absorbed, in the run that wrote `first`,
    by a longer or earlier record of `first`, and those order ties the same
    way here, so clustering this list with the semantics that wrote `first`
    gives back exactly the records of `first`."""
    mine = records(reference_result(first))
    other = records(reference_result("sycl" if first == "cuda" else "cuda"))
    have = set(mine)
    rest = [r for r in other if r not in have]
    keyed = [(len(r[1]), 0, i, r) for i, r in enumerate(mine)]
    keyed += [(len(r[1]), 1, i, r) for i, r in enumerate(rest)]
    keyed.sort(key=lambda x: (-x[0], x[1], x[2]))
    return [x[3] for x in keyed], have


# name: (input builder, cluster options as argv letters)
CASES = {
    "c0_10k_t95": (("synth", 0, 10000, None), ["t", "0.95"]),
    "c0_3k_t90": (("synth", 0, 3000, 2), ["t", "0.90"]),
    "c0_3k_t97": (("synth", 0, 3000, 3), ["t", "0.97"]),
    "c0_2k_t88": (("synth", 0, 2000, 4), ["t", "0.88"]),
    "c0_2k_w7": (("synth", 0, 2000, 5), ["t", "0.95", "w", "7"]),
    "c0_800_t85_drop": (("synth", 0, 800, 6), ["t", "0.85"]),
    "c0_800_t95_d1": (("synth", 0, 800, 7), ["t", "0.95", "d", "1"]),
    "c1_20k_t95": (("synth", 1, 20000, 21), ["t", "0.95"]),
    "c2_30k_t90": (("synth", 2, 30000, 31), ["t", "0.90"]),
    "c4_3k_t90": (("synth", 4, 3000, 41), ["t", "0.90"]),
    "ties_150bp_t95": (("fn", "ties"), ["t", "0.95"]),
    "edge_mixed_t95": (("fn", "edge"), ["t", "0.95"]),
    "edge_mixed_t90": (("fn", "edge"), ["t", "0.90"]),
    "ref_result_t95": (("fn", "refres"), ["t", "0.95"]),
    # the pigeon filter (p 1)
    "c0_3k_t95_p1": (("synth", 0, 3000, 8), ["t", "0.95", "p", "1"]),
    "c0_2k_t90_p1": (("synth", 0, 2000, 9), ["t", "0.90", "p", "1"]),
    "c4_2k_t93_p1": (("synth", 4, 2000, 42), ["t", "0.93", "p", "1"]),
    "edge_mixed_t95_p1": (("fn", "edge"), ["t", "0.95", "p", "1"]),
    # word lengths above 7 (w override)
    "c0_2k_w8": (("synth", 0, 2000, 10), ["t", "0.95", "w", "8"]),
    "c0_2k_w10": (("synth", 0, 2000, 11), ["t", "0.93", "w", "10"]),
    "c0_1k_w12": (("synth", 0, 1000, 12), ["t", "0.95", "w", "12"]),
}


def build_input(spec):
    if spec[0] == "synth":
        import gsdr

        _, cfg, n, seed = spec
        kw = {}
        if cfg == 4:
            kw = dict(n_seeds=max(1, n // 5), len_lo=150, len_hi=5000)
        return gsdr.synth_fasta(cfg, n_reads=n, seed=seed, **kw)
    name = spec[1]
    return {"ties": _ties, "edge": _edge_mixed, "refres": _reference_result}[name]()
