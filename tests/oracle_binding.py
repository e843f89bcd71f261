"""ctypes binding of the oracle (oracle/gsdr_oracle.cpp) -- test-side only."""
import ctypes as C
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
LIB = os.path.join(ORACLE_DIR, "_build", "liboracle.so")


class OrcStats(C.Structure):
    _fields_ = [(n, C.c_longlong) for n in
                "rounds prefilter_in prefilter_pass pigeon_pass word_pass aligned accepted cells".split()] + [
        ("seconds", C.c_double), ("k", C.c_int), ("drop", C.c_int), ("pigeon", C.c_int),
        ("threshold", C.c_float)]


def build():
    r = subprocess.run(["make", "-s", "-C", ORACLE_DIR], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        L.orc_run.restype = C.c_longlong
        L.orc_run.argtypes = [C.c_char_p, C.c_char_p, C.c_float, C.c_int, C.c_int, C.c_int,
                              C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                              C.POINTER(OrcStats)]
        L.orc_cutoffs.argtypes = [C.c_void_p, C.c_int, C.c_float, C.c_int, C.c_void_p,
                                  C.c_void_p, C.c_void_p]
        L.orc_lcs.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int]
        L.orc_pack.argtypes = [C.c_char_p, C.c_int, C.c_void_p, C.POINTER(C.c_int)]
        L.orc_kmers.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        L.orc_pair.argtypes = [C.c_char_p, C.c_int, C.c_char_p, C.c_int, C.c_float, C.c_int]
        L.orc_check_option.argtypes = [C.c_int, C.POINTER(C.c_char_p), C.POINTER(C.c_float),
                                       C.POINTER(C.c_int), C.POINTER(C.c_int),
                                       C.POINTER(C.c_int)]
        L.orc_pigeon_index.argtypes = [C.c_char_p, C.c_int, C.c_longlong, C.c_void_p,
                                       C.c_void_p]
        L.orc_run_v.restype = C.c_longlong
        L.orc_run_v.argtypes = L.orc_run.argtypes + [C.c_int]
        L.orc_check_option_sycl.argtypes = [C.c_int, C.POINTER(C.c_char_p),
                                            C.POINTER(C.c_float), C.POINTER(C.c_int)]
        L.orc_cutoffs_sycl.argtypes = [C.c_void_p, C.c_int, C.c_float, C.c_int, C.c_void_p,
                                       C.c_void_p]
        L.orc_kmers_raw.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        L.orc_set_keep_order.argtypes = [C.c_int]
        _lib = L
    return _lib


def run(path, out=None, t=0.95, w=0, d=3, p=0, lcs_mode=1, threads=0, max_rounds=-1, variant=0):
    """Runs the oracle on a FASTA file.  Returns (order, cluster, stats).
    variant 1: the SYCL program's semantics."""
    with open(path, "rb") as f:
        n_guess = max(1, f.read().count(b"\n>") + 2)
    order = np.zeros(n_guess, dtype=np.int32)
    cluster = np.zeros(n_guess, dtype=np.int32)
    st = OrcStats()
    n = lib().orc_run_v(os.fsencode(path), os.fsencode(out) if out else None, C.c_float(t), w,
                        d, p, lcs_mode, threads, max_rounds, order.ctypes.data,
                        cluster.ctypes.data, C.byref(st), variant)
    if n < 0:
        raise ValueError("oracle rejected the options")
    return order[:n], cluster[:n], st


def run_bytes_in_order(data: bytes, tmpdir, **kw):
    """run_bytes on a file already in length order, keeping its order of
    equal-length reads (a stable sort instead of the reference's std::sort)."""
    lib().orc_set_keep_order(1)
    try:
        return run_bytes(data, tmpdir, **kw)
    finally:
        lib().orc_set_keep_order(0)


def run_bytes(data: bytes, tmpdir, name="in.fa", **kw):
    path = os.path.join(str(tmpdir), name)
    with open(path, "wb") as f:
        f.write(data)
    out = path + ".oracle.out"
    order, cluster, st = run(path, out, **kw)
    with open(out, "rb") as f:
        fasta = f.read()
    return order, cluster, st, fasta


def cutoffs(lengths, t, k):
    L = np.ascontiguousarray(lengths, dtype=np.int32)
    w = np.zeros_like(L)
    b = np.zeros_like(L)
    p = np.zeros_like(L)
    lib().orc_cutoffs(L.ctypes.data, len(L), C.c_float(t), k, w.ctypes.data, b.ctypes.data,
                      p.ctypes.data)
    return w, b, p


def lcs(a: np.ndarray, b: np.ndarray, mode=1) -> int:
    a = np.ascontiguousarray(a, dtype=np.uint8)
    b = np.ascontiguousarray(b, dtype=np.uint8)
    return lib().orc_lcs(a.ctypes.data, len(a), b.ctypes.data, len(b), mode)


def gap_free_codes(s: bytes) -> np.ndarray:
    """ACGT/U (either case) -> 0..3 with every other byte dropped (the
    reference's packing, cuda-version/func.cu:139-179, 272-299)."""
    lut = np.full(256, 255, dtype=np.uint8)
    for i, ch in enumerate(b"ACGT"):
        lut[ch] = i
        lut[ch | 0x20] = i
    lut[ord("U")] = lut[ord("u")] = 3
    c = lut[np.frombuffer(s, dtype=np.uint8)]
    return c[c < 4]


def lcs_decisions(seqs, pairs, t):
    """The alignment-stage decision of kernel_align (cuda-version/func.cu:828-999)
    for each (pattern, text) pair: 1 iff the gap-free LCS reaches the pattern's
    base cutoff ceil(len * t) (func.cu:331-332)."""
    lens = np.array([len(s) for s in seqs], dtype=np.int32)
    _, base, _ = cutoffs(lens, t, 6)
    out = []
    for p, x in pairs:
        a = gap_free_codes(seqs[p])
        b = gap_free_codes(seqs[x])
        if len(b) == 0:
            out.append(0)
            continue
        out.append(1 if lcs(a, b) >= base[p] else 0)
    return np.array(out, dtype=np.uint8)


def pack(seq: bytes):
    out = np.zeros(len(seq) // 16 + 2, dtype=np.uint32)
    gaps = C.c_int()
    nw = lib().orc_pack(seq, len(seq), out.ctypes.data, C.byref(gaps))
    return out[:nw], gaps.value


def kmers(gf_codes: np.ndarray, k: int):
    g = np.ascontiguousarray(gf_codes, dtype=np.uint8)
    w = np.zeros(max(len(g), 1), dtype=np.uint32)
    c = np.zeros(max(len(g), 1), dtype=np.uint16)
    n = lib().orc_kmers(g.ctypes.data, len(g), k, w.ctypes.data, c.ctypes.data)
    return w[:n], c[:n]


def check_option(argv):
    args = [b"cluster"] + [a.encode() for a in argv]
    arr = (C.c_char_p * len(args))(*args)
    t, k, d, p = C.c_float(), C.c_int(), C.c_int(), C.c_int()
    rc = lib().orc_check_option(len(args), arr, C.byref(t), C.byref(k), C.byref(d), C.byref(p))
    if rc:
        return None
    return t.value, k.value, d.value, p.value


def pair(rep: bytes, q: bytes, t: float, k: int) -> int:
    return lib().orc_pair(rep, len(rep), q, len(q), C.c_float(t), k)


def check_option_sycl(argv):
    args = [b"cluster"] + [a.encode() for a in argv]
    arr = (C.c_char_p * len(args))(*args)
    t, k = C.c_float(), C.c_int()
    if lib().orc_check_option_sycl(len(args), arr, C.byref(t), C.byref(k)):
        return None
    return t.value, k.value


def cutoffs_sycl(lengths, t, k):
    L = np.ascontiguousarray(lengths, dtype=np.int32)
    w = np.zeros_like(L)
    b = np.zeros_like(L)
    lib().orc_cutoffs_sycl(L.ctypes.data, len(L), C.c_float(t), k, w.ctypes.data, b.ctypes.data)
    return w, b


def kmers_raw(seq: bytes, k: int):
    w = np.zeros(max(len(seq), 1), dtype=np.uint32)
    c = np.zeros(max(len(seq), 1), dtype=np.uint16)
    n = lib().orc_kmers_raw(seq, len(seq), k, w.ctypes.data, c.ctypes.data)
    return w[:n], c[:n]
