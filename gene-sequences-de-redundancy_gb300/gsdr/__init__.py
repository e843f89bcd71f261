"""Python view of the GB300 clustering library (ctypes over libgsdr.so).

The names follow the reference program's functions (cuda-version/func.h):
``check_option`` (checkOption), ``read_file`` (readFile), ``clustering``
(clustering / clusteringDrop with the preparation kernels before them),
``save_file`` (saveFile) and ``main``.  Everything runs through the C ABI
declared in include/gsdr.h; there is no Python or CPU fallback: a missing
library or CUDA device raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD_DIR = os.path.join(_PKG, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libgsdr.so")
SYNTH_PATH = os.path.join(BUILD_DIR, "libgsdr_synth.so")
CLI_PATH = os.path.join(BUILD_DIR, "cluster")

OK, EINVAL, ENOMEM, EDEVICE, ETIMEOUT, EIO, EUNSUPPORTED, EBUSY, ENOTFOUND = range(9)
# limits of gsdr_lcs_decide_noalloc (include/gsdr.h)
NOALLOC_MAX_PAIRS = 16384
NOALLOC_MAX_SEQS = 65536


class GsdrError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"gsdr status {status}: {msg}")
        self.status = status


class Opts(C.Structure):
    _fields_ = [
        ("threshold", C.c_float),
        ("word_length", C.c_int32),
        ("drop", C.c_int32),
        ("pigeon", C.c_int32),
        ("batch", C.c_int32),
        ("device", C.c_int32),
        ("stage_timing", C.c_int32),
        ("verbose", C.c_int32),
        ("word_filter", C.c_int32),
        ("variant", C.c_int32),  # 0 cuda-version semantics, 1 the SYCL program's
        ("band_serial", C.c_int32),  # lane-banded kernel's limit; 0 automatic, -1 none
        ("group_words", C.c_int32),  # group-banded kernel's widest window; 0 automatic, -1 none
        ("align_blocks", C.c_int32),  # block shape: CTAs per SM of the alignment kernels
        ("filter_blocks", C.c_int32),  # the same for the word-filter kernels
        ("graph_steps", C.c_int32),  # staging depth: rounds / passes per graph launch
    ]


class Reads(C.Structure):
    _fields_ = [
        ("bytes", C.c_void_p),
        ("n_bytes", C.c_int64),
        ("offset", C.c_void_p),
        ("length", C.c_void_p),
        ("n", C.c_int32),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("rounds", C.c_int64),
        ("passes", C.c_int64),
        ("pairs_prefilter", C.c_int64),
        ("pairs_word", C.c_int64),
        ("pairs_aligned", C.c_int64),
        ("pairs_accepted", C.c_int64),
        ("cells", C.c_double),
        ("filter_bytes", C.c_double),
        ("ms_h2d", C.c_double),
        ("ms_prep", C.c_double),
        ("ms_cluster", C.c_double),
        ("ms_d2h", C.c_double),
        ("ms_total", C.c_double),
        ("ms_filter", C.c_double),
        ("ms_align", C.c_double),
        ("k", C.c_int32),
        ("drop", C.c_int32),
        ("pigeon", C.c_int32),
        ("batch", C.c_int32),
        ("kernel_launches", C.c_int64),
        ("word_index", C.c_int32),
        ("filter_max_bytes", C.c_double),
        ("filter_max_ms", C.c_double),
        ("cells_computed", C.c_double),
        ("tuned", C.c_int32),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class ServerOpts(C.Structure):
    _fields_ = [
        ("device", C.c_int32),
        ("max_inflight", C.c_int32),
        ("mem_budget", C.c_int64),
        ("batch", C.c_int32),
        ("express_bytes", C.c_int64),
    ]


class SynthCfg(C.Structure):
    _fields_ = [
        ("n_reads", C.c_int64),
        ("n_seeds", C.c_int64),
        ("len_dist", C.c_int32),
        ("copies_max", C.c_int32),
        ("len_lo", C.c_double),
        ("len_hi", C.c_double),
        ("len_median", C.c_double),
        ("len_sigma", C.c_double),
        ("id_lo", C.c_double),
        ("sub_frac", C.c_double),
        ("indel_lo", C.c_int32),
        ("indel_hi", C.c_int32),
        ("gc_lo", C.c_double),
        ("gc_hi", C.c_double),
        ("mode", C.c_int32),
        ("pad_", C.c_int32),
        ("extra_indel_frac", C.c_double),
        ("seed", C.c_uint64),
    ]


_lib = None
_synth = None


def lib():
    """Loads libgsdr.so (built by build.py); raises if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise GsdrError(EDEVICE, f"{LIB_PATH} is not built; run the package build first")
        L = C.CDLL(LIB_PATH)
        P = C.POINTER
        L.gsdr_cluster.argtypes = [P(Reads), P(Opts), C.c_void_p, P(Stats)]
        L.gsdr_fasta_read.argtypes = [C.c_char_p, P(C.c_void_p)]
        L.gsdr_fasta_parse.argtypes = [C.c_char_p, C.c_int64, P(C.c_void_p)]
        L.gsdr_fasta_count.argtypes = [C.c_void_p]
        L.gsdr_fasta_view.argtypes = [C.c_void_p, P(Reads)]
        L.gsdr_fasta_order.argtypes = [C.c_void_p]
        L.gsdr_fasta_order.restype = C.c_void_p
        L.gsdr_fasta_name.argtypes = [C.c_void_p, C.c_int32, P(C.c_int64)]
        L.gsdr_fasta_name.restype = C.c_void_p
        L.gsdr_fasta_write.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, P(C.c_int64)]
        L.gsdr_fasta_format.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                                        P(C.c_int64)]
        L.gsdr_fasta_free.argtypes = [C.c_void_p]
        L.gsdr_cluster_fasta.argtypes = [C.c_void_p, C.c_int64, P(Opts), P(C.c_void_p),
                                         P(Stats)]
        L.gsdr_result_output.argtypes = [C.c_void_p, P(C.c_void_p), P(C.c_int64)]
        L.gsdr_result_count.argtypes = [C.c_void_p]
        for fn in ("gsdr_result_cluster", "gsdr_result_order", "gsdr_result_lengths"):
            getattr(L, fn).argtypes = [C.c_void_p]
            getattr(L, fn).restype = C.c_void_p
        L.gsdr_result_free.argtypes = [C.c_void_p]
        L.gsdr_job_run_limited.argtypes = [C.c_void_p, C.c_int32, P(Stats)]
        L.gsdr_fasta_format_clusters.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                                                 P(C.c_int64)]
        L.gsdr_fasta_write_clusters.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, P(C.c_int64)]
        L.gsdr_default_opts.argtypes = [P(Opts)]
        L.gsdr_resolve_opts.argtypes = [P(Opts), P(C.c_char_p)]
        L.gsdr_check_option.argtypes = [C.c_int, P(C.c_char_p), P(Opts), C.c_char_p,
                                        C.c_char_p, C.c_int64]
        L.gsdr_main.argtypes = [C.c_int, P(C.c_char_p)]
        L.gsdr_job_create.argtypes = [P(Reads), P(Opts), P(C.c_void_p)]
        L.gsdr_job_run.argtypes = [C.c_void_p, P(Stats)]
        L.gsdr_job_cluster.argtypes = [C.c_void_p, C.c_void_p]
        L.gsdr_job_free.argtypes = [C.c_void_p]
        L.gsdr_lcs_decide.argtypes = [C.c_char_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_int32,
                                      C.c_void_p, C.c_void_p, C.c_int32, C.c_float, C.c_int32,
                                      C.c_int32, C.c_void_p, C.POINTER(C.c_double)]
        L.gsdr_lcs_decide_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                              C.c_int32, C.c_void_p, C.c_void_p, C.c_int32,
                                              C.c_float, C.c_void_p, C.c_void_p]
        L.gsdr_set_spin_limit.argtypes = [C.c_int32, C.c_int32]
        L.gsdr_job_resume.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, P(Stats)]
        L.gsdr_autotune.argtypes = [P(Reads), P(Opts), C.c_int32, C.c_int32, C.c_char_p,
                                    P(Opts), C.c_char_p, C.c_int64, P(C.c_int64)]
        L.gsdr_server_times.argtypes = [C.c_void_p, C.c_int64, C.POINTER(C.c_double),
                                        C.POINTER(C.c_double)]
        L.gsdr_server_create.argtypes = [C.POINTER(ServerOpts), C.POINTER(C.c_void_p)]
        L.gsdr_server_submit.argtypes = [C.c_void_p, C.c_char_p, C.c_int64, C.c_float,
                                         C.POINTER(C.c_int64)]
        L.gsdr_server_wait.argtypes = [C.c_void_p, C.c_int64, C.POINTER(C.c_int64),
                                       C.POINTER(C.c_int32), C.POINTER(C.c_double)]
        L.gsdr_server_result.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64,
                                         C.POINTER(C.c_int64), C.c_void_p, C.POINTER(C.c_int32)]
        L.gsdr_server_release.argtypes = [C.c_void_p, C.c_int64]
        L.gsdr_server_destroy.argtypes = [C.c_void_p]
        L.gsdr_strerror.restype = C.c_char_p
        L.gsdr_last_error.restype = C.c_char_p
        _lib = L
    return _lib


def synth_lib():
    global _synth
    if _synth is None:
        if not os.path.exists(SYNTH_PATH):
            raise GsdrError(EDEVICE, f"{SYNTH_PATH} is not built")
        S = C.CDLL(SYNTH_PATH)
        S.gsdr_synth_preset.argtypes = [C.c_int, C.POINTER(SynthCfg)]
        S.gsdr_synth_generate.argtypes = [C.POINTER(SynthCfg), C.POINTER(C.c_void_p),
                                          C.POINTER(C.c_int64)]
        S.gsdr_synth_generate.restype = C.c_int64
        S.gsdr_synth_write.argtypes = [C.POINTER(SynthCfg), C.c_char_p]
        S.gsdr_synth_write.restype = C.c_int64
        S.gsdr_synth_free.argtypes = [C.c_void_p]
        _synth = S
    return _synth


def _check(status):
    if status != OK:
        msg = lib().gsdr_last_error().decode(errors="replace")
        raise GsdrError(status, msg or lib().gsdr_strerror(status).decode())


# ---- options -------------------------------------------------------------------

def default_opts(**kw) -> Opts:
    o = Opts()
    lib().gsdr_default_opts(C.byref(o))
    names = {f[0] for f in Opts._fields_}
    for k, v in kw.items():
        if k not in names:
            raise TypeError(f"unknown option {k!r}")
        setattr(o, k, v)
    return o


def resolve_opts(o: Opts) -> Opts:
    o2 = Opts.from_buffer_copy(o)
    _check(lib().gsdr_resolve_opts(C.byref(o2), None))
    return o2


def check_option(argv):
    """checkOption: argv without the program name.  Returns (opts, in, out)
    or raises GsdrError(EINVAL) where the reference prints its usage."""
    args = [b"cluster"] + [a.encode() if isinstance(a, str) else a for a in argv]
    arr = (C.c_char_p * len(args))(*args)
    o = Opts()
    cap = 4096
    ib, ob = C.create_string_buffer(cap), C.create_string_buffer(cap)
    _check(lib().gsdr_check_option(len(args), arr, C.byref(o), ib, ob, cap))
    return o, ib.value.decode(), ob.value.decode()


# ---- FASTA ---------------------------------------------------------------------

class Fasta:
    """Reads parsed and sorted as readFile does; owns the native object."""

    def __init__(self, handle):
        self._h = C.c_void_p(handle)
        self.n = lib().gsdr_fasta_count(self._h)
        v = Reads()
        _check(lib().gsdr_fasta_view(self._h, C.byref(v)))
        self.view = v

    @classmethod
    def read(cls, path):
        h = C.c_void_p()
        _check(lib().gsdr_fasta_read(os.fsencode(path), C.byref(h)))
        return cls(h.value)

    @classmethod
    def parse(cls, data: bytes):
        h = C.c_void_p()
        _check(lib().gsdr_fasta_parse(data, len(data), C.byref(h)))
        return cls(h.value)

    def order(self) -> np.ndarray:
        p = lib().gsdr_fasta_order(self._h)
        return np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_int32)), (self.n,)).copy()

    def lengths(self) -> np.ndarray:
        return np.ctypeslib.as_array(C.cast(self.view.length, C.POINTER(C.c_int32)),
                                     (self.n,)).copy()

    def format(self, cluster: np.ndarray) -> bytes:
        cl = np.ascontiguousarray(cluster, dtype=np.int32)
        need = C.c_int64()
        _check(lib().gsdr_fasta_format(self._h, cl.ctypes.data, None, 0, C.byref(need)))
        buf = C.create_string_buffer(max(need.value, 1))
        _check(lib().gsdr_fasta_format(self._h, cl.ctypes.data, buf, need.value, C.byref(need)))
        return buf.raw[: need.value]

    def write(self, path, cluster: np.ndarray) -> int:
        cl = np.ascontiguousarray(cluster, dtype=np.int32)
        n = C.c_int64()
        _check(lib().gsdr_fasta_write(os.fsencode(path), self._h, cl.ctypes.data, C.byref(n)))
        return n.value

    def format_clusters(self, cluster: np.ndarray) -> bytes:
        """Cluster membership text (.clstr, include/gsdr.h)."""
        cl = np.ascontiguousarray(cluster, dtype=np.int32)
        need = C.c_int64()
        _check(lib().gsdr_fasta_format_clusters(self._h, cl.ctypes.data, None, 0, C.byref(need)))
        buf = C.create_string_buffer(max(need.value, 1))
        _check(lib().gsdr_fasta_format_clusters(self._h, cl.ctypes.data, buf, need.value,
                                                C.byref(need)))
        return buf.raw[: need.value]

    def write_clusters(self, path, cluster: np.ndarray) -> int:
        cl = np.ascontiguousarray(cluster, dtype=np.int32)
        n = C.c_int64()
        _check(lib().gsdr_fasta_write_clusters(os.fsencode(path), self._h, cl.ctypes.data,
                                               C.byref(n)))
        return n.value

    def close(self):
        if self._h:
            lib().gsdr_fasta_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def read_file(path) -> Fasta:
    """readFile (cuda-version/func.cu:94-117)."""
    return Fasta.read(path)


def save_file(path, fasta: Fasta, cluster) -> int:
    """saveFile (cuda-version/func.cu:1099-1111); returns the cluster count."""
    return fasta.write(path, cluster)


def save_clusters(path, fasta: Fasta, cluster) -> int:
    """Cluster membership (.clstr text, include/gsdr.h); returns the cluster count."""
    return fasta.write_clusters(path, cluster)


# ---- clustering ----------------------------------------------------------------

def clustering(fasta: Fasta, opts: Opts | None = None, stats: bool = False, **kw):
    """The device path (cuda-version/func.cu:119-1097): returns cluster[] in
    sorted order (and the Stats when stats=True)."""
    o = opts if opts is not None else default_opts()
    if kw:
        o = Opts.from_buffer_copy(o)
        for k, v in kw.items():
            setattr(o, k, v)
    cl = np.empty(max(fasta.n, 1), dtype=np.int32)
    st = Stats()
    _check(lib().gsdr_cluster(C.byref(fasta.view), C.byref(o), cl.ctypes.data, C.byref(st)))
    cl = cl[: fasta.n]
    return (cl, st) if stats else cl


def cluster_reads(seqs, opts: Opts | None = None, stats: bool = False, **kw):
    """gsdr_cluster on reads the caller has already put in length order
    (longest first, any tie order): seqs is a list of sequence byte strings.
    Returns cluster[] in that order (and the Stats when stats=True)."""
    o = opts if opts is not None else default_opts()
    if kw:
        o = Opts.from_buffer_copy(o)
        for k, v in kw.items():
            setattr(o, k, v)
    lens = np.array([len(x) for x in seqs], dtype=np.int32)
    if len(lens) > 1 and np.any(lens[1:] > lens[:-1]):
        raise ValueError("reads must be in non-increasing length order")
    buf = b"".join(seqs)
    off = np.zeros(max(len(seqs), 1), dtype=np.int64)
    if len(seqs) > 1:
        off[1:len(seqs)] = np.cumsum(lens[:-1])
    r = Reads()
    keep = C.create_string_buffer(buf, max(len(buf), 1))
    r.bytes = C.cast(keep, C.c_void_p)
    r.n_bytes = len(buf)
    r.offset = off.ctypes.data
    r.length = lens.ctypes.data
    r.n = len(seqs)
    cl = np.empty(max(len(seqs), 1), dtype=np.int32)
    st = Stats()
    _check(lib().gsdr_cluster(C.byref(r), C.byref(o), cl.ctypes.data, C.byref(st)))
    cl = cl[: len(seqs)]
    return (cl, st) if stats else cl


class Job:
    """A clustering job whose reads stay on the device (gsdr_job_*)."""

    def __init__(self, fasta: Fasta, opts: Opts):
        self.fasta = fasta
        self.n = fasta.n
        h = C.c_void_p()
        _check(lib().gsdr_job_create(C.byref(fasta.view), C.byref(opts), C.byref(h)))
        self._h = h

    def run(self, max_passes: int = 0) -> Stats:
        """gsdr_job_run; with max_passes > 0, gsdr_job_run_limited (the
        clustering stops unfinished after that many passes or rounds; its
        cluster() is then a checkpoint for resume)."""
        st = Stats()
        if max_passes > 0:
            _check(lib().gsdr_job_run_limited(self._h, max_passes, C.byref(st)))
        else:
            _check(lib().gsdr_job_run(self._h, C.byref(st)))
        return st

    def resume(self, checkpoint: np.ndarray, max_passes: int = 0) -> Stats:
        """gsdr_job_resume: continues the unfinished clustering `checkpoint`
        (a cluster array, -1 = unclustered) for max_passes more passes or
        rounds (0: to the end)."""
        cp = np.ascontiguousarray(checkpoint, dtype=np.int32)
        if len(cp) != self.n:
            raise GsdrError(EINVAL, "checkpoint size differs from the job's read count")
        st = Stats()
        _check(lib().gsdr_job_resume(self._h, cp.ctypes.data, max_passes, C.byref(st)))
        return st

    def cluster(self) -> np.ndarray:
        cl = np.empty(max(self.n, 1), dtype=np.int32)
        _check(lib().gsdr_job_cluster(self._h, cl.ctypes.data))
        return cl[: self.n]

    def close(self):
        if self._h:
            lib().gsdr_job_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _host_bytes(data):
    """(pointer, size) of FASTA bytes given as bytes or as a uint8 numpy array
    (for example a view of pinned host memory, whose copy to the device is
    faster than a copy from pageable memory)."""
    if isinstance(data, bytes):
        return C.cast(C.c_char_p(data), C.c_void_p), len(data)
    a = np.asarray(data)
    if a.dtype != np.uint8 or a.ndim != 1 or not a.flags.c_contiguous:
        raise TypeError("FASTA bytes: bytes or a contiguous 1-D uint8 array")
    return C.c_void_p(a.ctypes.data), a.nbytes


class _Result:
    """Owns a gsdr_result; views over its buffers keep it alive."""

    def __init__(self, h):
        self.h = h

    def __del__(self):
        if self.h:
            lib().gsdr_result_free(self.h)
            self.h = None


def _view(owner, addr, n, ctype, dtype):
    """A numpy array over n ctype items at addr that keeps `owner` alive."""
    if n == 0:
        return np.empty(0, dtype=dtype)
    buf = (ctype * n).from_address(addr)
    buf._owner = owner
    return np.frombuffer(buf, dtype=dtype)


def cluster_fasta(data, opts: Opts | None = None, stats: bool = False, copy: bool = True,
                  **kw):
    """readFile + clustering + saveFile on the device (gsdr_cluster_fasta):
    FASTA bytes in (bytes, or a uint8 array such as a view of pinned host
    memory); returns (output FASTA bytes, cluster[] in sorted order, the sort
    permutation), and the Stats when stats=True.  copy=False returns the output
    as a uint8 array and the two int32 arrays as views of the library's result
    buffers (no host copy; the result lives as long as any of them)."""
    o = opts if opts is not None else default_opts()
    for k, v in kw.items():
        setattr(o, k, v)
    st = Stats()
    h = C.c_void_p()
    ptr, size = _host_bytes(data)
    _check(lib().gsdr_cluster_fasta(ptr, size, C.byref(o), C.byref(h), C.byref(st)))
    if not copy:
        res = _Result(h)
        p, n = C.c_void_p(), C.c_int64()
        _check(lib().gsdr_result_output(h, C.byref(p), C.byref(n)))
        cnt = lib().gsdr_result_count(h)
        out = _view(res, p.value or 0, n.value, C.c_uint8, np.uint8)
        cl = _view(res, lib().gsdr_result_cluster(h) or 0, cnt, C.c_int32, np.int32)
        order = _view(res, lib().gsdr_result_order(h) or 0, cnt, C.c_int32, np.int32)
        return (out, cl, order, st) if stats else (out, cl, order)
    try:
        ptr, n = C.c_void_p(), C.c_int64()
        _check(lib().gsdr_result_output(h, C.byref(ptr), C.byref(n)))
        out = C.string_at(ptr.value, n.value) if n.value else b""
        cnt = lib().gsdr_result_count(h)

        def arr(fn):
            a = np.empty(cnt, dtype=np.int32)
            if cnt:
                C.memmove(a.ctypes.data, getattr(lib(), fn)(h), 4 * cnt)
            return a

        cl, order = arr("gsdr_result_cluster"), arr("gsdr_result_order")
    finally:
        lib().gsdr_result_free(h)
    return (out, cl, order, st) if stats else (out, cl, order)


def cluster_bytes(data: bytes, **kw) -> bytes:
    """FASTA bytes in, representative FASTA bytes out (one call)."""
    f = Fasta.parse(data)
    try:
        cl = clustering(f, **kw)
        return f.format(cl)
    finally:
        f.close()


def lcs_decide(seqs, pairs, t, mapping=0, greedy=0):
    """Alignment stage alone (include/gsdr_testing.h): seqs is a list of
    byte strings, pairs a list of (pattern, text) indices (each pattern at
    most once).  Returns (accept array, device ms)."""
    data = b"".join(seqs)
    off = np.zeros(len(seqs), dtype=np.int64)
    if len(seqs) > 1:
        off[1:] = np.cumsum([len(x) for x in seqs])[:-1]
    ln = np.array([len(x) for x in seqs], dtype=np.int32)
    pat = np.ascontiguousarray([p for p, _ in pairs], dtype=np.int32)
    txt = np.ascontiguousarray([x for _, x in pairs], dtype=np.int32)
    acc = np.zeros(len(pairs), dtype=np.uint8)
    ms = C.c_double()
    _check(lib().gsdr_lcs_decide(data, len(data), off.ctypes.data, ln.ctypes.data, len(seqs),
                                 pat.ctypes.data, txt.ctypes.data, len(pairs), C.c_float(t),
                                 mapping, greedy, acc.ctypes.data, C.byref(ms)))
    return acc, ms.value


def lcs_decide_noalloc(d_packed, d_pack_off, d_len_raw, d_len_gf, n_seq, d_pat, d_txt,
                       n_pairs, t, d_accept, stream=None):
    """gsdr_lcs_decide_noalloc on device pointers (integers); raises on error."""
    _check(lib().gsdr_lcs_decide_noalloc(d_packed, d_pack_off, d_len_raw, d_len_gf, n_seq,
                                         d_pat, d_txt, n_pairs, C.c_float(t), d_accept, stream))


def set_spin_limit(polls, device=0):
    """gsdr_set_spin_limit: polls each bounded device-side wait of the
    alignment kernels makes before giving up (None or < 0: the default)."""
    _check(lib().gsdr_set_spin_limit(device, -1 if polls is None else int(polls)))


class Server:
    """Continuous batching of clustering jobs on one GPU (gsdr_server_*)."""

    def __init__(self, device=0, max_inflight=4, mem_budget=0, batch=0, express_bytes=0):
        so = ServerOpts(device, max_inflight, mem_budget, batch, express_bytes)
        h = C.c_void_p()
        _check(lib().gsdr_server_create(C.byref(so), C.byref(h)))
        self._h = h

    def submit(self, fasta, threshold: float) -> int:
        """Queues a job: FASTA as bytes or a contiguous uint8 array (copied by
        the server); returns its id."""
        j = C.c_int64()
        if isinstance(fasta, np.ndarray):
            a = np.ascontiguousarray(fasta, dtype=np.uint8)
            ptr, n = C.cast(a.ctypes.data, C.c_char_p), a.size
        else:
            ptr, n = fasta, len(fasta)
        _check(lib().gsdr_server_submit(self._h, ptr, n, C.c_float(threshold), C.byref(j)))
        return j.value

    def wait(self, timeout_ms=-1):
        """Next finished job: (id, status, latency_ms), or None on timeout."""
        j, st, lat = C.c_int64(), C.c_int32(), C.c_double()
        rc = lib().gsdr_server_wait(self._h, timeout_ms, C.byref(j), C.byref(st), C.byref(lat))
        if rc == ETIMEOUT:
            return None
        _check(rc)
        return j.value, st.value, lat.value

    def result(self, job):
        """(representative FASTA bytes, cluster array) of a finished job."""
        need, n = C.c_int64(), C.c_int32()
        _check(lib().gsdr_server_result(self._h, job, None, 0, C.byref(need), None, C.byref(n)))
        buf = C.create_string_buffer(max(need.value, 1))
        cl = np.empty(max(n.value, 1), dtype=np.int32)
        _check(lib().gsdr_server_result(self._h, job, buf, need.value, C.byref(need),
                                        cl.ctypes.data, C.byref(n)))
        return buf.raw[: need.value], cl[: n.value]

    def times(self, job):
        """(queued_ms, run_ms) of a finished job (gsdr_server_times)."""
        q, r = C.c_double(), C.c_double()
        _check(lib().gsdr_server_times(self._h, job, C.byref(q), C.byref(r)))
        return q.value, r.value

    def release(self, job):
        _check(lib().gsdr_server_release(self._h, job))

    def close(self):
        if self._h:
            lib().gsdr_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def main(argv) -> int:
    """main (cuda-version/main.cu:3-36)."""
    args = [b"cluster"] + [a.encode() if isinstance(a, str) else a for a in argv]
    arr = (C.c_char_p * len(args))(*args)
    return lib().gsdr_main(len(args), arr)


# ---- synthetic workloads ---------------------------------------------------------

def synth_config(config: int, n_reads: int | None = None, seed: int | None = None,
                 **kw) -> SynthCfg:
    c = SynthCfg()
    synth_lib().gsdr_synth_preset(config, C.byref(c))
    if n_reads is not None and n_reads != c.n_reads:
        c.n_seeds = max(1, int(round(c.n_seeds * n_reads / c.n_reads)))
        c.n_reads = n_reads
    if seed is not None:
        c.seed = seed
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def synth_fasta(config: int, n_reads: int | None = None, seed: int | None = None, **kw) -> bytes:
    c = synth_config(config, n_reads, seed, **kw)
    p = C.c_void_p()
    n = C.c_int64()
    r = synth_lib().gsdr_synth_generate(C.byref(c), C.byref(p), C.byref(n))
    if r < 0:
        raise GsdrError(EINVAL, f"synthetic generator failed ({r})")
    try:
        return C.string_at(p.value, n.value)
    finally:
        synth_lib().gsdr_synth_free(p)
