"""Empirical choice of the execution knobs through the library's own
autotuner (gsdr_autotune, include/gsdr.h; csrc/autotune.cu): R_max
(tentative representatives per pass), the word filter's form (per-tentative
tables, inverted k-mer index, k-mer presence bitmaps), the band tiles of the
banded alignment kernels, the block shape (CTAs per SM of the alignment and
filter kernels) and the staging depth (passes per CUDA-graph launch).  Every
setting gives the same clusters (the decisions are pure functions of each
pair), so the choice only moves time.

Each candidate setting runs the job itself, on the device-resident reads, for
its first representatives only: the early passes, where the remaining reads
are still all there, cost the most.  The chosen setting is stored in the
tuning cache, which later automatic jobs (batch 0) in the same workload
bucket read by themselves -- the `cluster` executable included.
"""
from __future__ import annotations

import ctypes as C
import json

from . import Fasta, Opts, _check, default_opts, lib

FORMS = {0: "automatic", 1: "tables", 2: "index", 3: "bitmaps"}
KNOBS = ("batch", "word_filter", "group_words", "band_serial", "align_blocks", "filter_blocks",
         "graph_steps")


def autotune(data: bytes, threshold: float, reps: int | None = None, runs: int = 2,
             device: int = 0, cache_path: str | None = None, **opts):
    """Runs gsdr_autotune on a FASTA text.  Returns {"best": {...}, "trials":
    [...], "bucket", "gpu", "cache", "reps"}; best/trials carry the knobs,
    the passes and representatives timed and ms / us per representative.
    cache_path None: the default cache; "": store nothing."""
    f = Fasta.parse(data)
    try:
        o = default_opts(threshold=threshold, device=device, **opts)
        best = Opts()
        need = C.c_int64()
        cp = None if cache_path is None else cache_path.encode()
        buf = C.create_string_buffer(1 << 20)
        _check(lib().gsdr_autotune(C.byref(f.view), C.byref(o), reps or 0, runs, cp,
                                   C.byref(best), buf, len(buf), C.byref(need)))
        rep = json.loads(buf.value.decode())
    finally:
        f.close()
    rep["best_opts"] = {k: getattr(best, k) for k in KNOBS}
    return rep


def tuned_opts(result, threshold: float, **kw):
    """gsdr_opts for the setting autotune chose."""
    b = result["best"]
    return default_opts(threshold=threshold, **{k: b.get(k, 0) for k in KNOBS}, **kw)
