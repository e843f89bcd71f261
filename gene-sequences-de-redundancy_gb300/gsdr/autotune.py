"""Empirical choice of the batched form's settings: R_max (tentative
representatives per pass), the word filter's form (per-tentative tables,
inverted k-mer index, k-mer presence bitmaps) and the band tiles of the
banded alignment kernels (the widest window the group-banded kernel takes,
and the serial work up to which a pair goes to the lane-per-pair banded
kernel).  Every setting gives the same clusters (the decisions are pure
functions of each pair), so the choice only moves time.

Each candidate setting runs the job itself, on the device-resident reads,
for the first representatives only (gsdr_job_run_limited): the early passes,
where the remaining reads are still all there, cost the most, and a sample
of the reads would not show their cost (a small job favours large R for its
few passes).  Settings are compared by time per representative over about
the same number of representatives.  The search is in two stages: R_max x
form first, then the band tiles with the best of those.
"""
from __future__ import annotations

import math

import numpy as np

from . import Fasta, Job, default_opts

R_VALUES = (64, 128, 256, 512, 1024)
FORMS = {0: "automatic", 1: "tables", 2: "index", 3: "bitmaps"}
# (group_words, band_serial) of the second stage; (0, 0) = the defaults, which
# the first stage already timed
TILES = ((0, 0), (-1, 0), (32, 0), (64, 0), (0, -1), (0, 4096), (0, 65536))


def sample_fasta(data: bytes, n_reads: int, seed: int = 1) -> bytes:
    """A seeded random subset of the records of a FASTA text (whole records,
    in file order)."""
    recs = data.split(b"\n>")
    if len(recs) <= n_reads:
        return data
    rng = np.random.default_rng(seed)
    keep = np.sort(rng.choice(len(recs), n_reads, replace=False))
    parts = [recs[i] if i == 0 else b">" + recs[i] for i in keep]
    out = b"\n".join(p.rstrip(b"\n") for p in parts) + b"\n"
    return out if out.startswith(b">") else b">" + out


def passes_for(r_max: int, reps: int) -> int:
    """Passes of a run whose R doubles from 1 up to r_max until about `reps`
    representatives are taken."""
    ramp = int(math.ceil(math.log2(max(r_max, 1)))) + 1
    return ramp + int(math.ceil(reps / max(r_max, 1)))


def _trial(f, threshold, r, form, tile, reps, device, runs, opts):
    """Times one setting on the first ~`reps` representatives; None when the
    setting does not apply (bitmaps above word length 6)."""
    gw, bs = tile
    o = default_opts(threshold=threshold, batch=r, word_filter=form, group_words=gw,
                     band_serial=bs, device=device, **opts)
    limit = passes_for(r if r else 256, reps)
    rec = {"batch": r, "word_filter": FORMS[form], "group_words": gw, "band_serial": bs}
    try:
        job = Job(f, o)
    except Exception as e:
        return dict(rec, error=str(e))
    try:
        job.run(limit)
        ms, taken = [], 0
        for _ in range(runs):
            st = job.run(limit)
            ms.append(st.ms_prep + st.ms_cluster)
            taken = st.rounds
        if form == 3 and st.word_index != 2:
            return None  # word length above 6: no bitmaps
        t = float(np.median(ms))
        return dict(rec, passes=limit, representatives=int(taken), ms=t,
                    ms_per_rep=t / max(1, taken))
    finally:
        job.close()


def autotune(data: bytes, threshold: float, reps: int | None = None, r_values=R_VALUES,
             forms=(0, 1, 2, 3), tiles=TILES, device: int = 0, runs: int = 2, **opts):
    """Times (R_max, word filter form) settings, then the band tiles with the
    best of them, on the job's first ~`reps` representatives (default: 8192
    or 1/20 of the reads, whichever is smaller) and returns
    {"best": {...}, "trials": [...]}.  Form 0 is the automatic choice with
    R_max 0 (automatic as well); the bitmap form only applies to word lengths
    up to 6."""
    f = Fasta.parse(data)
    n = f.n
    reps = reps if reps is not None else max(256, min(8192, n // 20))
    settings = [(0, 0)] + [(r, form) for form in forms if form for r in r_values]
    trials = []
    try:
        for r, form in settings:
            t = _trial(f, threshold, r, form, (0, 0), reps, device, runs, opts)
            if t is not None:
                trials.append(t)
        ok = [t for t in trials if "ms" in t]
        if ok and len(tiles) > 1:
            first = min(ok, key=lambda t: t["ms_per_rep"])
            inv = {v: k for k, v in FORMS.items()}
            for tile in tiles:
                if tuple(tile) == (0, 0):
                    continue
                t = _trial(f, threshold, first["batch"], inv[first["word_filter"]], tile, reps,
                           device, runs, opts)
                if t is not None:
                    trials.append(t)
    finally:
        f.close()
    ok = [t for t in trials if "ms" in t]
    best = min(ok, key=lambda t: t["ms_per_rep"]) if ok else None
    return {"best": best, "trials": trials, "representatives_timed": reps}


def tuned_opts(result, threshold: float, **kw):
    """gsdr_opts for the setting autotune chose."""
    b = result["best"]
    inv = {v: k for k, v in FORMS.items()}
    return default_opts(threshold=threshold, batch=b["batch"], word_filter=inv[b["word_filter"]],
                        group_words=b.get("group_words", 0), band_serial=b.get("band_serial", 0),
                        **kw)
