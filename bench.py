"""Benchmark: greedy exact-identity clustering of the 200k-read workload
(lognormal lengths, median 1500 bp, 40k seeds, t = 0.95) on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--config 1] [--reads N] [--batch R] [--no-cpu]
                    [--plain-steps K] [--serving-jobs J] [--autotune] [--stage-run]

One step = one full clustering of the workload (preparation kernels + every
round).  Prints one JSON line.
  value      sequences/s with the reads already in HBM (gsdr_job_run, CUDA
             events on the job's stream), batched form;
  e2e        sequences/s from FASTA bytes in pinned host memory to output FASTA
             bytes in host memory (gsdr_cluster_fasta: H2D of the file, device
             parse, host std::sort, clustering, device formatting, D2H of the
             output inside the timing); e2e.pre_parsed: gsdr_cluster on reads
             parsed by the host reader;
  plain      the one-representative-per-round form on the same reads, and
             the batched / plain ratio;
  serving    a Poisson stream of jobs through gsdr_server: p50 / p99 job
             latency and aggregate sequences/s;
  roofline   the filter stage (HBM) and align_roofline the alignment stage
             (integer ALU, GCUPS) from a stage-timed run;
  cpu_baseline  the oracle (CPU restatement of the reference path) on the
             host cores, on the same workload.
--impl reference times the oracle alone (the reference has no CPU path of its
own) and prints its line.  --stage-run runs one stage-timed clustering only
(with GSDR_TRACE=1 a line per pass on stderr): the run the ncu captures in
profiles/ use.  Under torchrun each rank clusters an independent replica (the
path keeps one GPU per job), rank 0 prints.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "gene-sequences-de-redundancy_gb300"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

CONFIG_NAMES = {
    0: "10k reads, 200-1000 bp, t=0.95",
    1: "200k reads, lognormal median 1500 bp sigma 0.5 (300-10000), 40k seeds, t=0.95",
    2: "2M reads of 150 bp, 300k seeds, t=0.90",
    3: "300k reads, log-uniform 2-30 kbp, 60k seeds, t=0.80",
}
CONFIG_T = {0: 0.95, 1: 0.95, 2: 0.90, 3: 0.80}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        loaded = [x for x in sm if smax and x > 0.5 * smax] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def key_figures():
    """`name: value` lines of profiles/key_figures.txt (figures read from ncu
    captures; the commands are in the per-kernel summaries beside it)."""
    out = {}
    try:
        with open(os.path.join(ROOT, "profiles", "key_figures.txt")) as fh:
            for ln in fh:
                ln = ln.split("#", 1)[0].strip()
                if ":" in ln:
                    k, v = ln.split(":", 1)
                    v = v.strip()
                    try:
                        out[k.strip()] = float(v)
                    except ValueError:
                        out[k.strip()] = v
    except OSError:
        pass
    return out


def libstdcxx_loaded():
    """File name of the libstdc++ this process loaded (its version suffix):
    the host sort reproduces std::sort's permutation with that library's own
    introsort steps, so the version goes into the line."""
    try:
        with open("/proc/self/maps") as fh:
            for ln in fh:
                if "libstdc++" in ln:
                    return os.path.realpath(ln.split()[-1]).rsplit("/", 1)[-1]
    except OSError:
        pass
    return None


def heaviest_launch(nbytes, ms, peak):
    """The filter launch that read the most input bytes in a stage-timed run:
    its bytes, event-timed duration and bandwidth against the HBM peak."""
    if not nbytes or not ms:
        return None
    gbs = nbytes / (ms * 1e-3) / 1e9
    return {"input_bytes": nbytes, "ms": ms, "achieved": gbs, "unit": "GB/s",
            "frac": gbs / peak if peak else None}


def filter_roofline(r, figures):
    """The filter stage against HBM: its input bytes (each remaining
    candidate's k-mer list, or bitmap, plus 28 bytes, once per launch) over
    the stage's event-timed launch durations; traffic = ncu's DRAM bytes per
    input byte for the same kernel on this workload (profiles/), scaled to
    this run's bytes per launch."""
    launches = max(1, r["filter_launches"])
    per_launch = r["filter_bytes"] / launches
    achieved = r["filter_gbs"]
    form = {0: "table", 1: "index", 2: "bits", 3: "masks"}.get(r["word_index"], "table")
    kernel = {"table": "k_bfilter_tab (per-tentative k-mer tables in shared memory, "
                       "transposed, paired 16-bit min/add)",
              "index": "k_bindex + k_bfilter_idx (inverted k-mer index in shared memory)",
              "bits": "k_bfilter_bits + k_bexact_t (two-level k-mer count bitmaps: AND + POPC "
                      "per tentative, exact sums for the pairs the bound leaves open, grouped "
                      "by tentative)",
              "masks": "k_bmask + k_bfilter_mask + k_bexact_t (per-k-mer rows of tentative "
                       "bits in L2, bit-sliced counts per candidate, exact sums for the pairs "
                       "the bound leaves open, grouped by tentative)"}[form]
    ratio = figures.get("c%d.filter_%s.dram_over_input" % (r["config"], form))
    return {"bound": "hbm", "kernel": kernel,
            "achieved": achieved, "peak": r["peak"], "unit": "GB/s",
            "frac": achieved / r["peak"] if r["peak"] else None,
            "peak_source": r["peak_kind"] + " (MEASURED_PEAKS.json hbm_gbs)"
            if r["peak_kind"] == "measured" else r["peak_kind"],
            "traffic": per_launch * ratio if isinstance(ratio, float) else None,
            "input_bytes_per_launch": per_launch, "launches": launches,
            "stage_ms": r["filter_ms"],
            "heaviest_launch": heaviest_launch(r["filter_max_bytes"], r["filter_max_ms"],
                                               r["peak"]),
            "measured_bound": measured_filter_bound(form, figures),
            "note": "R tentatives per streamed byte: the measured bound is on chip "
                    "(measured_bound, ncu), not HBM"}


def measured_filter_bound(form, figures):
    """The filter kernel's binding resource as ncu measured it (profiles/)."""
    if form == "table" and figures.get("c1.filter_table.l1tex_pct") is not None:
        return {"resource": "L1TEX / shared memory", "kernel": "k_bfilter_tab<6>",
                "l1tex_pct_of_peak": figures["c1.filter_table.l1tex_pct"],
                "smem_roofline_frac": figures.get(
                    "c1.filter_table.smem_wavefronts_per_sm_cycle"),
                "bank_conflict_wavefront_share": figures.get(
                    "c1.filter_table.bank_conflict_wavefront_share"),
                "source": "profiles/k_bfilter_tab_c1_smem.md (200k-read workload)"}
    if form == "bits" and figures.get("c1.filter_bits.alu_pipe_pct") is not None:
        return {"resource": "POPC (XU) and ALU pipes", "kernel": "k_bfilter_bits<6>",
                "sm_throughput_pct": figures.get("c1.filter_bits.sm_throughput_pct"),
                "xu_pipe_pct": figures.get("c1.filter_bits.xu_pipe_pct"),
                "alu_pipe_pct": figures["c1.filter_bits.alu_pipe_pct"],
                "ipc_of_4": figures.get("c1.filter_bits.ipc"),
                "dram_pct_of_peak": figures.get("c1.filter_bits.dram_pct"),
                "source": "profiles/k_bfilter_bits_c1.md (200k-read workload)"}
    if form == "masks" and figures.get("c2.filter_masks.ipc") is not None:
        return {"resource": "ALU pipe and L2 latency", "kernel": "k_bfilter_mask",
                "ipc_of_4": figures["c2.filter_masks.ipc"],
                "alu_pipe_pct": figures.get("c2.filter_masks.alu_pipe_pct"),
                "l2_pct_of_peak": figures.get("c2.filter_masks.l2_pct"),
                "dram_pct_of_peak": figures.get("c2.filter_masks.dram_pct"),
                "source": "profiles/k_bfilter_mask_c2_300k.md (2M-read workload slice)"}
    if form == "index" and figures.get("c2.filter_index.ipc") is not None:
        return {"resource": "instruction issue", "kernel": "k_bfilter_idx<7>",
                "ipc_of_4": figures["c2.filter_index.ipc"],
                "alu_pipe_pct": figures.get("c2.filter_index.alu_pipe_pct"),
                "source": "profiles/k_bfilter_idx_c2_300k.md (2M-read workload slice)"}
    return None


def align_roofline(r, figures):
    """The alignment stage is integer-ALU bound (bit-parallel LCS): GCUPS over
    the full-DP cells of the pairs it decides, and the ALU pipe utilisation
    ncu measured for its dominant kernel."""
    ms = r["align_ms"]
    done = r.get("cells_computed") or 0.0
    return {"bound": "int_alu", "kernel": "k_align_single / k_align",
            "gcups": r["gcups"], "stage_ms": ms, "cells": r["stats"]["cells"],
            "gcups_note": "cells = full-DP q x T of every aligned pair (the reference's DP "
                          "work); early exits, bands and the greedy bound skip most of them",
            "cells_computed": done,
            "computed_over_full_dp": done / r["stats"]["cells"] if r["stats"]["cells"] else None,
            "computed_gcups": done / (ms * 1e-3) / 1e9 if ms > 0 else None,
            "alu_pipe_pct_ncu": figures.get("align.alu_pipe_pct"),
            "ipc_ncu": figures.get("align.ipc")}


def pinned_host_copy(data: bytes):
    """The bytes in a page-locked host buffer (a torch uint8 tensor; keep it
    alive while its numpy view is in use), or None without CUDA."""
    try:
        import numpy as np
        import torch

        if not torch.cuda.is_available():
            return None
        t = torch.empty(len(data), dtype=torch.uint8, pin_memory=True)
        t.numpy()[:] = np.frombuffer(data, dtype=np.uint8)
        return t
    except Exception:
        return None


def oracle_lib():
    import oracle_binding

    oracle_binding.build()
    return oracle_binding


def cpu_run(data_path, t, threads):
    """The oracle on a FASTA file: (seconds, sort permutation, cluster array)."""
    orc = oracle_lib()
    t0 = time.perf_counter()
    order, cl, st = orc.run(data_path, None, t=t, threads=threads)
    dt = time.perf_counter() - t0
    return dt, order, cl


def write_workload(cfg, n_reads, seed, path):
    import gsdr

    c = gsdr.synth_config(cfg, n_reads, seed)
    n = gsdr.synth_lib().gsdr_synth_write(c, os.fsencode(path))
    if n < 0:
        raise RuntimeError("workload generation failed")
    return n


SERVING_T = (0.80, 0.85, 0.90, 0.95, 1.00)


def _record_ends(data):
    """Byte offset after each record of a single-line FASTA buffer."""
    import numpy as np

    a = np.frombuffer(data, dtype=np.uint8)
    starts = np.flatnonzero(a == ord(">"))
    return np.append(starts[1:], len(a))


def serving_jobs(args):
    """The serving workload's job stream: Poisson arrivals (args.serving_rate
    per second), threshold uniform over 0.80 .. 1.00, jobs of the 10k-read
    recipe with 150-5000 bp reads.  Jobs at t >= 0.88 (word filter on) draw
    their size log-uniform over 1k-200k reads, as the recipe says; jobs at
    t <= 0.879 turn the filters off (the reference's drop mode), which makes a
    job quadratic in its size, so they draw 300-1.5k reads of at most 2000 bp.
    A job of n reads is the first n records of one pre-generated file of the
    recipe (records are in random order, so a prefix is a sample of it); t =
    1.00 jobs are refused as the reference refuses them.  Returns (jobs as
    (payload array, t, n), gaps in seconds, recipe text)."""
    import gsdr
    import numpy as np

    rng = np.random.default_rng(20261207)
    big = gsdr.synth_fasta(4, n_reads=200000, seed=4100, n_seeds=40000, len_lo=150,
                           len_hi=5000)
    small = gsdr.synth_fasta(4, n_reads=1500, seed=4200, n_seeds=300, len_lo=150, len_hi=2000)
    pools = {}
    for key, data in (("filter", big), ("drop", small)):
        pools[key] = (np.frombuffer(data, dtype=np.uint8), _record_ends(data))
    jobs = []
    for i in range(args.serving_jobs):
        t = float(SERVING_T[rng.integers(0, len(SERVING_T))])
        drop = t < 0.88
        lo, hi = (300, 1500) if drop else (1000, 200000)
        n = int(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        arr, ends = pools["drop" if drop else "filter"]
        jobs.append((arr[: ends[n - 1]], t, n))
    gaps = rng.exponential(1.0 / args.serving_rate, len(jobs))
    recipe = ("Poisson arrivals; jobs of the 10k-read recipe, 150-5000 bp, t in "
              "{0.80,0.85,0.90,0.95,1.00}; sizes 1k-200k reads for t >= 0.88, 300-1.5k reads "
              "of <= 2000 bp for t <= 0.879 (alignment only, quadratic); each job the first n "
              "records of one generated file of the recipe")
    return jobs, gaps, recipe


def serve_stream(jobs, gaps, device, max_inflight, express_bytes=0):
    """Submits the jobs at their arrival times (gaps None: all at once) and
    waits for all.  Returns per-job (status, latency, run_ms, reads), wall s.
    express_bytes: the server's express slot (0: its default, -1: none)."""
    import gsdr

    srv = gsdr.Server(device=device, max_inflight=max_inflight, express_bytes=express_bytes)
    lat, status, run, results = {}, {}, {}, {}
    ids = []
    first = set()  # the first three jobs: their results are kept for the oracle check

    def done(r):
        # a finished job's times, then its result released at once (a long
        # stream would otherwise hold every job's output in host memory)
        jid = r[0]
        lat[jid], status[jid] = r[2], r[1]
        run[jid] = srv.times(jid)[1]
        if jid in first and r[1] == 0:
            results[jid] = srv.result(jid)[1]
        srv.release(jid)

    t0 = time.perf_counter()
    try:
        due = t0
        for k, (data, t, n) in enumerate(jobs):
            if gaps is not None:
                due += gaps[k]
                while True:
                    now = time.perf_counter()
                    if now >= due:
                        break
                    r = srv.wait(int((due - now) * 1000) + 1)
                    if r:
                        done(r)
            jid = srv.submit(data, t)
            if k < 3:
                first.add(jid)
            ids.append((jid, n))
        while len(lat) < len(ids):
            r = srv.wait(600000)
            if r is None:
                break
            done(r)
        wall = time.perf_counter() - t0
    finally:
        srv.close()
    rows = [(status.get(j), lat.get(j), run.get(j), n, jobs[k][1]) for k, (j, n) in enumerate(ids)]
    return rows, wall, results


def serving_run(args, device):
    """The serving stream through gsdr_server (continuous batching: jobs
    admitted by device footprint as slots free up, each on its own stream):
    p50 / p99 job latency, aggregate sequences/s, and two measures of overlap
    -- jobs running at once on average (sum of the jobs' run times over the
    stream's wall time) and the same 32 jobs submitted at once with 1 slot
    against 4 slots (wall-time ratio: > 1 means the device ran jobs side by
    side).  The first jobs' results are checked against the oracle."""
    import numpy as np

    jobs, gaps, recipe = serving_jobs(args)
    rows, wall, results = serve_stream(jobs, gaps, device, 4)
    ok = [r for r in rows if r[0] == 0]
    ls = np.array([r[1] for r in ok]) if ok else np.array([0.0])
    busy = sum(r[2] for r in ok if r[2] is not None) / 1e3
    done_reads = sum(r[3] for r in ok)
    # overlap: 32 filter-mode jobs of the stream of at most 20k reads (jobs too
    # small to fill the device alone), all submitted at once
    burst = [j for j in jobs if 0.88 <= j[1] < 1.0 and j[2] <= 20000][:32]
    # (the express slot off: the slots alone decide how many jobs run at once)
    _, wall1, _ = serve_stream(burst, None, device, 1, express_bytes=-1)
    _, wall4, _ = serve_stream(burst, None, device, 4, express_bytes=-1)
    # a sample of served results against the oracle
    checked, match = 0, True
    try:
        import tempfile

        import oracle_binding

        with tempfile.TemporaryDirectory() as td:
            for k, cl in results.items():
                data, t, n = jobs[k - 1]
                if n > 20000:
                    continue
                _, ocl, _, _ = oracle_binding.run_bytes(data.tobytes(), td, t=t)
                checked += 1
                match = match and len(ocl) == len(cl) and bool((ocl == cl).all())
    except Exception as e:  # the checker is optional here; say why it did not run
        match = f"not checked: {e}"
    by_t = {}
    for r in ok:
        b = by_t.setdefault(f"{r[4]:.2f}", {"jobs": 0, "reads": 0, "run_ms": 0.0,
                                             "max_run_ms": 0.0, "latency_ms": 0.0})
        b["jobs"] += 1
        b["reads"] += r[3]
        b["run_ms"] += r[2] or 0.0
        b["max_run_ms"] = max(b["max_run_ms"], r[2] or 0.0)
        b["latency_ms"] += r[1]
    for b in by_t.values():
        b["mean_run_ms"] = b.pop("run_ms") / b["jobs"]
        b["mean_latency_ms"] = b.pop("latency_ms") / b["jobs"]
    return {
        "jobs": len(rows), "completed": len(ok), "by_threshold": by_t,
        "rejected_t1": sum(1 for r in rows if r[0] == 1),
        "failed": sum(1 for r in rows if r[0] not in (0, 1)),
        "arrival_rate_per_s": args.serving_rate,
        "p50_latency_ms": float(np.percentile(ls, 50)),
        "p99_latency_ms": float(np.percentile(ls, 99)),
        "seqs_per_s": done_reads / wall, "reads": done_reads,
        "wall_s": wall, "max_inflight": 4, "express_slot_bytes": 4 << 20,
        "order": "smallest queued job first, a job waiting 1 s or more first",
        "mean_jobs_running": busy / wall if wall > 0 else None,
        "burst": {"jobs": len(burst), "wall_s_1_slot": wall1, "wall_s_4_slots": wall4,
                  "overlap_speedup": wall1 / wall4 if wall4 > 0 else None},
        "oracle_checked": checked, "oracle_match": match,
        "recipe": recipe,
    }


def combine_ranks(r, world):
    """Replicas: every rank clustered its own copy of the workload; the job's
    time per step is the slowest rank's (max over ranks, gloo), so value =
    all ranks' reads / that time.  Rank 0 then prints."""
    if world <= 1:
        return r
    import torch
    import torch.distributed as dist

    keys = [k for k in ("ms_step", "e2e_ms", "reads_ms") if k in r]
    t = torch.tensor([r[k] for k in keys], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    for i, k in enumerate(keys):
        r[k] = float(t[i])
    dist.barrier()
    return r


def config_line(args, n, t, world):
    """The `config` object of both arms' lines (same keys, same values)."""
    return {"workload": CONFIG_NAMES[args.config], "reads": n, "threshold": t,
            "form": "plain" if args.batch == 1 else f"batched R={args.batch}",
            "parallelism": f"replicas x{world}",
            "l2": "inputs larger than L2 (sequence bytes + k-mer tables > 1 GB per step)"}


def bench_reference(args, rank, world):
    """--impl reference: the oracle (CPU restatement) on the host cores."""
    if rank != 0:
        return None
    import gsdr  # noqa: F401  (generator)

    threads = os.cpu_count() or 1
    path = os.path.join("/tmp", f"gsdr_bench_c{args.config}_{os.getpid()}.fa")
    n = write_workload(args.config, args.reads, args.seed, path)
    t = CONFIG_T[args.config]
    times = []
    for i in range(args.warmup + args.steps):
        dt, _, _ = cpu_run(path, t, threads)
        if i >= args.warmup:
            times.append(dt)
    os.unlink(path)
    sec = sum(times) / len(times)
    value = n / sec
    return {
        "metric": "seqs/sec", "value": value, "unit": "seqs/s", "n_gpus": 0, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "impl": "reference",
        "config": config_line(args, n, t, 1),
        "cpu_baseline": {"value": value, "unit": "seqs/s", "cores": threads, "kind": "port",
                         "sample": f"whole workload ({n} reads) per step; the reference has "
                                   "no CPU path, so its restatement (oracle) runs"},
        "e2e": {"value": value, "unit": "seqs/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def bench_ours(args, rank, world, local):
    import gsdr

    device = local if world > 1 else 0
    data = gsdr.synth_fasta(args.config, args.reads, args.seed)
    t = CONFIG_T[args.config]
    f = gsdr.Fasta.parse(data)
    n = f.n
    opts = gsdr.default_opts(threshold=t, device=device, batch=args.batch)
    tune = None
    if args.autotune and args.batch == 0:
        # the library's autotuner times the knobs on the job's first
        # representatives and stores the winner in the tuning cache; the
        # automatic job below (batch 0) then takes it from there by itself
        from gsdr.autotune import autotune

        t_tune = time.perf_counter()
        rep = autotune(data, t, device=device)
        auto = [x for x in rep["trials"] if x.get("stage") == "R x form" and x.get("batch") == 0
                and x.get("word_filter") == 0 and "us_per_rep" in x]
        tune = {"best": rep["best"], "trials": len(rep["trials"]), "bucket": rep["bucket"],
                "gpu": rep["gpu"], "cache": rep["cache"], "reps_timed": rep["reps"],
                "automatic_us_per_rep": auto[0]["us_per_rep"] if auto else None,
                "seconds": time.perf_counter() - t_tune}
    h2d = f.view.n_bytes + n * 8 + n * 4 + 2 * (n + 1) * 8
    d2h = n * 4

    # value: device-resident input
    job = gsdr.Job(f, opts)
    for _ in range(args.warmup):
        job.run()
    clocks = ClockSampler(device)
    clocks.start()
    dev_ms = []
    launches = 0
    last = None
    for _ in range(args.steps):
        st = job.run()
        dev_ms.append(st.ms_prep + st.ms_cluster)
        launches += st.kernel_launches
        last = st
    clock_info = clocks.stop()
    cl_dev = job.cluster()
    job.close()
    order_dev = f.order().copy()

    # e2e: FASTA bytes in host memory to output FASTA bytes in host memory
    # through gsdr_cluster_fasta (parse on the device, the host std::sort,
    # clustering, output formatting on the device; H2D of the file, D2H of
    # the lengths, the output and the cluster array inside the timing)
    # the FASTA bytes sit in pinned host memory (filled once, outside the
    # timing), so each step's copy to the device is a DMA from page-locked memory
    pinned = pinned_host_copy(data)
    host_in = pinned.numpy() if pinned is not None else data
    # (copy=False: the output bytes and arrays stay in the library's result
    # buffers, in host memory, as a C caller would use them)
    for _ in range(min(args.warmup, 2)):
        gsdr.cluster_fasta(host_in, opts, copy=False)
    e2e_ms = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        out_view, cl, _ = gsdr.cluster_fasta(host_in, opts, copy=False)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    out_bytes = out_view.tobytes()
    same = bool((cl == cl_dev).all()) and out_bytes == f.format(cl_dev)
    # the same with pre-parsed reads (host reader) through gsdr_cluster
    reads_ms = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        gsdr.clustering(f, opts)
        reads_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_h2d = len(data) + n * 8 + n * 4
    e2e_d2h = n * 4 * 3 + len(out_bytes)

    # the plain form (one representative per round, the reference's loop) on
    # the same device-resident reads: the batched / plain ratio
    plain = None
    if args.batch != 1 and args.plain_steps > 0:
        pj = gsdr.Job(f, gsdr.default_opts(threshold=t, device=device, batch=1))
        pj.run()
        pms = []
        for _ in range(args.plain_steps):
            s = pj.run()
            pms.append(s.ms_prep + s.ms_cluster)
        plain = {"ms": sum(pms) / len(pms), "steps": len(pms),
                 "same": bool((pj.cluster() == cl_dev).all())}
        pj.close()
        # its filter stage (one representative per launch, HBM-shaped) from a
        # stage-timed run
        sp = gsdr.clustering(f, gsdr.default_opts(threshold=t, device=device, batch=1,
                                                  stage_timing=1), stats=True)[1]
        plain["filter_ms"] = sp.ms_filter
        plain["filter_bytes"] = sp.filter_bytes
        plain["filter_launches"] = sp.rounds
        plain["filter_max_bytes"] = sp.filter_max_bytes
        plain["filter_max_ms"] = sp.filter_max_ms

    serving = serving_run(args, device) if args.serving_jobs > 0 else None

    # stage-timed run for the roofline (events around each filter / align launch)
    st_t = gsdr.clustering(f, gsdr.default_opts(threshold=t, device=device, batch=args.batch,
                                                stage_timing=1), stats=True)[1]
    f.close()

    dev_ms_max = max(dev_ms)  # max over steps of this rank; max over ranks below
    ms_step = sum(dev_ms) / len(dev_ms)
    e2e_step = sum(e2e_ms) / len(e2e_ms)
    peak, peak_kind = measured_peaks()
    filt_gbs = st_t.filter_bytes / (st_t.ms_filter * 1e-3) / 1e9 if st_t.ms_filter > 0 else 0.0
    align_gcups = st_t.cells / (st_t.ms_align * 1e-3) / 1e9 if st_t.ms_align > 0 else 0.0
    return {
        "n": n, "ms_step": ms_step, "ms_step_max": dev_ms_max, "e2e_ms": e2e_step,
        "h2d": e2e_h2d, "d2h": e2e_d2h, "reads_ms": sum(reads_ms) / len(reads_ms),
        "reads_h2d": h2d, "reads_d2h": d2h, "launches_per_step": launches // max(1, args.steps),
        "stats": last.as_dict(), "clocks": clock_info, "same": same,
        "filter_gbs": filt_gbs, "filter_ms": st_t.ms_filter, "filter_bytes": st_t.filter_bytes,
        "filter_launches": st_t.passes if args.batch != 1 else st_t.rounds,
        "filter_max_bytes": st_t.filter_max_bytes, "filter_max_ms": st_t.filter_max_ms,
        "align_ms": st_t.ms_align, "gcups": align_gcups,
        "peak": peak, "peak_kind": peak_kind, "t": t, "plain": plain,
        "word_index": st_t.word_index, "r_max": st_t.batch, "config": args.config,
        "serving": serving, "autotune": tune, "cl_dev": cl_dev, "order_dev": order_dev,
        "cells_computed": st_t.cells_computed,
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=1)
    ap.add_argument("--reads", type=int, default=None)
    ap.add_argument("--seed", type=int, default=None)
    ap.add_argument("--batch", type=int, default=0,
                    help="0 = batched with adaptive R (up to the job's R_max, 1024 by "
                         "default); 1 = plain (one representative per round); R > 1 = R")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--serving-jobs", type=int, default=200,
                    help="jobs in the serving stream (p50/p99 latency); 0 = skip")
    ap.add_argument("--serving-rate", type=float, default=20.0, help="job arrivals per second")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="skip the autotuner (by default gsdr_autotune times R_max, the word "
                         "filter's form, band tiles, block shape and staging depth on the "
                         "job's first representatives before the timed runs, and the timed "
                         "automatic job takes the result from the tuning cache)")
    ap.add_argument("--stage-run", action="store_true",
                    help="one stage-timed clustering of the workload (CUDA events around "
                         "every filter and alignment launch; with GSDR_TRACE=1 a line per "
                         "pass on stderr), stats as JSON: the run the ncu captures use")
    ap.add_argument("--plain-steps", type=int, default=None,
                    help="timed runs of the plain form for the batched/plain ratio "
                         "(default 2 for the 10k and 200k workloads, else 0)")
    args = ap.parse_args()
    if args.plain_steps is None:
        args.plain_steps = 2 if args.config in (0, 1) else 0
    rank, world, local = dist_env()

    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    if args.impl == "reference":
        line = bench_reference(args, rank, world)
        if world > 1:
            dist.barrier()
        if rank == 0:
            print(json.dumps(line), flush=True)
        return

    import __graft_entry__

    __graft_entry__.build()
    if args.stage_run:
        import gsdr

        f = gsdr.Fasta.parse(gsdr.synth_fasta(args.config, args.reads, args.seed))
        _, st = gsdr.clustering(f, gsdr.default_opts(threshold=CONFIG_T[args.config],
                                                     batch=args.batch, stage_timing=1),
                                stats=True)
        f.close()
        print(json.dumps({"stage_run": CONFIG_NAMES[args.config], "batch": args.batch,
                          "stats": st.as_dict()}), flush=True)
        return
    if world > 1:
        dist.barrier()
    r = bench_ours(args, rank, world, local)
    combine_ranks(r, world)
    if rank != 0:
        return
    import numpy as np  # noqa: F401  (parity check below)

    n_total = r["n"] * world
    value = n_total / (r["ms_step"] * 1e-3)
    e2e = n_total / (r["e2e_ms"] * 1e-3)
    figures = key_figures()
    plain_line = None
    if r["plain"]:
        pv = n_total / (r["plain"]["ms"] * 1e-3)
        plain_line = {"value": pv, "unit": "seqs/s", "ms_per_step": r["plain"]["ms"],
                      "steps": r["plain"]["steps"], "batched_over_plain": value / pv,
                      "same_clusters": r["plain"]["same"]}
        if r["plain"].get("filter_ms"):
            pg = r["plain"]["filter_bytes"] / (r["plain"]["filter_ms"] * 1e-3) / 1e9
            plain_line["filter_roofline"] = {
                "bound": "hbm", "kernel": "k_filter (one representative per launch)",
                "achieved": pg, "peak": r["peak"], "unit": "GB/s",
                "frac": pg / r["peak"] if r["peak"] else None,
                "input_bytes_per_launch": r["plain"]["filter_bytes"] /
                max(1, r["plain"]["filter_launches"]),
                "launches": r["plain"]["filter_launches"], "stage_ms": r["plain"]["filter_ms"],
                "heaviest_launch": heaviest_launch(r["plain"]["filter_max_bytes"],
                                                   r["plain"]["filter_max_ms"], r["peak"]),
                "note": "bytes the filter reads: 28 per remaining candidate, its k-mer bitmap "
                        "and, where the bitmap bound leaves the pair open, its k-mer list. "
                        "The first round's representative (the longest read) absorbs most "
                        "reads; every later launch reads <= 75 MB and takes >= ~10 us of "
                        "dependent loads, so the stage average sits far below the heaviest "
                        "launch's bandwidth"}
    line = {
        "metric": "seqs/sec", "value": value, "unit": "seqs/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic",
        "config": config_line(args, r["n"], r["t"], world),
        "e2e": {"value": e2e, "unit": "seqs/s", "h2d_bytes_per_step": r["h2d"],
                "d2h_bytes_per_step": r["d2h"], "ms_per_step": r["e2e_ms"],
                "path": "gsdr_cluster_fasta: FASTA bytes in pinned host memory -> output FASTA "
                        "bytes (device parse)",
                "pre_parsed": {"value": n_total / (r["reads_ms"] * 1e-3),
                               "ms_per_step": r["reads_ms"],
                               "h2d_bytes_per_step": r["reads_h2d"],
                               "d2h_bytes_per_step": r["reads_d2h"],
                               "path": "gsdr_cluster on reads parsed by the host reader"}},
        "gpu_launches": r["launches_per_step"] * args.steps,
        "clocks": r["clocks"],
        "roofline": filter_roofline(r, figures),
        "align_roofline": align_roofline(r, figures),
        "dominant_kernel": figures.get("c%d.dominant_kernel" % args.config),
        "plain": plain_line,
        "serving": r["serving"],
        "autotune": r["autotune"],
        "stats": {k: r["stats"][k] for k in ("rounds", "passes", "pairs_prefilter", "pairs_word",
                                               "pairs_aligned", "pairs_accepted", "ms_prep",
                                               "ms_cluster", "word_index", "batch",
                                               "tuned")},
        "device_result_matches_e2e": r["same"],
        "host": {"libstdcxx": libstdcxx_loaded(), "cpu_cores": os.cpu_count()},
    }
    if not args.no_cpu:
        import tempfile

        with tempfile.TemporaryDirectory() as td:
            path = os.path.join(td, "w.fa")
            n = write_workload(args.config, args.reads, args.seed, path)
            threads = os.cpu_count() or 1
            dt, order, ocl = cpu_run(path, r["t"], threads)
        line["cpu_baseline"] = {"value": n / dt, "unit": "seqs/s", "cores": threads,
                                "kind": "port",
                                "sample": f"whole workload ({n} reads), one run"}
        # the oracle's result on the whole workload against the GPU's
        same = (len(ocl) == len(r["cl_dev"]) and bool((ocl == r["cl_dev"]).all())
                and bool((order == r["order_dev"]).all()))
        line["parity_vs_oracle"] = same
        line["parity_detail"] = {"reads": int(len(ocl)), "compared": "sort permutation and "
                                 "cluster array of every read, oracle vs device run",
                                 "representatives": int((ocl == np.arange(len(ocl))).sum())}
    print(json.dumps(line), flush=True)
    if line.get("parity_vs_oracle") is False:
        sys.exit("bench: the device result differs from the oracle's")


if __name__ == "__main__":
    main()
