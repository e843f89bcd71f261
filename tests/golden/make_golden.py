"""Runs the reference program itself (cuda-version/, built unmodified by
oracle/build_ref.sh on a GPU machine) on every golden case and records its
output: sha256 and size of the output FASTA and its record count, with the
sha256 of the input.  The oracle runs beside it and must agree.  Output:
tests/golden/reference_outputs.json (or the path given as argument).

    oracle/build_ref.sh stage        # where the reference tree is mounted
    oracle/build_ref.sh build        # on the GPU machine
    python tests/golden/make_golden.py [out.json] [case ...]

With case names, only those cases run and their entries are merged into the
existing output file.

    GSDR_REFERENCE=<reference tree> python tests/golden/make_golden.py --results

copies the reference's own output files (cuda-version/result.fasta and the
SYCL program's top-level result.fasta) into tests/golden/ as
ref_cuda_result.fasta.gz and ref_sycl_result.fasta.gz.
"""
import hashlib
import json
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "gene-sequences-de-redundancy_gb300"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import cases  # noqa: E402


def sha(b):
    return hashlib.sha256(b).hexdigest()


def ref_binary(max_len):
    for L in (2048, 12288):
        if max_len + 64 <= L:
            p = os.path.join(ROOT, "oracle", "_ref", f"cluster_ref_{L}")
            if os.path.exists(p):
                return p
    raise RuntimeError(f"no reference build for reads of {max_len} bases")


# root of the reference tree (read-only), for --results only
REFERENCE = os.environ.get("GSDR_REFERENCE", "")


def copy_results():
    import gzip

    if not REFERENCE:
        raise SystemExit("set GSDR_REFERENCE to the reference tree's root")

    for src, dst in (("cuda-version/result.fasta", "ref_cuda_result.fasta.gz"),
                     ("result.fasta", "ref_sycl_result.fasta.gz")):
        with open(os.path.join(REFERENCE, src), "rb") as f:
            data = f.read()
        with gzip.GzipFile(os.path.join(HERE, dst), "wb", mtime=0) as g:
            g.write(data)
        print(dst, len(data), sha(data))


def main():
    if sys.argv[1:] == ["--results"]:
        copy_results()
        return
    import oracle_binding

    out_path = sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "reference_outputs.json")
    only = sys.argv[2:]
    result = {}
    if only and os.path.exists(out_path):
        with open(out_path) as f:
            result = json.load(f)
    with tempfile.TemporaryDirectory() as td:
        for name, (spec, argv) in cases.CASES.items():
            if only and name not in only:
                continue
            data = cases.build_input(spec)
            inp = os.path.join(td, name + ".fa")
            with open(inp, "wb") as f:
                f.write(data)
            max_len = max((len(l) for l in data.split(b"\n") if not l.startswith(b">")), default=0)
            outp = os.path.join(td, name + ".out")
            t0 = time.time()
            r = subprocess.run([ref_binary(max_len), "i", inp, "o", outp] + argv,
                               capture_output=True, text=True, timeout=900, cwd=td)
            dt = time.time() - t0
            with open(outp, "rb") as f:
                ref_out = f.read()
            # the oracle on the same input and options
            opts = dict(zip(argv[0::2], argv[1::2]))
            oout = outp + ".oracle"
            oracle_binding.run(inp, oout, t=float(opts.get("t", 0.95)), w=int(opts.get("w", 0)),
                               d=int(opts.get("d", 3)), p=int(opts.get("p", 0)))
            with open(oout, "rb") as f:
                orc_out = f.read()
            result[name] = {
                "argv": argv,
                "input_sha256": sha(data),
                "input_bytes": len(data),
                "output_sha256": sha(ref_out),
                "output_bytes": len(ref_out),
                "records": ref_out.count(b"\n>") + (1 if ref_out.startswith(b">") else 0),
                "reference_seconds": round(dt, 2),
                "reference_rc": r.returncode,
                "oracle_matches": orc_out == ref_out,
            }
            print(name, result[name], flush=True)
    with open(out_path, "w") as f:
        json.dump(result, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
