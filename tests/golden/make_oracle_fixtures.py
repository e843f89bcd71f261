"""Runs the oracle (oracle/gsdr_oracle.cpp, the CPU restatement of the
reference path, pinned to the reference program's own outputs by
reference_outputs.json) on workloads too large to re-run inside the GPU test
suite, and records what the GPU path must reproduce:
tests/golden/oracle_outputs.json.

Per case: the generator call that rebuilds the input byte for byte, the
input's sha256, the read count, the representative count, the number of
rounds, and the sha256 of
  * the sorted-order cluster array (int32, little endian) -- clustering /
    clusteringDrop's cluster[] (cuda-version/func.cu:1001-1097),
  * the sort permutation (int32, sorted index -> file position) -- readFile's
    std::sort (func.cu:94-117),
  * the output FASTA -- saveFile's bytes (func.cu:1099-1111).

    python tests/golden/make_oracle_fixtures.py [case ...]

With case names only those cases are (re)made and merged into the file.
"""
import hashlib
import json
import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "gene-sequences-de-redundancy_gb300"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

OUT = os.path.join(HERE, "oracle_outputs.json")

# name -> (workload config, reads or None for the whole workload, seed, t)
CASES = {
    # the headline workload, whole: 200k reads, lognormal lengths, t = 0.95
    "c1_full": (1, None, None, 0.95),
    # 200k-read slice of the 2M-read 150 bp workload, t = 0.90
    "c2_200k": (2, 200000, 33, 0.90),
    # 3k-read slice of the 300k-read 2-30 kbp workload, t = 0.80 (drop mode)
    "c3_3k": (3, 3000, 43, 0.80),
}


def sha(b):
    return hashlib.sha256(b).hexdigest()


def make(name, spec, td):
    import gsdr
    import oracle_binding as orc

    cfg, n, seed, t = spec
    data = gsdr.synth_fasta(cfg, n_reads=n, seed=seed)
    path = os.path.join(td, name + ".fa")
    with open(path, "wb") as f:
        f.write(data)
    t0 = time.time()
    order, cl, st = orc.run(path, path + ".out", t=t, threads=os.cpu_count() or 1)
    dt = time.time() - t0
    with open(path + ".out", "rb") as f:
        out = f.read()
    return {
        "config": cfg, "reads": n, "seed": seed, "threshold": t,
        "input_sha256": sha(data), "input_bytes": len(data), "n": int(len(cl)),
        "representatives": int((cl == np.arange(len(cl))).sum()),
        "rounds": int(st.rounds), "aligned": int(st.aligned), "accepted": int(st.accepted),
        "cluster_sha256": sha(np.ascontiguousarray(cl, dtype="<i4").tobytes()),
        "order_sha256": sha(np.ascontiguousarray(order, dtype="<i4").tobytes()),
        "output_sha256": sha(out), "output_bytes": len(out),
        "oracle_seconds": round(dt, 1), "oracle_threads": os.cpu_count() or 1,
    }


def main():
    only = sys.argv[1:]
    result = {}
    if os.path.exists(OUT):
        with open(OUT) as f:
            result = json.load(f)
    with tempfile.TemporaryDirectory() as td:
        for name, spec in CASES.items():
            if only and name not in only:
                continue
            result[name] = make(name, spec, td)
            print(name, json.dumps(result[name]), flush=True)
    with open(OUT, "w") as f:
        json.dump(result, f, indent=1, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main()
